"""totri_gb300.util: argument normalisers and RBF splatting (reference totri/util)."""
from .format import colors_of_verts, faces_of_verts, origin_of_wallpoints, verts_transform
from .rbf2volume import Rbf2VolumeGaussian

__all__ = ["colors_of_verts", "faces_of_verts", "origin_of_wallpoints", "verts_transform",
           "Rbf2VolumeGaussian"]
