"""totri_gb300.util: argument normalisers (reference totri/util)."""
from .format import colors_of_verts, faces_of_verts, origin_of_wallpoints, verts_transform

__all__ = ["colors_of_verts", "faces_of_verts", "origin_of_wallpoints", "verts_transform"]
