"""totri_gb300.util: argument normalisers, RBF splatting, depth maps and shaded
previews (reference totri/util) and differentiable marching cubes (the
reference's tomcubes dependency)."""
from .depthmap import UnitDepthMapRender
from .format import colors_of_verts, faces_of_verts, origin_of_wallpoints, verts_transform
from .marching_cubes import MarchingCubesFunction
from .rbf2volume import Rbf2VolumeGaussian
from .render import UnitCubeMeshRender

__all__ = ["colors_of_verts", "faces_of_verts", "origin_of_wallpoints", "verts_transform",
           "Rbf2VolumeGaussian", "MarchingCubesFunction", "UnitDepthMapRender",
           "UnitCubeMeshRender"]
