"""totri_gb300.data: wall grids and mesh helpers (reference totri/data/util.py)."""
from .util import make_wall_grid, merge_meshes

__all__ = ["make_wall_grid", "merge_meshes"]
