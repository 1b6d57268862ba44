"""totri_gb300.data: wall grids, mesh helpers (reference totri/data/util.py),
the MATLAB-format dataset loaders (veltennc2012.py, otooleconfocal2018.py) and
the Zaragoza loader (zaragoza.py) over any mapping of its HDF5 datasets."""
from .mat_datasets import OTooleConfocal2018, VeltenNc2012
from .util import make_wall_grid, merge_meshes
from .zaragoza import Zaragoza, ZaragozaDataset

__all__ = ["make_wall_grid", "merge_meshes", "OTooleConfocal2018", "VeltenNc2012", "Zaragoza",
           "ZaragozaDataset"]
