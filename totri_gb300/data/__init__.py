"""totri_gb300.data: wall grids, mesh helpers (reference totri/data/util.py),
the MATLAB-format dataset loaders (veltennc2012.py, otooleconfocal2018.py) and
the Zaragoza and LindellFk2019 loaders (zaragoza.py, lindellfk2019.py) over
mappings or arrays of their HDF5 datasets."""
from .lindellfk2019 import LindellFk2019, LindellFk2019Dataset
from .mat_datasets import OTooleConfocal2018, VeltenNc2012
from .util import make_wall_grid, merge_meshes
from .zaragoza import Zaragoza, ZaragozaDataset

__all__ = ["make_wall_grid", "merge_meshes", "OTooleConfocal2018", "VeltenNc2012", "Zaragoza",
           "ZaragozaDataset", "LindellFk2019", "LindellFk2019Dataset"]
