"""Loader for the f-k migration dataset format of Lindell et al. 2019
(reference totri/data/lindellfk2019.py:8-57): a measurement file holding
``meas`` [T, W, H] and a time-of-flight file holding ``tofgrid`` [W, H], both
HDF5 (MATLAB v7.3).

``LindellFk2019(meas, tof, crop, dtype, device)`` takes paths (read with
h5py, which must then be installed: it is absent from this image) or the two
arrays. Each column's bins are rolled down by floor(tofgrid / 32 ps) (the
wall-to-device round trip), the first `crop` bins are kept, and the result is
arranged as [1, T, H, W] with rows and columns flipped; the scan points are
the reference's 512 x 512 grid on [-1, 1]^2 (whatever the data's size), bins
of 32 ps from 0.
"""
import numpy as np
import torch

from ..types import BinDef, VolumeDef
from .util import make_wall_grid


class LindellFk2019Dataset:
    __slots__ = ["is_confocal", "bin_def", "volume_def", "scan_point_extent", "transient",
                 "scan_points"]

    def __init__(self):
        self.is_confocal = True
        self.bin_def = BinDef(32e-12, 0, 512, unit_is_time=True)
        self.volume_def = VolumeDef([-1, -1, 0], [1, 1, 2], [512, 512, 512])
        self.scan_point_extent = (2, 2)

    def resize(self, height, width):
        pass


def _load(source, key):
    if isinstance(source, str):
        try:
            import h5py
        except ImportError as e:
            raise ImportError("reading LindellFk2019 files needs h5py; pass the arrays "
                              "instead") from e
        with h5py.File(source, "r") as f:
            return torch.tensor(np.asarray(f.get(key)))
    return torch.as_tensor(np.asarray(source))


def LindellFk2019(meas, tof, crop=512, dtype: torch.dtype = torch.float32,
                  device: torch.device = torch.device("cpu")) -> LindellFk2019Dataset:
    tofgrid = _load(tof, "tofgrid")     # [W, H]
    transient = _load(meas, "meas")     # [T, W, H]
    ds = LindellFk2019Dataset()
    shift = torch.floor(tofgrid / (ds.bin_def.width_s * 1e12)).int().long()
    T = transient.shape[0]
    t = torch.arange(T).view(T, 1, 1)
    transient = torch.gather(transient, 0, ((t + shift[None]) % T).expand_as(transient))
    transient = transient[:crop].permute(0, 2, 1).flip([1, 2])[None]
    ds.transient = transient.to(dtype=dtype, device=device)
    ds.scan_points = make_wall_grid(-1, 1, 512, -1, 1, 512, z_val=0, flattened=False,
                                    device=torch.device("cpu"))[None].to(dtype=dtype,
                                                                          device=device)
    return ds
