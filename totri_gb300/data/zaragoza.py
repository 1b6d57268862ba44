"""Loader for the Zaragoza NLOS dataset format (reference
totri/data/zaragoza.py:8-128): HDF5 files with the scene's bin, volume and
wall-grid definitions and a confocal transient.

``Zaragoza(source, rectify, dtype, device)`` takes a path (read with h5py,
which must then be installed: it is absent from this image) or any mapping
from the file's dataset names to arrays, such as an open ``h5py.File`` or a
dict of numpy arrays. Axes are moved from the file's y-up frame into the wall
frame by (x, y, z) -> (x, z, -y); the transient [1, N, 6, H, W] is summed
over its third axis into [1, N, H, W]; the scan points, normals and origin
come from the camera grid. ``rectify`` rolls each scan column's bins down by
int(2 |point - origin| / bin width) and drops the origin
(zaragoza.py:38-50). Exhaustive captures are not supported, as in the
reference.
"""
import typing

import numpy as np
import torch

from ..types import BinDef, VolumeDef


def swap_yz(t: torch.Tensor) -> torch.Tensor:
    return torch.stack((t[..., 0], t[..., 2], -t[..., 1]), dim=-1)


class ZaragozaDataset:
    __slots__ = ["is_confocal", "bin_def", "volume_def", "scan_point_extent",
                 "laser_point_extent", "transient", "scan_points", "laser_points",
                 "scan_normals", "laser_normals", "scan_origin", "laser_origin"]

    def rectify(self):
        """Shift each scan column's bins by the origin-to-wall round trip."""
        if not self.is_confocal or self.scan_origin is None:
            return
        d = ((self.scan_points[0] - self.scan_origin) ** 2).sum(dim=-1) ** 0.5  # [H, W]
        shift = (2 * d / self.bin_def.width).int().long()
        tr = self.transient[0]  # [N, H, W]
        N = tr.shape[0]
        t = torch.arange(N, device=tr.device).view(N, 1, 1)
        idx = (t + shift[None]) % N
        self.transient = torch.gather(tr, 0, idx)[None].contiguous()
        self.scan_origin = None


def _read(source, key):
    return np.asarray(source[key][()])


def Zaragoza(source: typing.Union[str, typing.Mapping], rectify: bool = False,
             dtype: torch.dtype = torch.float32,
             device: torch.device = torch.device("cpu")) -> ZaragozaDataset:
    if isinstance(source, str):
        try:
            import h5py
        except ImportError as e:
            raise ImportError("reading a Zaragoza file needs h5py; pass a mapping of its "
                              "datasets instead") from e
        with h5py.File(source, "r") as f:
            return Zaragoza(f, rectify, dtype, device)
    ds = ZaragozaDataset()
    ds.is_confocal = bool(_read(source, "isConfocal"))
    ds.bin_def = BinDef(float(_read(source, "deltaT")), float(_read(source, "t0")),
                        int(_read(source, "t").item()), unit_is_time=False)
    pos = swap_yz(torch.tensor(_read(source, "hiddenVolumePosition")).view(3)).tolist()
    size = float(_read(source, "hiddenVolumeSize"))
    res = torch.tensor(_read(source, "cameraGridPoints")).view(2).int().tolist()
    ds.volume_def = VolumeDef(tuple(p - size / 2 for p in pos), tuple(p + size / 2 for p in pos),
                              (ds.bin_def.num, res[1], res[0]))
    ds.scan_point_extent = torch.tensor(_read(source, "cameraGridSize")).view(2).float().tolist()
    if not ds.is_confocal:
        raise NotImplementedError("exhaustive Zaragoza captures are not supported")
    ds.laser_point_extent = None
    data = torch.tensor(_read(source, "data"))
    ds.transient = data.view(1, ds.bin_def.num, 6, res[1], res[0]).sum(dim=2).to(
        dtype=dtype, device=device)

    def grid(key):
        g = torch.tensor(_read(source, key)).view(1, 3, res[1], res[0]).permute(0, 2, 3, 1)
        return swap_yz(g).to(dtype=dtype, device=device)

    ds.scan_points = grid("cameraGridPositions")
    ds.scan_normals = grid("cameraGridNormals")
    ds.laser_points = ds.laser_normals = ds.laser_origin = None
    ds.scan_origin = swap_yz(torch.tensor(_read(source, "cameraPosition")).view(1, 3)).to(
        dtype=dtype, device=device)
    if rectify:
        ds.rectify()
    return ds
