"""Loaders for the two public NLOS measurement formats stored as MATLAB files
(reference totri/data/veltennc2012.py and otooleconfocal2018.py).

``VeltenNc2012(path, transform, rectify, device)`` reads the struct
``dataset`` (deltat, t0, t, data [L, S N], cameraPos, laserPos, cameraOrigin,
laserOrigin, all in cm) into transient [1, N, S, L] and wall points in metres,
moved into the wall frame by ``transform`` (default: translation by
(-3.75, -2.20, 0) m, 25 degree rotation about z, axes permuted to (y, z, -x)
and 2 m added to the depth, veltennc2012.py:8-42). ``rectify`` shifts each
scan (then laser) column's bins down by int(|point - origin| / bin width)
with wrap-around and drops the origins (veltennc2012.py:63-82).

``OTooleConfocal2018(path, dtype, device)`` reads ``rect_data`` [W, H, N]
into transient [1, N, H, W] (rows flipped, bins below 600 zeroed) on a
64 x 64 wall grid over the volume's x/y extent, 4 ps bins offset by 100 bins
(otooleconfocal2018.py:9-76), with ``downsample_temporal`` (sum of `factor`
consecutive bins) and ``downsample_spatial`` (bilinear resize of the
transient and the grid).

The HDF5 formats of the reference (Zaragoza, LindellFk2019) need h5py, which
is not installed.
"""
import math
import typing

import numpy as np
import torch
from scipy.io import loadmat

from ..types import BinDef, VolumeDef
from .util import make_wall_grid


def velten_nc2012_transform(x: torch.Tensor, is_normal: bool) -> torch.Tensor:
    """Reference frame of the VeltenNc2012 data -> wall frame (points [N, 3])."""
    a = 25 / 360 * 2 * math.pi
    rot = torch.tensor([[math.cos(a), -math.sin(a), 0.0], [math.sin(a), math.cos(a), 0.0],
                        [0.0, 0.0, 1.0]], device=x.device, dtype=x.dtype)
    if not is_normal:
        x = x + torch.tensor([[-3.75, -2.20, 0.0]], device=x.device, dtype=x.dtype)
    x = x @ rot.T
    x = torch.stack((x[:, 1], x[:, 2], -x[:, 0]), dim=1)
    if not is_normal:
        x = x + torch.tensor([[0.0, 0.0, 2.0]], device=x.device, dtype=x.dtype)
    return x


def _roll_columns(tr, shifts, dim):
    """tr [N, ...]: column c (along `dim` of tr) rolled by -shifts[c] over bins."""
    N = tr.shape[0]
    t = torch.arange(N, device=tr.device)
    shape = [1] * tr.dim()
    shape[dim] = -1
    idx = (t.view([-1] + [1] * (tr.dim() - 1)) + shifts.view(shape)) % N
    return torch.gather(tr, 0, idx.expand_as(tr))


class VeltenNc2012Dataset:
    __slots__ = ["transient", "scan_points", "laser_points", "volume_def", "bin_def",
                 "scan_origin", "laser_origin"]

    def rectify(self):
        """Bins shifted by the origin-to-wall distances (per scan, then laser)."""
        tr = self.transient[0]  # [N, S, L]
        if self.scan_origin is not None:
            d = ((self.scan_points[0] - self.scan_origin) ** 2).sum(dim=1) ** 0.5
            tr = _roll_columns(tr, (d / self.bin_def.width).int().long(), 1)
            self.scan_origin = None
        if self.laser_origin is not None:
            d = ((self.laser_points[0] - self.laser_origin) ** 2).sum(dim=1) ** 0.5
            tr = _roll_columns(tr, (d / self.bin_def.width).int().long(), 2)
            self.laser_origin = None
        self.transient = tr[None].contiguous()


def VeltenNc2012(path: str, transform: typing.Callable = velten_nc2012_transform,
                 rectify: bool = False, device=torch.device("cpu")) -> VeltenNc2012Dataset:
    ds = loadmat(path)["dataset"]
    field = lambda k: ds[k][0, 0]  # noqa: E731
    data = VeltenNc2012Dataset()
    num = int(field("t").item())
    data.bin_def = BinDef(field("deltat").item() / 100, field("t0").item() / 100, num)
    raw = field("data")  # [L, S N]
    raw = raw.reshape(1, raw.shape[0], -1, num)  # [1, L, S, N]
    data.transient = torch.tensor(raw, dtype=torch.float32, device=device).permute(0, 3, 2, 1)
    pts = lambda k: transform(torch.tensor(field(k) / 100, dtype=torch.float32,  # noqa: E731
                                           device=device), False)
    data.scan_points = pts("cameraPos")[None]
    data.laser_points = pts("laserPos")[None]
    data.scan_origin = pts("cameraOrigin")
    data.laser_origin = pts("laserOrigin")
    data.volume_def = VolumeDef((-0.75, 0.0, -0.44 + 2.0), (0.75, 3.0, 0.44 + 2.0),
                                (44, 150, 75))
    if rectify:
        data.rectify()
    return data


class OTooleConfocal2018Dataset:
    __slots__ = ["is_confocal", "bin_def", "volume_def", "scan_point_extent", "transient",
                 "scan_points"]

    def __init__(self):
        self.is_confocal = True
        self.bin_def = BinDef(4e-12, 100 * 4e-12, 2048, unit_is_time=True)
        self.volume_def = VolumeDef([-0.4, -0.4, 0.2], [0.4, 0.4, 1.0], [512, 64, 64])
        self.scan_point_extent = (2, 2)

    def downsample_temporal(self, factor):
        if not isinstance(factor, int):
            raise ValueError("Downsample factor must be integer.")
        if factor < 1:
            raise ValueError("Downsample factor must be positive.")
        if factor == 1:
            return
        N = self.transient.shape[1]
        if N % factor:
            raise ValueError("Number of bins must be divisible by factor.")
        t = self.transient
        self.transient = t.reshape(t.shape[0], N // factor, factor, *t.shape[2:]).sum(dim=2)
        self.bin_def.width = self.bin_def.width * factor
        self.bin_def.num = self.bin_def.num // factor

    def downsample_spatial(self, resolution):
        self.transient = torch.nn.functional.interpolate(self.transient, size=resolution,
                                                         mode="bilinear", align_corners=False)
        self.scan_points = torch.nn.functional.interpolate(
            self.scan_points.permute(0, 3, 1, 2), size=resolution, mode="bilinear",
            align_corners=False).permute(0, 2, 3, 1)


def OTooleConfocal2018(path: str, dtype: torch.dtype = torch.float32,
                       device=torch.device("cpu")) -> OTooleConfocal2018Dataset:
    ds = OTooleConfocal2018Dataset()
    raw = loadmat(path)["rect_data"].astype(np.float32)
    tr = torch.tensor(raw).permute(2, 1, 0).flip([1])  # [N, H, W]
    tr[:600] = 0
    ds.transient = tr[None].to(dtype=dtype, device=device)
    vd = ds.volume_def
    ds.scan_points = make_wall_grid(vd.start[0], vd.end[0], 64, vd.start[1], vd.end[1], 64,
                                    z_val=0, device=torch.device("cpu"),
                                    flattened=False)[None].to(dtype=dtype, device=device)
    return ds
