"""Value types of the reference API: ``BinDef`` and ``VolumeDef``.

Same fields, conversions and helpers as totri/types.py (C0 :5, VolumeDef :41,
BinDef :118) so that existing call sites keep working unchanged.
"""
import typing

import torch

C0 = 299792458.0

Vec3 = typing.Tuple[float, float, float]
Size3 = typing.Tuple[int, int, int]
Vec3_ = typing.Union[Vec3, Size3, int, float]
Size3_ = typing.Union[Size3, int]


def to_vec3(value: Vec3_) -> Vec3:
    if isinstance(value, (int, float)):
        return (float(value),) * 3
    if isinstance(value, (tuple, list)):
        if len(value) != 3:
            raise ValueError(f'Vec3 must be tuple of length 3, got {len(value)}')
        for v in value:
            if not isinstance(v, (int, float)):
                raise ValueError(f'Vec3 entries must be int or float, got {type(v)}')
        return (float(value[0]), float(value[1]), float(value[2]))
    raise ValueError(f'Vec3 must be float or tuple, got {type(value)}')


def to_size3(value: Size3_) -> Size3:
    if isinstance(value, int):
        return (value, value, value)
    if isinstance(value, (tuple, list)):
        if len(value) != 3:
            raise ValueError(f'Size3 must be tuple of length 3, got {len(value)}')
        for v in value:
            if not isinstance(v, int):
                raise ValueError(f'Size3 entries must be int, got {type(v)}')
        return (value[0], value[1], value[2])
    raise ValueError(f'Size3 must be int or tuple, got {type(value)}')


class VolumeDef():
    """Axis-aligned voxel volume: start/end corners (x, y, z) and resolution (D, H, W)."""
    __slots__ = ['start', 'end', 'resolution']

    def __init__(self, start: Vec3_, end: Vec3_, resolution: Size3_):
        self.start: Vec3 = to_vec3(start)
        self.end: Vec3 = to_vec3(end)
        self.resolution: Size3 = to_size3(resolution)

    def __str__(self):
        start = ', '.join(f'{v:.3e} m' for v in self.start)
        end = ', '.join(f'{v:.3e} m' for v in self.end)
        res = ', '.join(f'{v}' for v in self.resolution)
        return f'VolumeDef(start={start}, end={end}, resolution={res})'

    def clone(self):
        return VolumeDef(self.start, self.end, self.resolution)

    def extent(self):
        """(x, y, z) extent"""
        return tuple(abs(self.start[i] - self.end[i]) for i in range(3))

    def corner_points(self) -> torch.Tensor:
        """Corner coordinates of the volume [3, 8]."""
        s, e = self.start, self.end
        return torch.Tensor([
            [s[0], s[1], s[2]], [s[0], e[1], s[2]], [s[0], s[1], e[2]], [s[0], e[1], e[2]],
            [e[0], s[1], s[2]], [e[0], e[1], s[2]], [e[0], s[1], e[2]], [e[0], e[1], e[2]],
        ]).T

    def flat_idx_to_3d_idx(self, idx):
        r = self.resolution
        return (idx % r[2], (idx // r[2]) % r[1], (idx // r[2]) // r[1])

    def index_to_coordinates(self, idx: Size3_):
        idx = to_size3(idx)
        r, s, e = self.resolution, self.start, self.end
        return (idx[0] / r[2] * (e[0] - s[0]) + s[0],
                idx[1] / r[1] * (e[1] - s[1]) + s[1],
                idx[2] / r[0] * (e[2] - s[2]) + s[2])

    def coordinates_inclusive(self, resolution: Size3_ = None,
                              device: torch.device = torch.device('cpu')) -> torch.Tensor:
        """Voxel coordinates [D, H, W, 3] (x, y, z) from start to end inclusive."""
        if resolution is None:
            if self.resolution is None:
                raise ValueError('No resolution specified.')
            resolution = self.resolution
        else:
            resolution = to_size3(resolution)
        x = torch.linspace(self.start[0], self.end[0], resolution[2], device=device)
        y = torch.linspace(self.start[1], self.end[1], resolution[1], device=device)
        z = torch.linspace(self.start[2], self.end[2], resolution[0], device=device)
        return torch.stack(torch.meshgrid(z, y, x, indexing='ij')[::-1], dim=-1)


class BinDef():
    """Time bins: width and offset in metres of path length (or seconds) and count."""
    __slots__ = ['width', 'offset', 'num']

    def __init__(self, width: float, offset: float = 0, num: typing.Optional[int] = None,
                 unit_is_time: bool = False):
        if unit_is_time:
            width *= C0
            offset *= C0
        self.width = width
        self.offset = offset
        self.num = num

    def __str__(self):
        return f'BinDef(width={self.width/C0:.3e}s [{self.width:.3e}m], ' \
            f'offset={self.offset/C0:.3e}s [{self.offset:.3e}m], num={self.num})'

    @property
    def width_s(self):
        return self.width / C0

    @width_s.setter
    def width_s(self, value):
        self.width = value * C0

    @property
    def offset_s(self):
        return self.offset / C0

    @offset_s.setter
    def offset_s(self, value):
        self.offset = value * C0
