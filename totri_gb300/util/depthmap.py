"""Orthographic depth maps of meshes: the drop-in for the reference's
UnitDepthMapRender (totri/util/depthmap.py:6-36), which rasterises with
pytorch3d. Same constructor (resolution, xysize, znear, zfar, device) and
``apply(verts [V, 3], faces [F, 3]) -> (depth [H, W], mask [H, W])``; the
rasteriser is ``csrc/raster.cu`` (screen conventions documented there). The
reference's zbuf is -1 where no face covers a pixel; so is this one's."""
import torch

from .. import _lib


class UnitDepthMapRender:
    def __init__(self, resolution=512, xysize=2, znear=0, zfar=2, device=torch.device("cpu")):
        self.resolution = int(resolution)
        self.half = 0.5 * float(xysize)
        self.znear, self.zfar = float(znear), float(zfar)
        self.device = device

    def apply(self, verts: torch.Tensor, faces: torch.Tensor):
        _lib.require_cuda(verts, faces)
        v = verts.detach().contiguous().float()
        f = faces.detach().contiguous().long()
        R = self.resolution
        depth = torch.empty((R, R), dtype=torch.float32, device=v.device)
        mask = torch.empty((R, R), dtype=torch.int32, device=v.device)
        lib = _lib.load()
        n = int(lib.totri_depth_raster_workspace(R, R))
        ws = torch.empty(max(n, 1), dtype=torch.uint8, device=v.device)
        import ctypes
        _lib.check(lib.totri_depth_raster(
            _lib.array(v), _lib.array(f), _lib.array(depth), _lib.array(mask),
            -self.half, self.half, -self.half, self.half, self.znear, self.zfar,
            ctypes.c_void_p(ws.data_ptr()), n, _lib.stream_of(v.device)))
        return depth, mask.bool()
