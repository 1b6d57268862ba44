"""Shaded preview images of meshes: the drop-in for the reference's
UnitCubeMeshRender (totri/util/render.py:17-81), which the fitting loops use
for TensorBoard images (pose.py:108-161, rbf.py:212) and which draws with
pytorch3d. Same constructor (resolution, distance, specular, eye) and
``apply(verts [V, 3], faces [F, 3] = None, colors [V, 3] = None,
volume_def = None) -> image [3, H, W]``.

The camera is pytorch3d's look-at camera (eye at ``eye``, default
(0, 0, -distance), looking at (0, 0, 1) with +y up) with a 60 degree
perspective field of view, znear 0.1 and zfar 100; one point light at
(2, 2, -2) with ambient 0.5, diffuse 0.3 and the given specular colour, white
materials with shininess 64, a white background and blend sharpness 1e-4.
The camera matrices are formed here in FP32 as pytorch3d forms them
(look_at_rotation, FoVPerspectiveCameras' projection, the camera centre from
the inverse world-to-view matrix); rasterisation and shading run in
``csrc/shade.cu``.
"""
import ctypes
import math
import typing

import torch

from .. import _lib
from ..types import VolumeDef


def _normalize(x: torch.Tensor, eps: float) -> torch.Tensor:
    return x / torch.clamp(torch.linalg.vector_norm(x), min=eps)


def look_at_view_transform(eye, at=(0.0, 0.0, 1.0), up=(0.0, 1.0, 0.0)):
    """(R [3, 3], T [3]) with view = world @ R + T, FP32 on the CPU.

    The view axes are z = normalize(at - eye), x = normalize(up x z),
    y = normalize(z x x) (x replaced by normalize(y x z) when up is parallel
    to the viewing direction); R holds them as columns and T = -eye @ R."""
    eye = torch.tensor(eye, dtype=torch.float32)
    at = torch.tensor(at, dtype=torch.float32)
    up = torch.tensor(up, dtype=torch.float32)
    z = _normalize(at - eye, 1e-5)
    x = _normalize(torch.linalg.cross(up, z), 1e-5)
    y = _normalize(torch.linalg.cross(z, x), 1e-5)
    if bool(torch.isclose(x, torch.zeros(()), atol=5e-3).all()):
        x = _normalize(torch.linalg.cross(y, z), 1e-5)
    R = torch.stack((x, y, z), dim=1)
    T = -(R.T @ eye)
    return R, T


def fov_focal(fov_degrees=60.0, znear=0.1, aspect_ratio=1.0):
    """(focal_x, focal_y): ndc = focal * view.xy / view.z of a symmetric
    perspective frustum with the given vertical field of view."""
    fov = torch.tensor(math.pi / 180, dtype=torch.float32) * torch.tensor(fov_degrees,
                                                                            dtype=torch.float32)
    zn = torch.tensor(znear, dtype=torch.float32)
    max_y = torch.tan(fov / 2) * zn
    max_x = max_y * aspect_ratio
    return float(2.0 * zn / (max_x - (-max_x))), float(2.0 * zn / (max_y - (-max_y)))


class UnitCubeMeshRender:
    def __init__(self, resolution=512, distance=0.5, specular=0.2, eye=None):
        if eye is None:
            eye = [0.0, 0.0, -distance]
        self.resolution = int(resolution)
        R, T = look_at_view_transform(eye)
        M = torch.eye(4, dtype=torch.float32)
        M[:3, :3] = R
        M[3, :3] = T
        center = torch.linalg.inv(M)[3, :3]
        s = _lib.Shading()
        s.rotation[:] = [float(v) for v in R.reshape(-1)]
        s.translation[:] = [float(v) for v in T]
        s.focal[:] = list(fov_focal(60.0, 0.1, 1.0))
        s.znear, s.zfar = 0.1, 100.0
        s.camera_center[:] = [float(v) for v in center]
        s.light_location[:] = [2.0, 2.0, -2.0]
        s.light_ambient[:] = [0.5] * 3
        s.light_diffuse[:] = [0.3] * 3
        s.light_specular[:] = [float(specular)] * 3
        s.material_ambient[:] = [1.0] * 3
        s.material_diffuse[:] = [1.0] * 3
        s.material_specular[:] = [1.0] * 3
        s.shininess = 64.0
        s.background[:] = [1.0] * 3
        s.sigma, s.gamma = 1e-4, 1e-4
        self.shading = s

    @staticmethod
    def fit_volume(verts: torch.Tensor, volume_def: VolumeDef) -> torch.Tensor:
        """Vertices of a volume's box mapped to the camera's unit view
        (render.py:61-69): the longest side spans [-1, 1], x and y centred,
        the box's far face at z = 2."""
        start = [min(x, y) for x, y in zip(volume_def.start, volume_def.end)]
        sizes = [abs(x - y) for x, y in zip(volume_def.start, volume_def.end)]
        m = max(sizes)
        return torch.stack((
            (verts[:, 0] - start[0]) / m * 2 - sizes[0] / m,
            (verts[:, 1] - start[1]) / m * 2 - sizes[1] / m,
            (verts[:, 2] - start[2]) / m * 2 + (1 - 0.5 * sizes[2] / m)), dim=1)

    def render(self, verts: torch.Tensor, faces: typing.Optional[torch.Tensor] = None,
               colors: typing.Optional[torch.Tensor] = None,
               volume_def: typing.Optional[VolumeDef] = None):
        """(image [3, H, W], pix_to_face [H, W] int32, -1 where empty)."""
        _lib.require_cuda(verts)
        v = verts.detach().float()
        if volume_def is not None:
            v = self.fit_volume(v, volume_def)
        v = v.contiguous()
        if faces is None:
            faces = torch.arange(0, v.shape[0], dtype=torch.int64, device=v.device).view(-1, 3)
        f = faces.detach().to(device=v.device, dtype=torch.int64).contiguous()
        if colors is None:
            colors = torch.ones((1, 3), dtype=torch.float32, device=v.device)
        c = colors.detach().to(device=v.device, dtype=torch.float32).expand(v.shape[0], -1)
        R = self.resolution
        image = torch.empty((3, R, R), dtype=torch.float32, device=v.device)
        pix = torch.empty((R, R), dtype=torch.int32, device=v.device)
        lib = _lib.load()
        n = int(lib.totri_shaded_raster_workspace(v.shape[0], R, R))
        ws = torch.empty(max(n, 1), dtype=torch.uint8, device=v.device)
        _lib.check(lib.totri_shaded_raster(
            _lib.array(v), _lib.array(f), _lib.array(c), ctypes.byref(self.shading),
            _lib.array(image), _lib.array(pix), ctypes.c_void_p(ws.data_ptr()), n,
            _lib.stream_of(v.device)))
        return image, pix

    def apply(self, verts, faces=None, colors=None,
              volume_def: typing.Optional[VolumeDef] = None) -> torch.Tensor:
        return self.render(verts, faces, colors, volume_def)[0]
