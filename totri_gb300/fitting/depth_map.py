"""Depth-map fitting: a height field over the wall, rendered as a triangle
mesh, fitted to a transient (reference totri/fitting/depth_map.py:12-422).

``DepthMap`` holds depth and albedo grids [H, W] over the x/y extent of a
VolumeDef (resolution (D, H, W)); vertex (x, y) sits on the inclusive
linspace of that extent and z = offset - (|z1 - z0| / 2) (depth - 0.5); every
grid cell is two triangles. ``DepthMapFitting.fit`` renders it confocally or
exhaustively (optionally plus a background model and an intensity scale
solved once by least squares), minimises
10 mse + 1000 lambda_depth tv(depth) + 10 lambda_color tv(color)
+ 10 lambda_black mean(color) with ``TotriOptimizer``, clamps depth to [0, 1]
and albedo to a unit maximum after every step, pins the border, and can
cycle through random scan-point subsets and refine the grid (bilinear resize
plus a Gaussian blur) at given iterations. TensorBoard logging is not
reproduced.
"""
import math
import typing

import torch

from ..render import MeshRenderConfocal, MeshRenderExhaustive
from ..types import BinDef, VolumeDef
from ..util.optim import Interpolator, MultiplicativeInterpolator, TotriOptimizer


def dx_dy(t: torch.Tensor) -> typing.Tuple[torch.Tensor, torch.Tensor]:
    """Forward differences along x (columns) and y (rows), zero on the last one."""
    dx = torch.zeros_like(t)
    dy = torch.zeros_like(t)
    dx[:, :-1] = t[:, 1:] - t[:, :-1]
    dy[:-1, :] = t[1:, :] - t[:-1, :]
    return dx, dy


def tv_loss(t: torch.Tensor) -> torch.Tensor:
    """Mean of sqrt(dx^2 + dy^2 + 1e-3) - sqrt(1e-3)."""
    dx, dy = dx_dy(t)
    eps = 1.e-3
    return torch.mean(torch.sqrt(dx * dx + dy * dy + eps) - math.sqrt(eps))


def gaussian_blur(img: torch.Tensor, kernel_size: int) -> torch.Tensor:
    """Separable Gaussian blur of [C, H, W] with reflected borders; sigma
    0.3 ((k - 1) / 2 - 1) + 0.8 as torchvision's default for kernel size k."""
    sigma = 0.3 * ((kernel_size - 1) * 0.5 - 1) + 0.8
    r = kernel_size // 2
    x = torch.arange(-r, r + 1, dtype=img.dtype, device=img.device)
    k = torch.exp(-0.5 * (x / sigma) ** 2)
    k = k / k.sum()
    out = torch.nn.functional.pad(img[None], (r, r, r, r), mode="reflect")
    C = img.shape[0]
    out = torch.nn.functional.conv2d(out, k.view(1, 1, 1, -1).expand(C, 1, 1, -1), groups=C)
    out = torch.nn.functional.conv2d(out, k.view(1, 1, -1, 1).expand(C, 1, -1, 1), groups=C)
    return out[0]


class DepthMap:
    def __init__(self, volume_def: VolumeDef, device="cuda"):
        self.volume_def = volume_def
        self.device = device
        self.depth_scaling = 0.5 * abs(volume_def.end[2] - volume_def.start[2])
        H, W = volume_def.resolution[1], volume_def.resolution[2]
        self.depth = torch.full((H, W), 0.5, device=device)
        self.offset = torch.full((1,), 0.5 * (volume_def.start[2] + volume_def.end[2]),
                                 device=device)
        self.color = torch.full((H, W), 1.0, device=device)
        self.xy_coordinates = self.get_xy_coords()
        self.faces = self.get_faces()
        self.clamp_params(None)

    def requires_grad(self, flag):
        for t in (self.depth, self.offset, self.color):
            t.requires_grad = flag

    def params(self):
        return [t for t in (self.depth, self.offset, self.color) if t.requires_grad]

    def clamp_params(self, intensity):
        with torch.no_grad():
            scale = 1.0 / (1.e-12 + self.color.max())
            if intensity is not None:
                intensity[0] = intensity[0] / scale
            self.color[:] = torch.clamp(self.color * scale, min=1.e-12)
            for t, border in ((self.color, 1.e-12), (self.depth, None)):
                if border is None:
                    t[:] = torch.clamp(t, min=0, max=1)
                    border = 0.5
                t[:, 0] = border
                t[:, -1] = border
                t[0, :] = border
                t[-1, :] = border

    def abs_depth(self):
        return self.offset - self.depth_scaling * (self.depth - 0.5)

    def verts(self) -> torch.Tensor:
        """[H W, 3], x fastest."""
        return torch.cat((self.xy_coordinates, self.abs_depth()[:, :, None]), dim=2).view(-1, 3)

    def colors(self) -> torch.Tensor:
        return self.color[:, :, None].expand(-1, -1, 3).reshape(-1, 3)

    def resize(self, resolution):
        vd = self.volume_def
        vd.resolution = (vd.resolution[0], resolution[0], resolution[1])
        up = lambda t: torch.nn.functional.interpolate(  # noqa: E731
            t[None, None], size=resolution, mode="bilinear", align_corners=False)[0, 0]
        self.depth = up(self.depth)
        self.color = up(self.color)
        self.xy_coordinates = self.get_xy_coords()
        self.faces = self.get_faces()

    def blur(self, kernel_size):
        self.depth[:] = gaussian_blur(self.depth[None], kernel_size)[0]
        self.color[:] = gaussian_blur(self.color[None], kernel_size)[0]

    def get_xy_coords(self):
        vd = self.volume_def
        x = torch.linspace(vd.start[0], vd.end[0], vd.resolution[2], device=self.device)
        y = torch.linspace(vd.start[1], vd.end[1], vd.resolution[1], device=self.device)
        return torch.stack((x[None, :].expand(len(y), -1), y[:, None].expand(-1, len(x))), -1)

    def get_faces(self):
        H, W = self.volume_def.resolution[1], self.volume_def.resolution[2]
        y, x = torch.meshgrid(torch.arange(H - 1), torch.arange(W - 1), indexing="ij")
        i00 = (x + y * W).reshape(-1)
        i10, i01, i11 = i00 + 1, i00 + W, i00 + W + 1
        faces = torch.stack((torch.stack((i00, i11, i10), 1), torch.stack((i00, i01, i11), 1)), 1)
        return faces.reshape(-1, 3).to(device=self.device, dtype=torch.int32)


class DepthMapFitting:
    def __init__(self, bin_def: BinDef, tensorboard: bool = False, log_dir: str = None,
                 log_val_interval: int = 1, log_img_interval: int = 50):
        if tensorboard:
            raise NotImplementedError("TensorBoard logging is not part of totri_gb300")
        self.bin_def = bin_def
        self.log_dir = log_dir
        self.iter = 0
        self.intensity = None
        self.losses = []

    def _render(self, depth_map, scan_points, laser_points, scan_origin, laser_origin):
        colors = depth_map.color.view(1, -1, 1)
        verts, faces = depth_map.verts()[None], depth_map.faces[None]
        if laser_points is None:
            return MeshRenderConfocal.apply(verts, faces, scan_points, self.bin_def, colors,
                                            scan_origin)[0]
        return MeshRenderExhaustive.apply(verts, faces, scan_points, laser_points,
                                          self.bin_def, colors, scan_origin, laser_origin)[0]

    def fit(self, depth_map: DepthMap, transient_input: torch.Tensor,
            scan_points: torch.Tensor, laser_points=None, scan_origin=None, laser_origin=None,
            background_model=None, scan_point_limit=0, num_iter: int = 2000,
            lr_interpolator: Interpolator = None, lambda_depth=0.2, lambda_color=0.1,
            lambda_w=0.05, lambda_black=0, warmup=0, subdivide_at=(), callback=None):
        """transient_input [T, S] (or [T, S, L] with laser_points [L, 3]),
        scan_points [S, 3]; returns the fitted DepthMap."""
        if lr_interpolator is None:
            lr_interpolator = MultiplicativeInterpolator(1.e-2, 1.e-4, gamma=0.99)
        add_b = lambda t: None if t is None else t[None]  # noqa: E731
        scan_points, laser_points = scan_points[None], add_b(laser_points)
        scan_origin, laser_origin = add_b(scan_origin), add_b(laser_origin)
        transient_input = transient_input / transient_input.mean()
        subsets = None
        if scan_point_limit > 0:
            S = transient_input.shape[1]
            perm = torch.randperm(S, device=transient_input.device)
            subsets = [(transient_input[:, perm[a:a + scan_point_limit]].contiguous(),
                        scan_points[:, perm[a:a + scan_point_limit]].contiguous())
                       for a in range(0, S, scan_point_limit)]
            transient_input, scan_points = subsets[0]
        if self.intensity is None:
            with torch.no_grad():
                r = self._render(depth_map, scan_points, laser_points, scan_origin,
                                 laser_origin)
            num = (r * transient_input).sum()
            den = (r * r).sum()
            self.intensity = (num / den.clamp(min=1.e-6)).clamp(min=1.e-6).view(1)
            self.intensity.requires_grad = True
        depth_map.requires_grad(True)
        bg_params = [] if background_model is None else list(background_model.parameters())
        optim = TotriOptimizer(depth_map.params() + [self.intensity] + bg_params,
                               lr_interpolator, warmup)
        for i in range(num_iter):
            if self.iter in subdivide_at:
                res = depth_map.volume_def.resolution[1:]
                depth_map.requires_grad(False)
                depth_map.resize((res[0] * 2, res[1] * 2))
                depth_map.blur(4 * 2 + 1)
                depth_map.requires_grad(True)
                optim.set_params(depth_map.params() + [self.intensity] + bg_params, warmup)
            optim.zero_grad()
            if subsets is not None:
                transient_input, scan_points = subsets[i % len(subsets)]
            rendered = self._render(depth_map, scan_points, laser_points, scan_origin,
                                    laser_origin)
            transient = rendered
            background = None
            if background_model is not None:
                background = (background_model(scan_points) if laser_points is None
                              else background_model(scan_points, laser_points))[0]
                transient = rendered + background
            transient = self.intensity * transient
            loss = (10.0 * torch.mean((transient - transient_input) ** 2)
                    + lambda_depth * 1000.0 * tv_loss(depth_map.depth)
                    + lambda_color * 10.0 * tv_loss(depth_map.color)
                    + lambda_black * 10.0 * depth_map.color.mean())
            loss.backward()
            optim.step()
            self.iter += 1
            self.losses.append(loss.detach())
            depth_map.clamp_params(self.intensity)
            if background_model is not None and hasattr(background_model, "clamp_parameters"):
                background_model.clamp_parameters(rendered, background)
            if callback is not None:
                callback(self.iter, depth_map, transient, loss)
        depth_map.requires_grad(False)
        return depth_map
