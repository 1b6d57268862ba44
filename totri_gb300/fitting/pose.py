"""Rigid pose fitting of known meshes to a confocal transient (reference
totri/fitting/pose.py:10-163).

Each mesh gets a translation and a rotation (a quaternion normalised on use,
pose.py:28-47); the posed meshes are merged (totri/data/util.py:67-76) and
rendered with ``MeshRenderConfocal``, and Adam (lr 1e-2, MultiStepLR at
50/100/200/400 iterations with gamma 0.8) minimises
100 mean((render / max - input / max)^2), stopping early once the loss falls
below 1e-6 (pose.py:113-155). The reference rotates with pytorch3d's
``quaternion_apply``; ``quaternion_apply`` here is the same rotation written
out (v' = v + 2 w (u x v) + 2 u x (u x v) for q = (w, u)). TensorBoard
logging is not reproduced.
"""
import typing

import torch

from ..data.util import merge_meshes
from ..render import MeshRenderConfocal
from ..types import BinDef


def quaternion_apply(quaternion: torch.Tensor, points: torch.Tensor) -> torch.Tensor:
    """Rotates points [..., 3] by unit quaternion(s) [..., 4] (w, x, y, z)."""
    w = quaternion[..., :1]
    u = quaternion[..., 1:]
    uv = torch.cross(u.expand_as(points), points, dim=-1)
    return points + 2 * (w * uv + torch.cross(u.expand_as(points), uv, dim=-1))


class Translation(torch.nn.Module):
    """verts + t, t a [1, 3] parameter (pose.py:10-26)."""

    def __init__(self, translation=(0, 0, 0), device="cuda"):
        super().__init__()
        t = torch.tensor([translation], dtype=torch.float32, device=device)
        self.translation = torch.nn.Parameter(t)

    def forward(self, verts: torch.Tensor) -> torch.Tensor:
        return verts + self.translation


class Rotation(torch.nn.Module):
    """Rotation by the normalised [1, 4] quaternion parameter (pose.py:28-47)."""

    def __init__(self, quaternion=(1, 0, 0, 0), device="cuda"):
        super().__init__()
        q = torch.tensor([quaternion], dtype=torch.float32, device=device)
        self.quaternion = torch.nn.Parameter(q)

    def forward(self, verts: torch.Tensor) -> torch.Tensor:
        q = self.quaternion / (((self.quaternion ** 2).sum() + 1.e-8) ** 0.5)
        return quaternion_apply(q, verts)


def apply_transform(verts_list, translation_list, rotation_list):
    return [translation_list[i](rotation_list[i](verts_list[i]))
            for i in range(len(verts_list))]


class PoseFitting:
    """fit(transient_input [T, S], scan_points [S, 3], verts_list, faces_list)
    -> (translation_list, rotation_list)."""

    def __init__(self, bin_def: BinDef, tensorboard: bool = False, log_dir: str = None):
        if tensorboard:
            raise NotImplementedError("TensorBoard logging is not part of totri_gb300")
        self.bin_def = bin_def
        self.log_dir = log_dir
        self.losses = []

    def fit(self, transient_input: torch.Tensor, scan_points: torch.Tensor,
            verts_list: typing.List[torch.Tensor], faces_list: typing.List[torch.Tensor],
            verts_gt_list=None, translation_list=None, rotation_list=None, num_iter=500,
            stop_loss: typing.Optional[float] = 1.e-6, colors_list=None):
        """``stop_loss`` None skips the per-iteration early-stop test (and its
        device-to-host read), which request servers use to keep the loop
        asynchronous; ``colors_list`` (extension) renders with albedo."""
        device = transient_input.device
        num_meshes = len(verts_list)
        max_val = torch.max(transient_input)
        transient_input = transient_input / max_val
        if translation_list is None:
            translation_list = [Translation(device=device) for _ in range(num_meshes)]
        if rotation_list is None:
            rotation_list = [Rotation(device=device) for _ in range(num_meshes)]
        params = [p for m in translation_list for p in m.parameters()]
        params += [p for m in rotation_list for p in m.parameters()]
        colors = None
        if colors_list is not None:
            colors = torch.cat(colors_list, dim=0)[None]
        optim = torch.optim.Adam(params, lr=1.e-2)
        scheduler = torch.optim.lr_scheduler.MultiStepLR(optim, [50, 100, 200, 400], gamma=0.8)
        for _ in range(num_iter):
            optim.zero_grad()
            verts, faces = merge_meshes(apply_transform(verts_list, translation_list,
                                                        rotation_list), faces_list)
            transient = MeshRenderConfocal.apply(verts[None], faces[None], scan_points[None],
                                                 self.bin_def, colors, None)[0] / max_val
            loss = 100 * torch.mean((transient - transient_input) ** 2)
            loss.backward()
            self.losses.append(loss.detach())
            optim.step()
            scheduler.step()
            if stop_loss is not None and loss < stop_loss:
                break
        return translation_list, rotation_list
