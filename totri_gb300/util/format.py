"""Argument normalisers of the reference API (totri/util/format.py:8-94)."""
import typing

import torch


def origin_of_wallpoints(origin: typing.Optional[torch.Tensor], wall_points: torch.Tensor,
                         origin_name: str) -> torch.Tensor:
    """Origin as [B, N', 3]: N' = 0 when origin is None, else N (format.py:8-35)."""
    if origin is None:
        origin = torch.empty_like(wall_points[:, :0, :])
    elif origin.ndim == 2:
        origin = origin[:, None, :].expand_as(wall_points)
    elif origin.ndim == 3:
        if origin.shape[1] > 0:
            origin = origin.expand_as(wall_points)
    else:
        raise ValueError(f'Shape {origin.shape} of {origin_name} is invalid.')
    return origin


def faces_of_verts(verts: torch.Tensor,
                   faces: typing.Optional[torch.Tensor] = None) -> torch.Tensor:
    """Faces [..., V/3, 3] of consecutive vertex triples when faces is None (format.py:52-71)."""
    if faces is None:
        num_faces = verts.shape[-2] // 3
        faces = torch.arange(0, 3 * num_faces, dtype=torch.int32,
                             device=verts.device).view(-1, 3)
        while faces.ndim < verts.ndim:
            faces = faces[None]
        faces = faces.expand_as(verts[..., :num_faces, :3])
    return faces


def colors_of_verts(colors: typing.Optional[torch.Tensor], verts: torch.Tensor) -> torch.Tensor:
    """Colors as [B, V, {0, 1}] (format.py:73-94)."""
    if colors is None:
        colors = torch.empty_like(verts[:, :, :0])
    if (colors.ndim != 3 or colors.shape[0] != verts.shape[0] or
            colors.shape[1] != verts.shape[1]):
        raise ValueError(f'Shape {colors.shape} of colors is invalid for '
                         f'verts of shape {verts.shape}.')
    return colors


def verts_transform(verts: torch.Tensor) -> torch.Tensor:
    """Vertex coordinates flipped for viewers that look down -z (format.py:37-50)."""
    return torch.stack((-verts[..., 0], verts[..., 1], -verts[..., 2]), dim=-1)
