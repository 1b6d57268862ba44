"""Backprojection reconstructions (reference totri/reconstruct/backprojection.py).

Same classes, argument conventions and layouts as the reference. Differences:
``BackprojectionExhaustiveArellano.apply`` works (the reference's ``forward``
lacks ``ctx`` and cannot be applied, backprojection.py:48), and
``BackprojectionConfocalVelten`` has a backward with respect to the transient
(the adjoint backprojection).
"""
import typing

import torch

from ..totri_cpp import reconstruct as K
from ..types import BinDef, VolumeDef
from ..util.format import origin_of_wallpoints


def second_derivative_filter(volume):
    """Negative part of the second z-derivative (backprojection.py:12-18)."""
    def dz(v):
        v = torch.cat((v, v[:, -1:, :, :]), dim=1)
        return v[:, 1:, :, :] - v[:, :-1, :, :]
    volume = dz(dz(volume))
    volume[volume > 0] = 0
    return -volume


def _origin_b3n(origin, points, name):
    if origin is None:
        return torch.empty_like(points[:, :, :0])
    if origin.ndim == 2:
        return origin[:, :, None].expand_as(points)
    if origin.ndim == 3:
        return origin.expand_as(points)
    raise ValueError(f'Shape {origin.shape} of {name} is invalid.')


def _device():
    if not torch.cuda.is_available():
        raise RuntimeError('backprojection needs a CUDA device, but none is available.')
    return torch.device('cuda')


class BackprojectionExhaustiveArellano(torch.autograd.Function):
    """Probability volume [B, D, H, W] from transient [B, T, S, L] by ellipsoid
    backprojection (Arellano, Gutierrez, Jarabo 2017). Points [B, 3, S] / [B, 3, L]."""

    @staticmethod
    def forward(ctx, transient: torch.Tensor, scan_points: torch.Tensor,
                laser_points: torch.Tensor, volume_def: VolumeDef, bin_def: BinDef,
                scan_origin: typing.Optional[torch.Tensor] = None,
                laser_origin: typing.Optional[torch.Tensor] = None) -> torch.Tensor:
        dev = transient.device if transient.is_cuda else _device()
        volume = torch.zeros((transient.shape[0],) + tuple(volume_def.resolution), device=dev)
        scan_origin = _origin_b3n(scan_origin, scan_points, 'scan_origin')
        laser_origin = _origin_b3n(laser_origin, laser_points, 'laser_origin')
        K.backprojection_exhaustive_arellano_forward(
            transient.to(dev), scan_points.to(dev), laser_points.to(dev), scan_origin.to(dev),
            laser_origin.to(dev), volume, volume_def.start, volume_def.end, bin_def.width,
            bin_def.offset)
        return volume.to(transient.device)


class BackprojectionConfocalVelten(torch.autograd.Function):
    """Probability volume [B, D, H, W] from a confocal transient [B, T, S]
    (Velten et al. 2012). Scan points [B, S, 3]; scan_origin [B, S, 3], [B, 1, 3]
    or [B, 3]."""

    @staticmethod
    def forward(ctx, transient: torch.Tensor, scan_points: torch.Tensor, volume_def: VolumeDef,
                bin_def: BinDef,
                scan_origin: typing.Optional[torch.Tensor] = None) -> torch.Tensor:
        dev = transient.device if transient.is_cuda else _device()
        volume = torch.empty((transient.shape[0],) + tuple(volume_def.resolution), device=dev)
        scan_origin = origin_of_wallpoints(scan_origin, scan_points, 'scan_origin')
        ctx.save_for_backward(scan_points, scan_origin)
        ctx.volume_def = volume_def
        ctx.bin_def = bin_def
        ctx.num_bins = transient.shape[1]
        K.backprojection_confocal_velten_forward(
            transient.to(dev), scan_points.to(dev), scan_origin.to(dev), volume,
            volume_def.start, volume_def.end, bin_def.width, bin_def.offset)
        return volume.to(transient.device)

    @staticmethod
    def backward(ctx, volume_grad: torch.Tensor):
        grad = [None] * 5
        if volume_grad is not None and ctx.needs_input_grad[0]:
            scan_points, scan_origin = ctx.saved_tensors
            dev = volume_grad.device
            tr = torch.empty((volume_grad.shape[0], ctx.num_bins, scan_points.shape[1]),
                             device=dev)
            K.backprojection_confocal_velten_adjoint(
                volume_grad.contiguous(), scan_points.to(dev), scan_origin.to(dev), tr,
                ctx.volume_def.start, ctx.volume_def.end, ctx.bin_def.width, ctx.bin_def.offset)
            grad[0] = tr
        return tuple(grad)


class BackprojectionExhaustiveVelten(torch.autograd.Function):
    """Probability volume [B, D, H, W] from transient [B, T, S, L]; scan points
    [B, S, 3], laser points [B, L, 3]."""

    @staticmethod
    def forward(ctx, transient: torch.Tensor, scan_points: torch.Tensor,
                laser_points: torch.Tensor, volume_def: VolumeDef, bin_def: BinDef,
                scan_origin: typing.Optional[torch.Tensor] = None,
                laser_origin: typing.Optional[torch.Tensor] = None) -> torch.Tensor:
        dev = transient.device if transient.is_cuda else _device()
        volume = torch.empty((transient.shape[0],) + tuple(volume_def.resolution), device=dev)
        scan_origin = origin_of_wallpoints(scan_origin, scan_points, 'scan_origin')
        laser_origin = origin_of_wallpoints(laser_origin, laser_points, 'laser_origin')
        K.backprojection_exhaustive_velten_forward(
            transient.to(dev), scan_points.to(dev), laser_points.to(dev), scan_origin.to(dev),
            laser_origin.to(dev), volume, volume_def.start, volume_def.end, bin_def.width,
            bin_def.offset)
        return volume.to(transient.device)
