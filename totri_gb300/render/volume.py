"""Differentiable voxel-volume transient rendering (reference totri/render/volume.py).

``VolumeRenderConfocal`` keeps the reference's signatures (volume [X, Y, Z],
measurement points [3, N], transient [N, T]). Its backward uses the exact
adjoint of the forward for the volume gradient; the reference's transposed
operator (still available as ``apply_transposed`` and as
``totri_cpp.render.volume_confocal_grad_volume``) adds samples in the top z
slice that the forward drops. ``VolumeRenderExhaustive`` keeps the reference's
layouts (volume [B, D, H, W], points [B, 3, S] / [B, 3, L], transient
[B, T, S, L]); its backward is the adjoint of the forward (the reference's
gradient kernel is empty).
"""
import typing

import torch

from ..totri_cpp import render as R
from ..types import BinDef, VolumeDef


class VolumeRenderConfocal(torch.autograd.Function):

    @staticmethod
    def apply_transposed(transient: torch.Tensor, measurement_points: torch.Tensor,
                         volume_bbox_origin: typing.Tuple, volume_bbox_size: typing.Tuple,
                         volume_resolution: typing.Tuple, bin_width: float, bin_offset: float):
        volume = torch.empty(volume_resolution, device=transient.device, dtype=transient.dtype)
        R.volume_confocal_grad_volume(volume, measurement_points, transient, volume_bbox_origin,
                                      volume_bbox_size, bin_width, bin_offset)
        return volume

    @staticmethod
    def forward(ctx, volume: torch.Tensor, measurement_points: torch.Tensor,
                volume_bbox_origin: typing.Tuple, volume_bbox_size: typing.Tuple,
                bin_num: int, bin_width: float, bin_offset: float):
        if volume.ndim != 3:
            raise ValueError('Volume tensor must be 3d')
        if not volume.is_cuda or not measurement_points.is_cuda:
            raise NotImplementedError('VolumeRenderConfocal is only implemented for cuda tensors')
        if measurement_points.ndim != 2:
            raise ValueError('Measurement Point Tensor must be 2d')
        if measurement_points.shape[0] != 3:
            raise ValueError('Measurement Point Tensor must be 3xn')
        if len(volume_bbox_origin) != 3:
            raise ValueError('volume_bbox_origin must have 3 entries')
        if len(volume_bbox_size) != 3:
            raise ValueError('volume_bbox_size must have 3 entries')
        ctx.set_materialize_grads(False)
        ctx.save_for_backward(volume, measurement_points)
        ctx.volume_bbox_origin = volume_bbox_origin
        ctx.volume_bbox_size = volume_bbox_size
        ctx.bin_width = bin_width
        ctx.bin_offset = bin_offset
        transient = torch.empty((measurement_points.shape[1], bin_num), device=volume.device,
                                dtype=volume.dtype)
        R.volume_confocal_forward(volume, measurement_points, transient, volume_bbox_origin,
                                  volume_bbox_size, bin_width, bin_offset)
        return transient

    @staticmethod
    def backward(ctx, transient_grad: torch.Tensor):
        if transient_grad is None:
            return (None,) * 7
        volume, measurement_points = ctx.saved_tensors
        volume_grad = None
        points_grad = None
        if ctx.needs_input_grad[0]:
            volume_grad = torch.empty_like(volume)
            R.volume_confocal_adjoint(volume_grad, measurement_points, transient_grad,
                                      ctx.volume_bbox_origin, ctx.volume_bbox_size,
                                      ctx.bin_width, ctx.bin_offset)
        if ctx.needs_input_grad[1]:
            points_grad = torch.empty_like(measurement_points)
            R.volume_confocal_grad_measurement_points(points_grad, volume, measurement_points,
                                                      transient_grad, ctx.volume_bbox_origin,
                                                      ctx.volume_bbox_size, ctx.bin_width,
                                                      ctx.bin_offset)
        return (volume_grad, points_grad) + (None,) * 5


def _origin_b3n(origin, points, name):
    """Origins in the [B, 3, n] point layout (reference volume.py:227-244)."""
    if origin is None:
        return torch.empty_like(points[:, :, :0])
    if origin.ndim == 2:
        return origin[:, :, None].expand_as(points)
    if origin.ndim == 3:
        return origin.expand_as(points) if origin.shape[2] > 0 else origin
    raise ValueError(f'Shape {origin.shape} of {name} is invalid.')


class VolumeRenderExhaustive(torch.autograd.Function):
    """Render occupancy volume [B, D, H, W] to transient image [B, T, S, L].

    Scan/laser points are [B, 3, S] / [B, 3, L]; volume_def.start/end are the
    (x, y, z) corners, volume resolution is (D, H, W).
    """

    @staticmethod
    def forward(ctx, volume: torch.Tensor, scan_points: torch.Tensor,
                laser_points: torch.Tensor, volume_def: VolumeDef, bin_def: BinDef,
                scan_origin: typing.Optional[torch.Tensor] = None,
                laser_origin: typing.Optional[torch.Tensor] = None) -> torch.Tensor:
        if not torch.cuda.is_available():
            raise RuntimeError('VolumeRenderExhaustive needs to run on CUDA device, '
                               'but no devices are available.')
        scan_origin = _origin_b3n(scan_origin, scan_points, 'scan_origin')
        laser_origin = _origin_b3n(laser_origin, laser_points, 'laser_origin')
        ctx.set_materialize_grads(False)
        ctx.save_for_backward(volume, scan_points, laser_points, scan_origin, laser_origin)
        ctx.volume_def = volume_def
        ctx.bin_def = bin_def
        dev = volume.device if volume.is_cuda else torch.device('cuda')
        transient = torch.empty((volume.shape[0], bin_def.num, scan_points.shape[2],
                                 laser_points.shape[2]), device=dev)
        R.volume_render_exhaustive_forward(
            volume.to(dev), scan_points.to(dev), laser_points.to(dev), scan_origin.to(dev),
            laser_origin.to(dev), transient, volume_def.start, volume_def.end, bin_def.width,
            bin_def.offset)
        return transient.to(volume.device)

    @staticmethod
    def backward(ctx, transient_grad: torch.Tensor):
        grad = [None] * 7
        if transient_grad is None:
            return tuple(grad)
        if ctx.needs_input_grad[0]:
            volume, scan_points, laser_points, scan_origin, laser_origin = ctx.saved_tensors
            dev = transient_grad.device if transient_grad.is_cuda else torch.device('cuda')
            volume_grad = torch.empty(volume.shape, device=dev)
            R.volume_render_exhaustive_grad_volume(
                transient_grad.to(dev), scan_points.to(dev), laser_points.to(dev),
                scan_origin.to(dev), laser_origin.to(dev), volume_grad, ctx.volume_def.start,
                ctx.volume_def.end, ctx.bin_def.width, ctx.bin_def.offset)
            grad[0] = volume_grad.to(volume.device)
        for i in range(1, len(ctx.needs_input_grad)):
            if ctx.needs_input_grad[i]:
                raise NotImplementedError()
        return tuple(grad)
