"""Gaussian RBF to volume (reference totri/util/rbf2volume.py:9-50)."""
import torch

from ..totri_cpp import util as K
from ..types import VolumeDef


class Rbf2VolumeGaussian(torch.autograd.Function):
    """Gaussian RBFs [B, N, 4+A] (x, y, z, sigma, attributes) to a volume
    [B, 1+A, D, H, W]: channel 0 the summed weights, channels 1.. the
    weight-normalised attributes."""

    @staticmethod
    def forward(ctx, rbf: torch.Tensor, volume_def: VolumeDef) -> torch.Tensor:
        num_attributes = rbf.shape[2] - 4
        shape = (rbf.shape[0], 1 + num_attributes) + tuple(volume_def.resolution)
        if rbf.shape[1] == 0:
            volume = torch.zeros(shape, device=rbf.device, dtype=rbf.dtype)
        else:
            volume = torch.empty(shape, device=rbf.device, dtype=rbf.dtype)
            K.rbf2volume_gaussian_forward(rbf, volume, volume_def.start, volume_def.end)
        ctx.set_materialize_grads(False)
        ctx.save_for_backward(rbf, volume)
        ctx.volume_def = volume_def
        return volume

    @staticmethod
    def backward(ctx, volume_grad: torch.Tensor):
        rbf_grad = None
        if volume_grad is None:
            return rbf_grad, None
        if ctx.needs_input_grad[0]:
            rbf, volume = ctx.saved_tensors
            rbf_grad = torch.zeros_like(rbf)
            if rbf.shape[1] > 0:
                K.rbf2volume_gaussian_grad(rbf, volume, volume_grad, rbf_grad,
                                           ctx.volume_def.start, ctx.volume_def.end)
        if ctx.needs_input_grad[1]:
            raise NotImplementedError()
        return rbf_grad, None
