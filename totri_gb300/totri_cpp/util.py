"""Drop-in for ``totri_cpp.util`` (reference src/totri.cpp:48-53)."""
from .. import _lib
from ._common import dense_out, finish_out


def rbf2volume_gaussian_forward(rbf, volume, volume_start, volume_end):
    """volume [B,1+A,D,H,W] <- Gaussian RBF splat of rbf [B,N,4+A]
    (reference src/util/rbf2volume.cpp:7-15)."""
    _lib.require_cuda(rbf, volume)
    out = dense_out(volume)
    st = _lib.load().totri_rbf2volume_gaussian_forward(
        _lib.array(rbf), _lib.array(out), _lib.vec3(volume_start), _lib.vec3(volume_end),
        _lib.stream_of(rbf.device))
    _lib.check(st)
    finish_out(volume, out)


def rbf2volume_gaussian_grad(rbf, volume, volume_grad, rbf_grad, volume_start, volume_end):
    """rbf_grad [B,N,4+A] += d loss / d rbf (reference src/util/rbf2volume.cpp:17-28)."""
    _lib.require_cuda(rbf, volume, volume_grad, rbf_grad)
    out = dense_out(rbf_grad)
    if out is not rbf_grad:
        out.copy_(rbf_grad)
    st = _lib.load().totri_rbf2volume_gaussian_grad(
        _lib.array(rbf), _lib.array(volume.contiguous()), _lib.array(volume_grad.contiguous()),
        _lib.array(out), _lib.vec3(volume_start), _lib.vec3(volume_end),
        _lib.stream_of(rbf.device))
    _lib.check(st)
    finish_out(rbf_grad, out)
