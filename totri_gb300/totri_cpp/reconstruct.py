"""Drop-in for ``totri_cpp.reconstruct`` (reference src/totri.cpp:18-25)."""
from .. import _lib
from ._common import dense_out, finish_out


def _call(name, tensors, a3, b3, bw, bo, device):
    lib = _lib.load()
    st = getattr(lib, name)(*[_lib.array(t) for t in tensors], _lib.vec3(a3), _lib.vec3(b3),
                            float(bw), float(bo), _lib.stream_of(device))
    _lib.check(st)


def backprojection_exhaustive_arellano_forward(transient, scan_points, laser_points,
                                               scan_origin, laser_origin, volume, volume_start,
                                               volume_end, bin_width, bin_offset):
    """volume [B,D,H,W] += Arellano backprojection of transient [B,T,S,L]
    (reference src/reconstruct/backprojection.cpp:8-20)."""
    _lib.require_cuda(transient, scan_points, laser_points, scan_origin, laser_origin, volume)
    out = dense_out(volume)
    if out is not volume:
        out.copy_(volume)
    _call("totri_backprojection_exhaustive_arellano_forward",
          (transient.contiguous(), scan_points, laser_points, scan_origin, laser_origin, out),
          volume_start, volume_end, bin_width, bin_offset, volume.device)
    finish_out(volume, out)


def backprojection_confocal_velten_forward(transient, scan_points, scan_origin, volume,
                                           volume_start, volume_end, bin_width, bin_offset):
    """volume [B,D,H,W] <- Velten confocal backprojection of transient [B,T,S]
    (reference src/reconstruct/backprojection.cpp:22-34)."""
    _lib.require_cuda(transient, scan_points, scan_origin, volume)
    out = dense_out(volume)
    _call("totri_backprojection_confocal_velten_forward",
          (transient.contiguous(), scan_points, scan_origin, out), volume_start, volume_end,
          bin_width, bin_offset, volume.device)
    finish_out(volume, out)


def backprojection_confocal_velten_adjoint(volume, scan_points, scan_origin, transient,
                                           volume_start, volume_end, bin_width, bin_offset):
    """transient [B,T,S] <- adjoint of the Velten confocal backprojection (no reference
    counterpart)."""
    _lib.require_cuda(volume, scan_points, scan_origin, transient)
    out = dense_out(transient)
    _call("totri_backprojection_confocal_velten_adjoint",
          (volume.contiguous(), scan_points, scan_origin, out), volume_start, volume_end,
          bin_width, bin_offset, volume.device)
    finish_out(transient, out)


def backprojection_exhaustive_velten_forward(transient, scan_points, laser_points, scan_origin,
                                             laser_origin, volume, volume_start, volume_end,
                                             bin_width, bin_offset):
    """volume [B,D,H,W] <- Velten exhaustive backprojection of transient [B,T,S,L]
    (reference src/reconstruct/backprojection.cpp:36-49)."""
    _lib.require_cuda(transient, scan_points, laser_points, scan_origin, laser_origin, volume)
    out = dense_out(volume)
    _call("totri_backprojection_exhaustive_velten_forward",
          (transient.contiguous(), scan_points, laser_points, scan_origin, laser_origin, out),
          volume_start, volume_end, bin_width, bin_offset, volume.device)
    finish_out(volume, out)
