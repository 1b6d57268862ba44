"""f-k migration (reference totri/reconstruct/fk_migration.py:5-120).

``FkMigration(depth, height, width)(transient [N, D, H, W]) -> volume
[N, D, H, W]``: depth is the time range (bins x bin width) and height/width
the scan grid's extent on the wall, in metres. The preparation, the Stolt
resampling and the final magnitude are hand-written kernels
(``csrc/fk.cu``); the 3-D FFTs are cuFFT's, through ``torch.fft``. The
reference returns ``volume[0]`` of its [N, 1, D, H, W] result, i.e. the
first item's [1, D, H, W]; this returns every item, identical for N = 1.
``StoltInterpolation`` is the resampling alone on a centred complex spectrum
[N, C, 2D, H, W], as in the reference.
"""
import torch

from .. import _lib


def _c(t):
    return _lib.array(torch.view_as_real(t))


def stolt(fourier: torch.Tensor, depth, height, width, input_centred=True,
          output_centred=True) -> torch.Tensor:
    """Stolt resampling of complex [M, 2D, H, W] (centred unless stated)."""
    _lib.require_cuda(fourier)
    f = fourier.contiguous().to(torch.complex64)
    out = torch.empty_like(f)
    _lib.check(_lib.load().totri_fk_stolt(_c(f), _c(out), float(depth), float(height),
                                          float(width), int(input_centred),
                                          int(output_centred), _lib.stream_of(f.device)))
    return out


class StoltInterpolation(torch.nn.Module):
    def __init__(self, depth, height, width):
        super().__init__()
        self.depth, self.height, self.width = depth, height, width

    def forward(self, fourier: torch.Tensor) -> torch.Tensor:
        N, C, D2, H, W = fourier.shape
        if D2 % 2 != 0:
            raise ValueError("the spectrum needs an even number of time bins")
        out = stolt(fourier.reshape(N * C, D2, H, W), self.depth, self.height, self.width)
        return out.view(N, C, D2, H, W)


class FkMigration(torch.nn.Module):
    def __init__(self, depth, height, width):
        super().__init__()
        self.depth, self.height, self.width = depth, height, width

    def forward(self, transient: torch.Tensor) -> torch.Tensor:
        _lib.require_cuda(transient)
        lib = _lib.load()
        t = transient.contiguous().float()
        N, D, H, W = t.shape
        stream = _lib.stream_of(t.device)
        padded = torch.empty((N, 2 * D, H, W), dtype=torch.complex64, device=t.device)
        _lib.check(lib.totri_fk_prepare(_lib.array(t), _c(padded), stream))
        spectrum = torch.fft.fftn(padded, dim=(1, 2, 3))
        resampled = stolt(spectrum, self.depth, self.height, self.width,
                          input_centred=False, output_centred=False)
        volume = torch.fft.ifftn(resampled, dim=(1, 2, 3))
        out = torch.empty((N, D, H, W), dtype=torch.float32, device=t.device)
        _lib.check(lib.totri_fk_finish(_c(volume), _lib.array(out), stream))
        return out
