"""CPU oracle for f-k migration (TEST INFRASTRUCTURE).

A numpy restatement (FP64, complex128 FFTs) of the reference's
totri/reconstruct/fk_migration.py, pinned against tests/golden/fk_migration.npz
(the reference's own code run by tests/golden/make_golden_fk.py):

* ``stolt(fourier, depth, height, width)`` (fk_migration.py:5-86): on the
  centred spectrum [..., 2D, H, W], the sample at normalised coordinates
  (x, y, z) (x, y, z each on linspace(-1, 1) of W, H, 2D points) is the
  trilinear interpolation, with zeros outside and pixel centres at
  ((c + 1) n - 1) / 2 (grid_sample without aligned corners), of the spectrum
  at (x, y, sqrt(x^2 (W depth / (2D width))^2 + y^2 (H depth / (2D height))^2
  + z^2)), weighted by |z| / max(that root, 1e-6) for z > 0 and 0 otherwise;
* ``fk_migration(transient, depth, height, width)`` (fk_migration.py:88-120):
  sqrt(transient) scaled by linspace(0, 1, D) along time, zero-padded to 2D
  bins, centred 3-D FFT, Stolt resampling, inverse FFT of the un-centred
  result, magnitude of the first D bins.
"""
import numpy as np


def _unnormalise(c, n):
    return ((c + 1.0) * n - 1.0) / 2.0


def _trilinear(vol, pd, ph, pw):
    """vol [M, D2, H, W] complex; coordinates [D2, H, W] in pixel units."""
    M, D2, H, W = vol.shape
    out = np.zeros((M,) + pd.shape, np.complex128)
    d0, h0, w0 = np.floor(pd).astype(np.int64), np.floor(ph).astype(np.int64), \
        np.floor(pw).astype(np.int64)
    fd, fh, fw = pd - d0, ph - h0, pw - w0
    for dd in (0, 1):
        for hh in (0, 1):
            for ww in (0, 1):
                d, h, w = d0 + dd, h0 + hh, w0 + ww
                wt = (fd if dd else 1 - fd) * (fh if hh else 1 - fh) * (fw if ww else 1 - fw)
                ok = (d >= 0) & (d < D2) & (h >= 0) & (h < H) & (w >= 0) & (w < W)
                dc, hc, wc = np.clip(d, 0, D2 - 1), np.clip(h, 0, H - 1), np.clip(w, 0, W - 1)
                out += np.where(ok, wt, 0.0)[None] * vol[:, dc, hc, wc]
    return out


def stolt(fourier, depth, height, width):
    """fourier [..., 2D, H, W] complex (centred) -> same shape."""
    shape = fourier.shape
    D2, H, W = shape[-3:]
    D = D2 // 2
    vol = fourier.reshape((-1, D2, H, W)).astype(np.complex128)
    x = np.linspace(-1, 1, W)[None, None, :]
    y = np.linspace(-1, 1, H)[None, :, None]
    z = np.linspace(-1, 1, D2)[:, None, None]
    zz = np.sqrt(x ** 2 * ((W * depth) / (2 * D * width)) ** 2
                 + y ** 2 * ((H * depth) / (2 * D * height)) ** 2 + z ** 2)
    full = np.broadcast_to
    pd = _unnormalise(zz, D2)
    ph = _unnormalise(full(y, zz.shape), H)
    pw = _unnormalise(full(x, zz.shape), W)
    out = _trilinear(vol, pd, ph, pw)
    weight = (z > 0) * np.abs(z) / np.maximum(zz, 1e-6)
    return (out * weight[None]).reshape(shape)


def fk_migration(transient, depth, height, width):
    """transient [N, D, H, W] -> volume [N, D, H, W] (float64)."""
    t = np.asarray(transient, np.float64)
    N, D, H, W = t.shape
    t = np.sqrt(t) * np.linspace(0, 1, D)[None, :, None, None]
    t = np.concatenate([t, np.zeros_like(t)], axis=1)
    axes = (1, 2, 3)
    f = np.fft.fftshift(np.fft.fftn(t, axes=axes), axes=axes)
    f = stolt(f, depth, height, width)
    v = np.fft.ifftn(np.fft.ifftshift(f, axes=axes), axes=axes)
    return np.abs(v[:, :D])
