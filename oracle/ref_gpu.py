"""The reference's own volume, backprojection and RBF kernels on the GPU (TEST
INFRASTRUCTURE: a same-device parity anchor for those operators and the
baseline that ``bench.py --impl reference`` times beside its CPU leg).

``oracle/ref_harness.py`` compiles them for sm_103a into
``oracle/_ref/ref_kernels.cubin`` where the reference tree is present; this
module loads that image through the CUDA driver (libcuda, via ctypes) into the
current context and launches each kernel with the grid and block of the
reference's host launcher, on torch's current stream, over contiguous FP32
CUDA tensors. Outputs that the reference launchers zero are zeroed here. The
functions mirror the ``ref_*`` functions of oracle/ref_harness/
kernel_driver.cpp (the same kernels built for the CPU).
"""
import ctypes
import os

import torch

CUBIN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "_ref", "ref_kernels.cubin")

_state = {}


class _F3(ctypes.Structure):
    _fields_ = [("x", ctypes.c_float), ("y", ctypes.c_float), ("z", ctypes.c_float)]


def available():
    return os.path.exists(CUBIN) and torch.cuda.is_available()


def _cu(status, what):
    if status != 0:
        raise RuntimeError("CUDA driver error %d in %s" % (status, what))


def _module():
    if "mod" in _state:
        return _state
    cuda = ctypes.CDLL("libcuda.so.1")
    torch.zeros(1, device="cuda")  # the runtime's primary context becomes current
    ctx = ctypes.c_void_p()
    _cu(cuda.cuCtxGetCurrent(ctypes.byref(ctx)), "cuCtxGetCurrent")
    if not ctx.value:
        raise RuntimeError("no current CUDA context")
    mod = ctypes.c_void_p()
    _cu(cuda.cuModuleLoad(ctypes.byref(mod), CUBIN.encode()), "cuModuleLoad")
    cuda.cuLaunchKernel.argtypes = [ctypes.c_void_p] + [ctypes.c_uint] * 7 + [
        ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    _state.update(cuda=cuda, mod=mod, fn={})
    return _state


def _launch(name, grid, block, args):
    st = _module()
    fn = st["fn"].get(name)
    if fn is None:
        fn = ctypes.c_void_p()
        _cu(st["cuda"].cuModuleGetFunction(ctypes.byref(fn), st["mod"], name.encode()), name)
        st["fn"][name] = fn
    vals = []
    for a in args:
        if isinstance(a, torch.Tensor):
            vals.append(ctypes.c_void_p(a.data_ptr()))
        elif isinstance(a, float):
            vals.append(ctypes.c_float(a))
        elif isinstance(a, int):
            vals.append(ctypes.c_int(a))
        else:  # a 3-vector
            vals.append(_F3(*[float(x) for x in a]))
    params = (ctypes.c_void_p * len(vals))(*[ctypes.cast(ctypes.pointer(v), ctypes.c_void_p)
                                             for v in vals])
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    g = list(grid) + [1] * (3 - len(grid))
    b = list(block) + [1] * (3 - len(block))
    _cu(st["cuda"].cuLaunchKernel(fn, *g, *b, 0, stream, params, None), name)


def _cdiv(a, b):
    return (a + b - 1) // b


def _check(*ts):
    for t in ts:
        if not (t.is_cuda and t.dtype == torch.float32 and t.is_contiguous()):
            raise ValueError("contiguous float32 CUDA tensors only")


def volume_confocal_forward(volume, mp, transient, origin, size, bw, bo):
    """volume [X,Y,Z], mp [3,N] -> transient [N,T] (volume_cuda.cu:68-93)."""
    _check(volume, mp, transient)
    X, Y, Z = volume.shape
    N, T = transient.shape
    _launch("ref_volume_confocal_forward", (_cdiv(N, 8), _cdiv(T, 8)), (8, 8),
            [volume, X, Y, Z, mp, N, transient, T, origin, size, float(bw), float(bo)])


def volume_confocal_grad_volume(volume, mp, transient, origin, size, bw, bo):
    """transient [N,T] -> volume [X,Y,Z] (volume_cuda.cu:161-186)."""
    _check(volume, mp, transient)
    X, Y, Z = volume.shape
    N, T = transient.shape
    _launch("ref_volume_confocal_grad_volume", (_cdiv(X, 8), _cdiv(Y, 8), _cdiv(Z, 8)),
            (8, 8, 8), [volume, X, Y, Z, mp, N, transient, T, origin, size, float(bw),
                        float(bo)])


def volume_confocal_grad_mp(mpg, volume, mp, tgrad, origin, size, bw, bo):
    """d loss / d measurement points [3,N] (volume_cuda.cu:267-295)."""
    _check(mpg, volume, mp, tgrad)
    X, Y, Z = volume.shape
    N, T = tgrad.shape
    mpg.zero_()
    _launch("ref_volume_confocal_grad_mp", (_cdiv(N, 8), _cdiv(T, 8)), (8, 8),
            [mpg, volume, X, Y, Z, mp, N, tgrad, T, origin, size, float(bw), float(bo)])


def volume_exhaustive_forward(volume, sp, lp, so, lo, transient, start, end, bw, bo):
    """volume [B,D,H,W], points [B,3,S]/[B,3,L] -> transient [B,T,S,L]
    (volume_cuda.cu:379-412)."""
    _check(volume, sp, lp, so, lo, transient)
    B, D, H, W = volume.shape
    S, L, T = sp.shape[2], lp.shape[2], transient.shape[1]
    transient.zero_()
    for b in range(B):
        _launch("ref_volume_exhaustive_forward", (_cdiv(H * W, 8), _cdiv(S, 8), _cdiv(L, 8)),
                (8, 8, 8), [volume, B, D, H, W, sp, S, lp, L, so, so.shape[2], lo, lo.shape[2],
                            transient, T, start, end, float(bw), float(bo), b])


def backprojection_confocal_velten(transient, sp, so, volume, start, end, bw, bo):
    """transient [B,T,S], sp [B,S,3] -> volume [B,D,H,W] (backprojection_cuda.cu:196-226)."""
    _check(transient, sp, so, volume)
    B, T, S = transient.shape
    D, H, W = volume.shape[1:]
    for b in range(B):
        _launch("ref_backprojection_confocal_velten", (_cdiv(W, 8), _cdiv(H, 8), _cdiv(D, 8)),
                (8, 8, 8), [transient, B, T, sp, S, so, so.shape[1], volume, D, H, W, start,
                            end, float(bw), float(bo), b])


def backprojection_exhaustive_velten(transient, sp, lp, so, lo, volume, start, end, bw, bo):
    """transient [B,T,S,L], sp [B,S,3], lp [B,L,3] -> volume [B,D,H,W]
    (backprojection_cuda.cu:289-322)."""
    _check(transient, sp, lp, so, lo, volume)
    B, T, S, L = transient.shape
    D, H, W = volume.shape[1:]
    for b in range(B):
        _launch("ref_backprojection_exhaustive_velten", (_cdiv(W, 8), _cdiv(H, 8), _cdiv(D, 8)),
                (8, 8, 8), [transient, B, T, sp, S, lp, L, so, so.shape[1], lo, lo.shape[1],
                            volume, D, H, W, start, end, float(bw), float(bo), b])


def backprojection_exhaustive_arellano(transient, sp, lp, so, lo, volume, start, end, bw, bo):
    """transient [B,T,S,L], sp [B,3,S], lp [B,3,L] -> volume [B,D,H,W] (zeroed, then
    accumulated; backprojection_cuda.cu:117-150)."""
    _check(transient, sp, lp, so, lo, volume)
    B, T, S, L = transient.shape
    D, H, W = volume.shape[1:]
    volume.zero_()
    for b in range(B):
        _launch("ref_backprojection_exhaustive_arellano", (_cdiv(H * W, 64), S, L), (64,),
                [transient, B, T, sp, S, lp, L, so, so.shape[2], lo, lo.shape[2], volume, D, H,
                 W, start, end, float(bw), float(bo), b])


def rbf2volume_forward(rbf, volume, start, end):
    """rbf [B,N,4+A] -> volume [B,1+A,D,H,W] (rbf2volume_cuda.cu:95-117)."""
    _check(rbf, volume)
    B, N, C = rbf.shape
    D, H, W = volume.shape[2:]
    for b in range(B):
        _launch("ref_rbf2volume_forward", (_cdiv(W, 4), _cdiv(H, 4), _cdiv(D, 4)), (4, 4, 4),
                [rbf, B, N, C, volume, D, H, W, start, end, b])


def rbf2volume_grad(rbf, volume, volume_grad, rbf_grad, start, end):
    """d loss / d rbf [B,N,4+A] (zeroed, then accumulated; rbf2volume_cuda.cu:203-229)."""
    _check(rbf, volume, volume_grad, rbf_grad)
    B, N, C = rbf.shape
    D, H, W = volume.shape[2:]
    rbf_grad.zero_()
    for b in range(B):
        _launch("ref_rbf2volume_grad", (_cdiv(W * H, 16), _cdiv(D, 4), N), (16, 4, 1),
                [rbf, B, N, C, volume, volume_grad, D, H, W, rbf_grad, start, end, b])
