"""Helpers shared by the drop-in ``totri_cpp`` functions."""
import ctypes

import torch

from .. import _lib


def dense_out(t):
    """A C-contiguous tensor to write into (t itself when already dense)."""
    return t if t.is_contiguous() else torch.empty_like(t, memory_format=torch.contiguous_format)


def finish_out(t, out):
    if out is not t:
        t.copy_(out)


def mesh_workspace(B, V, F, P, device, extra=0):
    """Scratch for one mesh call (BVH + visibility masks, then `extra` bytes),
    from the caching allocator."""
    n = int(_lib.load().totri_mesh_workspace(int(B), int(V), int(F), int(P)))
    if n == 0:
        return None
    return torch.empty(n + int(extra), dtype=torch.uint8, device=device)


def exhaustive_grad_scratch(S, L, T):
    """Bytes of the exhaustive gradient's optional bins-last scratch."""
    return int(_lib.load().totri_mesh_exhaustive_grad_scratch(int(S), int(L), int(T)))


# Status bits that report internal errors (a BVH search at its limit, an index
# read from device data out of range in the bounds-checking build); the face
# index bit reports an input and is documented behaviour.
INTERNAL_STATUS = 2 | 4


def check_device_status(ws, device):
    """Bounds-checking build only: synchronises and raises RuntimeError when the
    call whose workspace is `ws` raised an internal-error status bit."""
    from .. import build
    if ws is None or not build.bounds_check():
        return
    flags = ctypes.c_uint32(0)
    _lib.load().totri_mesh_workspace_status(ctypes.c_void_p(ws.data_ptr()), ws.numel(),
                                            ctypes.byref(flags), _lib.stream_of(device))
    if flags.value & INTERNAL_STATUS:
        raise RuntimeError("device status flags 0x%x after a mesh call" % flags.value)


def ws_args(ws):
    if ws is None:
        return ctypes.c_void_p(None), 0
    return ctypes.c_void_p(ws.data_ptr()), ws.numel()
