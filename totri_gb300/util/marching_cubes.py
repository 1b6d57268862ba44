"""Differentiable marching cubes: the drop-in for ``tomcubes.MarchingCubesFunction``.

The reference builds meshes from RBF volumes with
``MarchingCubesFunction.apply(volume[None], iso, volume_def.start,
volume_def.end)[0]`` (totri/fitting/rbf.py:88-98, rbf_backup.py:154-160) and
renders the result as consecutive vertex triples (``faces_of_verts(verts,
None)``, rbf.py:719) with channels 3.. as colours (rbf.py:253-258). tomcubes
is an un-vendored submodule of the reference (.gitmodules:4-6), so the
conventions here follow those call sites: input [B, 1+A, D, H, W] (channel 0
the field, channels 1.. attributes), output [B, N, 3+A] (x, y, z, then the
attributes interpolated along the same cell edges), N = 3 x triangles of the
largest item; rows past an item's own vertices are zero (degenerate
triangles at the origin, which render to nothing). A grid point is inside
when its value is above ``iso``; triangles face from inside to outside.
Gradients flow to the volume (all channels) through the edge interpolation;
the triangulation itself is piecewise constant.
"""
import ctypes

import torch

from .. import _lib


def _workspace(volume):
    B, _, D, H, W = volume.shape
    n = int(_lib.load().totri_marching_cubes_workspace(B, D, H, W))
    return torch.empty(max(n, 1), dtype=torch.uint8, device=volume.device), n


def marching_cubes(volume: torch.Tensor, iso: float, volume_start, volume_end):
    """(verts [B, N, 3+A], edges [B, N] int64, triangles [B] int64) of
    volume [B, 1+A, D, H, W] (float32, CUDA)."""
    _lib.require_cuda(volume)
    if volume.dim() != 5:
        raise ValueError("volume must be [B, 1+A, D, H, W]")
    volume = volume.detach().contiguous().float()
    lib = _lib.load()
    stream = _lib.stream_of(volume.device)
    B, C = volume.shape[:2]
    tri = torch.zeros(B, dtype=torch.int64, device=volume.device)
    ws, n = _workspace(volume)
    ptr = ctypes.c_void_p(ws.data_ptr())
    _lib.check(lib.totri_marching_cubes_count(_lib.array(volume), float(iso), _lib.array(tri),
                                              ptr, n, stream))
    rows = 3 * int(tri.max().item()) if B > 0 else 0
    verts = torch.zeros((B, rows, 2 + C), dtype=torch.float32, device=volume.device)
    edges = torch.full((B, rows), -1, dtype=torch.int64, device=volume.device)
    if rows > 0:
        _lib.check(lib.totri_marching_cubes_emit(
            _lib.array(volume), float(iso), _lib.vec3(volume_start), _lib.vec3(volume_end),
            _lib.array(verts), _lib.array(edges), ptr, n, stream))
    return verts, edges, tri


def marching_cubes_grad(volume, iso, volume_start, volume_end, edges, verts_grad):
    """d loss / d volume for verts_grad [B, N, 3+A] at the vertices of ``edges``."""
    _lib.require_cuda(volume, edges, verts_grad)
    volume = volume.detach().contiguous().float()
    out = torch.zeros_like(volume)
    if edges.numel() > 0:
        _lib.check(_lib.load().totri_marching_cubes_grad(
            _lib.array(volume), float(iso), _lib.vec3(volume_start), _lib.vec3(volume_end),
            _lib.array(edges.contiguous()), _lib.array(verts_grad.contiguous().float()),
            _lib.array(out), _lib.stream_of(volume.device)))
    return out


class MarchingCubesFunction(torch.autograd.Function):
    """apply(volume [B, 1+A, D, H, W], iso, start, end) -> verts [B, N, 3+A]."""

    @staticmethod
    def forward(ctx, volume, iso, volume_start, volume_end):
        verts, edges, _ = marching_cubes(volume, iso, volume_start, volume_end)
        ctx.save_for_backward(volume, edges)
        ctx.args = (float(iso), tuple(volume_start), tuple(volume_end))
        ctx.mark_non_differentiable(edges)
        return verts

    @staticmethod
    def backward(ctx, verts_grad):
        volume, edges = ctx.saved_tensors
        grad = None
        if ctx.needs_input_grad[0] and verts_grad is not None:
            iso, start, end = ctx.args
            grad = marching_cubes_grad(volume, iso, start, end, edges, verts_grad)
            grad = grad.to(volume.dtype)
        return grad, None, None, None
