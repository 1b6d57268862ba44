"""Differentiable mesh transient rendering (reference totri/render/mesh.py:12-168).

``MeshRenderConfocal`` and ``MeshRenderExhaustive`` keep the reference's
``apply`` signatures, argument normalisation and output layouts. Differences:
the output has the batch size of ``verts`` (the reference always allocates a
batch of one, mesh.py:44-46) and lives on the device of ``verts``; the forward
keeps its BVH and visibility masks for the backward instead of rebuilding them.
"""
import typing

import torch

from .. import _lib
from ..totri_cpp._common import exhaustive_grad_scratch, mesh_workspace, ws_args
from ..types import BinDef
from ..util.format import colors_of_verts, faces_of_verts, origin_of_wallpoints


def _needs(ctx):
    """needs_input_grad lookup that treats omitted optional arguments as False."""
    flags = ctx.needs_input_grad
    return lambda i: i < len(flags) and bool(flags[i])


def _run(name, tensors, bin_def, ws, device):
    st = getattr(_lib.load(), name)(*[_lib.array(t) for t in tensors], float(bin_def.width),
                                    float(bin_def.offset), 0, *ws_args(ws),
                                    _lib.stream_of(device))
    _lib.check(st)


class MeshRenderConfocal(torch.autograd.Function):
    """Render mesh to transient image.

    Args:
        verts (torch.Tensor): Vertices [B, V, 3]
        faces (torch.Tensor, optional): Face indices [B, F, 3]
        scan_points (torch.Tensor): Laser/Scan points on the wall [B, S, 3]
        bin_def (BinDef): Bin count, width and offset
        colors (torch.Tensor, optional): Color of each vertex [B, V, 1].
        scan_origin (torch.Tensor, optional): Laser/detector position per scan point
            [B, S, 3], [B, 1, 3] or [B, 3].
        visibility (bool, optional): False renders every (scan point, face) pair
            as visible (the unoccluded render; an extension, default True as the
            reference).

    Returns:
        torch.Tensor: Transient image [B, T, S]
    """

    @staticmethod
    def forward(ctx, verts: torch.Tensor, faces: typing.Optional[torch.Tensor],
                scan_points: torch.Tensor, bin_def: BinDef,
                colors: typing.Optional[torch.Tensor] = None,
                scan_origin: typing.Optional[torch.Tensor] = None,
                visibility: bool = True) -> torch.Tensor:
        _lib.require_cuda(verts, scan_points)
        faces = faces_of_verts(verts, faces)
        colors = colors_of_verts(colors, verts)
        scan_origin = origin_of_wallpoints(scan_origin, scan_points, 'scan_origin')
        ctx.set_materialize_grads(False)
        ctx.save_for_backward(verts, faces, colors, scan_points, scan_origin)
        ctx.bin_def = bin_def
        B, V, F, S = verts.shape[0], verts.shape[1], faces.shape[1], scan_points.shape[1]
        transient = torch.empty((B, bin_def.num, S), device=verts.device, dtype=torch.float32)
        ws = mesh_workspace(B, V, F, S, verts.device)
        _run("totri_mesh_confocal_forward" if visibility
             else "totri_mesh_confocal_forward_unoccluded",
             (verts, faces, colors, scan_points, scan_origin, transient), bin_def, ws,
             verts.device)
        ctx.workspace = ws  # the backward reuses its masks (all visible when unoccluded)
        return transient

    @staticmethod
    def backward(ctx, transient_grad: torch.Tensor):
        grad = [None] * 7
        if transient_grad is None:
            return tuple(grad)
        need = _needs(ctx)
        if need(0) or need(4):
            verts, faces, colors, scan_points, scan_origin = ctx.saved_tensors
            verts_grad = torch.empty_like(verts) if need(0) \
                else torch.empty_like(verts[:, :, :0])
            colors_grad = torch.empty_like(colors) if need(4) \
                else torch.empty_like(colors[:, :, :0])
            _run("totri_mesh_confocal_grad_verts_reuse",
                 (verts, faces, colors, scan_points, scan_origin, transient_grad.contiguous(),
                  verts_grad, colors_grad), ctx.bin_def, ctx.workspace, verts.device)
            if need(0):
                grad[0] = verts_grad
            if need(4):
                grad[4] = colors_grad
        for i in (1, 2, 3, 5):
            if need(i):
                raise NotImplementedError()
        return tuple(grad)


class MeshRenderExhaustive(torch.autograd.Function):
    """Render mesh to transient image with separate laser and detector points.

    Args:
        verts (torch.Tensor): Vertices [B, V, 3]
        faces (torch.Tensor, optional): Face indices [B, F, 3]
        scan_points (torch.Tensor): Scan points on the visible wall [B, S, 3]
        laser_points (torch.Tensor): Laser points on the visible wall [B, L, 3]
        bin_def (BinDef): Bin count, width and offset
        colors (torch.Tensor, optional): Color of each vertex [B, V, 1].
        scan_origin (torch.Tensor, optional): Detector position per scan point.
        laser_origin (torch.Tensor, optional): Laser position per laser point.

    Returns:
        torch.Tensor: Transient image [B, T, S, L]
    """

    @staticmethod
    def forward(ctx, verts: torch.Tensor, faces: typing.Optional[torch.Tensor],
                scan_points: torch.Tensor, laser_points: torch.Tensor, bin_def: BinDef,
                colors: typing.Optional[torch.Tensor] = None,
                scan_origin: typing.Optional[torch.Tensor] = None,
                laser_origin: typing.Optional[torch.Tensor] = None) -> torch.Tensor:
        _lib.require_cuda(verts, scan_points, laser_points)
        faces = faces_of_verts(verts, faces)
        colors = colors_of_verts(colors, verts)
        scan_origin = origin_of_wallpoints(scan_origin, scan_points, 'scan_origin')
        laser_origin = origin_of_wallpoints(laser_origin, laser_points, 'laser_points')
        ctx.set_materialize_grads(False)
        ctx.save_for_backward(verts, faces, colors, scan_points, laser_points, scan_origin,
                              laser_origin)
        ctx.bin_def = bin_def
        B, V, F = verts.shape[0], verts.shape[1], faces.shape[1]
        S, L = scan_points.shape[1], laser_points.shape[1]
        transient = torch.empty((B, bin_def.num, S, L), device=verts.device,
                                dtype=torch.float32)
        # the backward reuses this workspace: room for its bins-last scratch
        # when a gradient will be asked for
        grads = ctx.needs_input_grad[0] or ctx.needs_input_grad[5]
        ws = mesh_workspace(B, V, F, S + L, verts.device,
                            exhaustive_grad_scratch(S, L, bin_def.num) if grads else 0)
        _run("totri_mesh_exhaustive_forward",
             (verts, faces, colors, scan_points, laser_points, scan_origin, laser_origin,
              transient), bin_def, ws, verts.device)
        ctx.workspace = ws
        return transient

    @staticmethod
    def backward(ctx, transient_grad: torch.Tensor):
        grad = [None] * 8
        if transient_grad is None:
            return tuple(grad)
        need = _needs(ctx)
        if need(0) or need(5):
            (verts, faces, colors, scan_points, laser_points, scan_origin,
             laser_origin) = ctx.saved_tensors
            verts_grad = torch.empty_like(verts) if need(0) \
                else torch.empty_like(verts[:, :, :0])
            colors_grad = torch.empty_like(colors) if need(5) \
                else torch.empty_like(colors[:, :, :0])
            _run("totri_mesh_exhaustive_grad_verts_reuse",
                 (verts, faces, colors, scan_points, laser_points, scan_origin, laser_origin,
                  transient_grad.contiguous(), verts_grad, colors_grad), ctx.bin_def,
                 ctx.workspace, verts.device)
            if need(0):
                grad[0] = verts_grad
            if need(5):
                grad[5] = colors_grad
        for i in (1, 2, 3, 4, 6, 7):
            if need(i):
                raise NotImplementedError()
        return tuple(grad)
