"""Drop-in for ``totri_cpp.render`` (reference src/totri.cpp:28-46).

Same function names, argument order, tensor layouts and in-place output
semantics as the reference's pybind11 functions; each call enqueues the
sm_103a kernels of libtotri_gb300.so on the current CUDA stream.
"""
import torch

from .. import _lib
from ._common import (check_device_status, dense_out, exhaustive_grad_scratch, finish_out,
                      mesh_workspace, ws_args)


def _mesh_call(name, tensors, bw, bo, model, points, extra=0):
    lib = _lib.load()
    verts, faces = tensors[0], tensors[1]
    ws = mesh_workspace(verts.shape[0], verts.shape[1], faces.shape[1], points, verts.device,
                        extra)
    st = getattr(lib, name)(*[_lib.array(t) for t in tensors], float(bw), float(bo), int(model),
                            *ws_args(ws), _lib.stream_of(verts.device))
    _lib.check(st)
    check_device_status(ws, verts.device)
    return ws


def mesh_confocal_forward(verts, faces, material, scan_points, scan_origin, transient,
                          bin_width, bin_offset, model):
    """transient [B,T,S] <- confocal render (reference src/render/mesh.cpp:9-20)."""
    _lib.require_cuda(verts, faces, material, scan_points, scan_origin, transient)
    out = dense_out(transient)
    _mesh_call("totri_mesh_confocal_forward",
               (verts, faces, material, scan_points, scan_origin, out), bin_width, bin_offset,
               model, scan_points.shape[1])
    finish_out(transient, out)


def mesh_confocal_grad_verts(verts, faces, material, scan_points, scan_origin, transient_grad,
                             verts_grad, material_grad, bin_width, bin_offset, model):
    """verts_grad, material_grad <- d loss (reference src/render/mesh.cpp:22-36)."""
    _lib.require_cuda(verts, faces, material, scan_points, scan_origin, transient_grad,
                      verts_grad, material_grad)
    _mesh_call("totri_mesh_confocal_grad_verts",
               (verts, faces, material, scan_points, scan_origin,
                transient_grad.contiguous(), verts_grad, material_grad),
               bin_width, bin_offset, model, scan_points.shape[1])


def mesh_confocal_forward_unoccluded(verts, faces, material, scan_points, scan_origin,
                                     transient, bin_width, bin_offset, model):
    """mesh_confocal_forward with every (scan point, face) pair visible: the
    unoccluded three-bounce render (an extension; the reference always tests
    visibility)."""
    _lib.require_cuda(verts, faces, material, scan_points, scan_origin, transient)
    out = dense_out(transient)
    _mesh_call("totri_mesh_confocal_forward_unoccluded",
               (verts, faces, material, scan_points, scan_origin, out), bin_width, bin_offset,
               model, scan_points.shape[1])
    finish_out(transient, out)


def mesh_confocal_grad_verts_unoccluded(verts, faces, material, scan_points, scan_origin,
                                        transient_grad, verts_grad, material_grad, bin_width,
                                        bin_offset, model):
    """mesh_confocal_grad_verts of the unoccluded render."""
    _lib.require_cuda(verts, faces, material, scan_points, scan_origin, transient_grad,
                      verts_grad, material_grad)
    _mesh_call("totri_mesh_confocal_grad_verts_unoccluded",
               (verts, faces, material, scan_points, scan_origin,
                transient_grad.contiguous(), verts_grad, material_grad),
               bin_width, bin_offset, model, scan_points.shape[1])


def mesh_exhaustive_forward(verts, faces, material, scan_points, laser_points, scan_origin,
                            laser_origin, transient, bin_width, bin_offset, model):
    """transient [B,T,S,L] <- exhaustive render (reference src/render/mesh.cpp:38-52)."""
    _lib.require_cuda(verts, faces, material, scan_points, laser_points, scan_origin,
                      laser_origin, transient)
    out = dense_out(transient)
    _mesh_call("totri_mesh_exhaustive_forward",
               (verts, faces, material, scan_points, laser_points, scan_origin, laser_origin,
                out), bin_width, bin_offset, model,
               scan_points.shape[1] + laser_points.shape[1])
    finish_out(transient, out)


def mesh_exhaustive_grad_verts(verts, faces, material, scan_points, laser_points, scan_origin,
                               laser_origin, transient_grad, verts_grad, material_grad,
                               bin_width, bin_offset, model):
    """verts_grad, material_grad <- d loss (reference src/render/mesh.cpp:54-71)."""
    _lib.require_cuda(verts, faces, material, scan_points, laser_points, scan_origin,
                      laser_origin, transient_grad, verts_grad, material_grad)
    _mesh_call("totri_mesh_exhaustive_grad_verts",
               (verts, faces, material, scan_points, laser_points, scan_origin, laser_origin,
                transient_grad.contiguous(), verts_grad, material_grad),
               bin_width, bin_offset, model, scan_points.shape[1] + laser_points.shape[1],
               exhaustive_grad_scratch(scan_points.shape[1], laser_points.shape[1],
                                       transient_grad.shape[1]))


def _vol_call(name, tensors, a3, b3, bw, bo, device, voxels=None):
    """Calls a volume entry point; `voxels` (voxels per batch item) adds the
    occupied-voxel scratch those entry points need."""
    lib = _lib.load()
    extra = ()
    if voxels is not None:
        n = int(lib.totri_volume_workspace(int(voxels)))
        ws = torch.empty(max(n, 1), dtype=torch.uint8, device=device)
        extra = ws_args(ws)
    st = getattr(lib, name)(*[_lib.array(t) for t in tensors], _lib.vec3(a3), _lib.vec3(b3),
                            float(bw), float(bo), *extra, _lib.stream_of(device))
    _lib.check(st)


def volume_confocal_forward(volume, measurement_points, transient, volume_origin, volume_size,
                            bin_width, bin_offset):
    """transient [N,T] <- volume [X,Y,Z] (reference src/render/volume.cpp:7-23)."""
    _lib.require_cuda(volume, measurement_points, transient)
    if measurement_points.shape[1] != transient.shape[0]:
        raise ValueError("Measurement and transient dimensions do not match.")
    out = dense_out(transient)
    _vol_call("totri_volume_confocal_forward", (volume.contiguous(), measurement_points, out),
              volume_origin, volume_size, bin_width, bin_offset, volume.device, volume.numel())
    finish_out(transient, out)


def volume_confocal_grad_volume(volume, measurement_points, transient, volume_origin,
                                volume_size, bin_width, bin_offset):
    """volume [X,Y,Z] <- transposed render of transient [N,T]
    (reference src/render/volume.cpp:25-41)."""
    _lib.require_cuda(volume, measurement_points, transient)
    if measurement_points.shape[1] != transient.shape[0]:
        raise ValueError("Measurement and transient dimensions do not match.")
    out = dense_out(volume)
    _vol_call("totri_volume_confocal_grad_volume",
              (out, measurement_points, transient.contiguous()), volume_origin, volume_size,
              bin_width, bin_offset, volume.device)
    finish_out(volume, out)


def volume_confocal_adjoint(volume, measurement_points, transient, volume_origin, volume_size,
                            bin_width, bin_offset):
    """volume [X,Y,Z] <- exact adjoint of volume_confocal_forward (no reference counterpart)."""
    _lib.require_cuda(volume, measurement_points, transient)
    out = dense_out(volume)
    _vol_call("totri_volume_confocal_adjoint",
              (out, measurement_points, transient.contiguous()), volume_origin, volume_size,
              bin_width, bin_offset, volume.device)
    finish_out(volume, out)


def volume_confocal_grad_measurement_points(measurement_points_grad, volume,
                                            measurement_points, transient_grad, volume_origin,
                                            volume_size, bin_width, bin_offset):
    """measurement_points_grad [3,N] (reference src/render/volume.cpp:43-81)."""
    _lib.require_cuda(measurement_points_grad, volume, measurement_points, transient_grad)
    out = dense_out(measurement_points_grad)
    _vol_call("totri_volume_confocal_grad_measurement_points",
              (out, volume.contiguous(), measurement_points, transient_grad.contiguous()),
              volume_origin, volume_size, bin_width, bin_offset, volume.device, volume.numel())
    finish_out(measurement_points_grad, out)


def volume_render_exhaustive_forward(volume, scan_points, laser_points, scan_origin,
                                     laser_origin, transient, volume_start, volume_end,
                                     bin_width, bin_offset):
    """transient [B,T,S,L] <- volume [B,D,H,W] (reference src/render/volume.cpp:83-96)."""
    _lib.require_cuda(volume, scan_points, laser_points, scan_origin, laser_origin, transient)
    out = dense_out(transient)
    _vol_call("totri_volume_exhaustive_forward",
              (volume.contiguous(), scan_points, laser_points, scan_origin, laser_origin, out),
              volume_start, volume_end, bin_width, bin_offset, volume.device,
              volume[0].numel() if volume.shape[0] > 0 else 0)
    finish_out(transient, out)


def volume_render_exhaustive_grad_volume(transient_grad, scan_points, laser_points, scan_origin,
                                         laser_origin, volume_grad, volume_start, volume_end,
                                         bin_width, bin_offset):
    """volume_grad [B,D,H,W] <- adjoint of the exhaustive volume render
    (reference src/render/volume.cpp:98-111, whose kernel body is empty)."""
    _lib.require_cuda(transient_grad, scan_points, laser_points, scan_origin, laser_origin,
                      volume_grad)
    out = dense_out(volume_grad)
    _vol_call("totri_volume_exhaustive_grad_volume",
              (transient_grad.contiguous(), scan_points, laser_points, scan_origin,
               laser_origin, out), volume_start, volume_end, bin_width, bin_offset,
              volume_grad.device)
    finish_out(volume_grad, out)


def mesh_visibility(verts, faces, points, brute_force=False):
    """int32 [B,P,ceil(F/32)] visibility bit masks (diagnostics; no reference counterpart)."""
    _lib.require_cuda(verts, faces, points)
    lib = _lib.load()
    B, V, F, P = verts.shape[0], verts.shape[1], faces.shape[1], points.shape[1]
    mask = torch.zeros((B, P, (F + 31) // 32), dtype=torch.int32, device=verts.device)
    ws = mesh_workspace(B, V, F, P, verts.device)
    st = lib.totri_mesh_visibility(_lib.array(verts), _lib.array(faces), _lib.array(points),
                                   _lib.array(mask), int(bool(brute_force)), *ws_args(ws),
                                   _lib.stream_of(verts.device))
    _lib.check(st)
    return mask
