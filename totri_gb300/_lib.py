"""ctypes binding of libtotri_gb300.so (the C ABI in include/totri_gb300.h).

The product path has no fallback: if the shared library is missing or fails to
load, every operator raises. Build it with ``totri_gb300.build.build()`` (or
``__graft_entry__.build()``).
"""
import ctypes
import os
import threading

import torch

from . import build as _build

MAX_DIMS = 5

TOTRI_OK = 0
TOTRI_ERR_INVALID_ARGUMENT = 1
TOTRI_ERR_WORKSPACE = 2
TOTRI_ERR_CUDA = 3
TOTRI_ERR_UNSUPPORTED = 4
TOTRI_ERR_DEVICE = 5

_DTYPES = {
    torch.float32: 0,
    torch.float64: 1,
    torch.int32: 2,
    torch.int64: 3,
}


class Array(ctypes.Structure):
    """totri_array_t: device pointer, dtype, rank, shape and element strides."""
    _fields_ = [
        ("data", ctypes.c_void_p),
        ("dtype", ctypes.c_int32),
        ("ndim", ctypes.c_int32),
        ("shape", ctypes.c_int64 * MAX_DIMS),
        ("strides", ctypes.c_int64 * MAX_DIMS),
    ]


class Shading(ctypes.Structure):
    """totri_shading_t: camera, light, material and blend settings of the
    shaded preview rasteriser."""
    _fields_ = [
        ("rotation", ctypes.c_float * 9),
        ("translation", ctypes.c_float * 3),
        ("focal", ctypes.c_float * 2),
        ("znear", ctypes.c_float),
        ("zfar", ctypes.c_float),
        ("camera_center", ctypes.c_float * 3),
        ("light_location", ctypes.c_float * 3),
        ("light_ambient", ctypes.c_float * 3),
        ("light_diffuse", ctypes.c_float * 3),
        ("light_specular", ctypes.c_float * 3),
        ("material_ambient", ctypes.c_float * 3),
        ("material_diffuse", ctypes.c_float * 3),
        ("material_specular", ctypes.c_float * 3),
        ("shininess", ctypes.c_float),
        ("background", ctypes.c_float * 3),
        ("sigma", ctypes.c_float),
        ("gamma", ctypes.c_float),
    ]


_ArrP = ctypes.POINTER(Array)
_F3 = ctypes.c_float * 3
_vp = ctypes.c_void_p
_sz = ctypes.c_size_t
_i64 = ctypes.c_int64
_flt = ctypes.c_float
_int = ctypes.c_int

# name -> argtypes (restype int unless listed in _RESTYPES)
_SIGNATURES = {
    "totri_version": [],
    "totri_last_error": [],
    "totri_tune_set": [ctypes.c_char_p, _int],
    "totri_tune_get": [ctypes.c_char_p],
    "totri_fill_normal": [_vp, _i64, ctypes.c_uint64, _vp],
    "totri_profile_enable": [_int],
    "totri_profile_reset": [],
    "totri_profile_read": [_int, ctypes.c_char_p, ctypes.POINTER(ctypes.c_int64),
                           ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(ctypes.c_double),
                           ctypes.POINTER(ctypes.c_int)],
    "totri_mesh_workspace": [_i64, _i64, _i64, _i64],
    "totri_mesh_exhaustive_grad_scratch": [_i64, _i64, _i64],
    "totri_mesh_confocal_forward": [_ArrP] * 6 + [_flt, _flt, _int, _vp, _sz, _vp],
    "totri_mesh_confocal_grad_verts": [_ArrP] * 8 + [_flt, _flt, _int, _vp, _sz, _vp],
    "totri_mesh_confocal_grad_verts_reuse": [_ArrP] * 8 + [_flt, _flt, _int, _vp, _sz, _vp],
    "totri_mesh_confocal_forward_unoccluded": [_ArrP] * 6 + [_flt, _flt, _int, _vp, _sz, _vp],
    "totri_mesh_confocal_grad_verts_unoccluded": [_ArrP] * 8 + [_flt, _flt, _int, _vp, _sz,
                                                               _vp],
    "totri_mesh_exhaustive_forward": [_ArrP] * 8 + [_flt, _flt, _int, _vp, _sz, _vp],
    "totri_mesh_exhaustive_grad_verts": [_ArrP] * 10 + [_flt, _flt, _int, _vp, _sz, _vp],
    "totri_mesh_exhaustive_grad_verts_reuse": [_ArrP] * 10 + [_flt, _flt, _int, _vp, _sz, _vp],
    "totri_mesh_visibility": [_ArrP] * 4 + [_int, _vp, _sz, _vp],
    "totri_mesh_workspace_status": [_vp, _sz, ctypes.POINTER(ctypes.c_uint32), _vp],
    "totri_mesh_mask_bytes": [_i64, _i64, _i64],
    "totri_mesh_prepare": [_ArrP] * 3 + [_vp, _sz, _vp],
    "totri_mesh_prepared_visibility": [_ArrP] * 4 + [_vp, _sz, _vp, _sz, _vp],
    "totri_mesh_prepared_confocal_forward": [_ArrP] * 6 + [_flt, _flt, _vp, _sz, _vp, _sz, _vp],
    "totri_mesh_prepared_confocal_grad_verts": [_ArrP] * 8 + [_flt, _flt, _vp, _sz, _vp, _sz,
                                                              _vp],
    "totri_volume_workspace": [_i64],
    "totri_volume_confocal_forward": [_ArrP] * 3 + [_F3, _F3, _flt, _flt, _vp, _sz, _vp],
    "totri_volume_confocal_grad_volume": [_ArrP] * 3 + [_F3, _F3, _flt, _flt, _vp],
    "totri_volume_confocal_adjoint": [_ArrP] * 3 + [_F3, _F3, _flt, _flt, _vp],
    "totri_volume_confocal_grad_measurement_points": [_ArrP] * 4 + [_F3, _F3, _flt, _flt, _vp,
                                                                    _sz, _vp],
    "totri_volume_exhaustive_forward": [_ArrP] * 6 + [_F3, _F3, _flt, _flt, _vp, _sz, _vp],
    "totri_volume_exhaustive_grad_volume": [_ArrP] * 6 + [_F3, _F3, _flt, _flt, _vp],
    "totri_backprojection_confocal_velten_forward": [_ArrP] * 4 + [_F3, _F3, _flt, _flt, _vp],
    "totri_backprojection_confocal_velten_adjoint": [_ArrP] * 4 + [_F3, _F3, _flt, _flt, _vp],
    "totri_backprojection_exhaustive_velten_forward": [_ArrP] * 6 + [_F3, _F3, _flt, _flt, _vp],
    "totri_backprojection_exhaustive_arellano_forward": [_ArrP] * 6 + [_F3, _F3, _flt, _flt,
                                                                       _vp],
    "totri_rbf2volume_gaussian_forward": [_ArrP] * 2 + [_F3, _F3, _vp],
    "totri_rbf2volume_gaussian_grad": [_ArrP] * 4 + [_F3, _F3, _vp],
    "totri_depth_raster_workspace": [_i64, _i64],
    "totri_depth_raster": [_ArrP] * 4 + [_flt] * 6 + [_vp, _sz, _vp],
    "totri_shaded_raster_workspace": [_i64, _i64, _i64],
    "totri_shaded_raster": [_ArrP, _ArrP, _ArrP, ctypes.POINTER(Shading), _ArrP, _ArrP, _vp,
                            _sz, _vp],
    "totri_fk_prepare": [_ArrP, _ArrP, _vp],
    "totri_fk_stolt": [_ArrP, _ArrP, _flt, _flt, _flt, _int, _int, _vp],
    "totri_fk_finish": [_ArrP, _ArrP, _vp],
    "totri_marching_cubes_workspace": [_i64, _i64, _i64, _i64],
    "totri_marching_cubes_count": [_ArrP, _flt, _ArrP, _vp, _sz, _vp],
    "totri_marching_cubes_emit": [_ArrP, _flt, _F3, _F3, _ArrP, _ArrP, _vp, _sz, _vp],
    "totri_marching_cubes_grad": [_ArrP, _flt, _F3, _F3, _ArrP, _ArrP, _ArrP, _vp],
    "totri_marching_cubes_table": [ctypes.POINTER(ctypes.c_uint8),
                                   ctypes.POINTER(ctypes.c_int8)],
}
_RESTYPES = {
    "totri_version": ctypes.c_char_p,
    "totri_last_error": ctypes.c_char_p,
    "totri_mesh_workspace": ctypes.c_size_t,
    "totri_mesh_exhaustive_grad_scratch": ctypes.c_size_t,
    "totri_mesh_mask_bytes": ctypes.c_size_t,
    "totri_volume_workspace": ctypes.c_size_t,
    "totri_marching_cubes_workspace": ctypes.c_size_t,
    "totri_depth_raster_workspace": ctypes.c_size_t,
    "totri_shaded_raster_workspace": ctypes.c_size_t,
    "totri_profile_reset": None,
}


def profile_enable(on=True):
    load().totri_profile_enable(int(bool(on)))


def profile_reset():
    load().totri_profile_reset()


def profile_read(max_entries=64):
    """{kernel name: (launches, timed launches, total ms)} since the last reset."""
    names = ctypes.create_string_buffer(64 * max_entries)
    launches = (ctypes.c_int64 * max_entries)()
    timed = (ctypes.c_int64 * max_entries)()
    ms = (ctypes.c_double * max_entries)()
    n = ctypes.c_int(0)
    check(load().totri_profile_read(max_entries, names, launches, timed, ms, ctypes.byref(n)))
    out = {}
    for i in range(n.value):
        name = names.raw[64 * i:64 * (i + 1)].split(b"\0", 1)[0].decode()
        out[name] = (int(launches[i]), int(timed[i]), float(ms[i]))
    return out

_lib = None
_lock = threading.Lock()


def library_path():
    return _build.LIB_PATH


def load():
    """Loads the shared library (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = library_path()
        if not os.path.exists(path):
            raise RuntimeError(
                "totri_gb300 CUDA library not found at %s; run totri_gb300.build.build()" % path)
        handle = ctypes.CDLL(path)
        for name, args in _SIGNATURES.items():
            fn = getattr(handle, name)
            fn.argtypes = args
            fn.restype = _RESTYPES.get(name, ctypes.c_int)
        _lib = handle
    return _lib


def array(t):
    """totri_array_t describing tensor t (no copy)."""
    if t.dim() > MAX_DIMS:
        raise ValueError("tensors of rank > %d are not supported" % MAX_DIMS)
    a = Array()
    a.data = t.data_ptr() if t.numel() > 0 else None
    a.dtype = _DTYPES.get(t.dtype, -1)
    a.ndim = t.dim()
    for i, (s, st) in enumerate(zip(t.shape, t.stride())):
        a.shape[i] = s
        a.strides[i] = st
    return ctypes.byref(a)


def vec3(v):
    return _F3(*[float(x) for x in v])


def stream_of(device):
    return ctypes.c_void_p(torch.cuda.current_stream(device).cuda_stream)


def check(status):
    """Raises the Python exception matching a C status code."""
    if status == TOTRI_OK:
        return
    msg = load().totri_last_error().decode(errors="replace")
    if status == TOTRI_ERR_INVALID_ARGUMENT:
        raise ValueError(msg)
    if status == TOTRI_ERR_UNSUPPORTED:
        raise NotImplementedError(msg)
    raise RuntimeError("totri_gb300 error %d: %s" % (status, msg))


def require_cuda(*tensors):
    for t in tensors:
        if t is not None and not t.is_cuda:
            raise ValueError("totri_gb300 operators take CUDA tensors")
