"""CPU oracle for the totrilib transient-rendering path (TEST INFRASTRUCTURE).

A C++ restatement of the reference algorithms, bound with ctypes over numpy
arrays. It is the checker for the CUDA path: only tests/,
``__graft_entry__.smoke()`` and the CPU-baseline leg of ``bench.py`` may import
it. Every function handles one batch item; arrays are C-contiguous numpy
arrays (float32 inputs, int64 faces, float64 outputs).

Parity anchors: the restatement is pinned against golden vectors produced by
the reference's own kernel sources compiled for the CPU (``oracle/ref_harness``
and ``tests/golden``).
"""
import ctypes
import os

import numpy as np

from . import build as _build

_lib = None

_f32p = ctypes.POINTER(ctypes.c_float)
_f64p = ctypes.POINTER(ctypes.c_double)
_i64p = ctypes.POINTER(ctypes.c_int64)
_u8p = ctypes.POINTER(ctypes.c_uint8)
_long = ctypes.c_long


_int = ctypes.c_int
_flt = ctypes.c_float

# argtypes of every exported oracle function (all pointers are host pointers).
_SIGNATURES = {
    "oracle_mesh_count_faces": (_long, [_i64p, _long, _long]),
    "oracle_mesh_visibility": (_int, [_f32p, _long, _i64p, _long, _f32p, _long, _u8p]),
    "oracle_mesh_visibility_bvh": (_int, [_f32p, _long, _i64p, _long, _f32p, _long, _u8p]),
    "oracle_mesh_visibility_pairs": (
        _int, [_f32p, _long, _i64p, _long, _f32p, _i64p, _i64p, _long, _u8p]),
    "oracle_mesh_confocal_forward": (
        _int, [_f32p, _long, _i64p, _long, _f32p, _long, _f32p, _long, _f32p, _u8p, _long,
               _flt, _flt, _int, _f64p]),
    "oracle_mesh_confocal_grad": (
        _int, [_f32p, _long, _i64p, _long, _f32p, _long, _f32p, _long, _f32p, _u8p, _long,
               _flt, _flt, _f64p, _int, _int, _f64p, _f64p]),
    "oracle_mesh_exhaustive_forward": (
        _int, [_f32p, _long, _i64p, _long, _f32p, _long, _f32p, _long, _f32p, _long, _f32p,
               _f32p, _u8p, _u8p, _long, _flt, _flt, _int, _f64p]),
    "oracle_mesh_exhaustive_grad": (
        _int, [_f32p, _long, _i64p, _long, _f32p, _long, _f32p, _long, _f32p, _long, _f32p,
               _f32p, _u8p, _u8p, _long, _flt, _flt, _f64p, _int, _int, _f64p, _f64p]),
    "oracle_volume_confocal_forward": (
        _int, [_f32p, _int, _int, _int, _f32p, _int, _int, _f32p, _f32p, _flt, _flt, _int,
               _f64p]),
    "oracle_volume_confocal_adjoint": (
        _int, [_f64p, _int, _int, _int, _f32p, _int, _int, _f32p, _f32p, _flt, _flt, _int,
               _f64p]),
    "oracle_volume_confocal_transposed": (
        _int, [_f64p, _int, _int, _int, _f32p, _int, _int, _f32p, _f32p, _flt, _flt, _int,
               _f64p]),
    "oracle_volume_confocal_grad_mp": (
        _int, [_f32p, _int, _int, _int, _f32p, _int, _int, _f64p, _f32p, _f32p, _flt, _flt,
               _int, _f64p]),
    "oracle_volume_exhaustive_forward": (
        _int, [_f32p, _int, _int, _int, _f32p, _int, _f32p, _int, _int, _f32p, _f32p, _flt,
               _flt, _int, _f64p]),
    "oracle_volume_exhaustive_adjoint": (
        _int, [_f64p, _int, _int, _int, _f32p, _int, _f32p, _int, _int, _f32p, _f32p, _flt,
               _flt, _f64p]),
    "oracle_bp_confocal_velten": (
        _int, [_f32p, _int, _f32p, _int, _f32p, _int, _int, _int, _int, _f32p, _f32p, _flt,
               _flt, _f64p]),
    "oracle_bp_confocal_velten_adjoint": (
        _int, [_f64p, _int, _int, _int, _f32p, _int, _f32p, _int, _int, _f32p, _f32p, _flt,
               _flt, _f64p]),
    "oracle_bp_exhaustive_velten": (
        _int, [_f32p, _int, _f32p, _int, _f32p, _int, _f32p, _int, _f32p, _int, _int, _int,
               _int, _f32p, _f32p, _flt, _flt, _f64p]),
    "oracle_bp_exhaustive_arellano": (
        _int, [_f32p, _int, _f32p, _int, _f32p, _int, _f32p, _int, _f32p, _int, _int, _int,
               _int, _f32p, _f32p, _flt, _flt, _f64p]),
    "oracle_rbf2volume_forward": (
        _int, [_f32p, _int, _int, _int, _int, _int, _f32p, _f32p, _f64p]),
    "oracle_rbf2volume_grad": (
        _int, [_f32p, _int, _int, _int, _int, _int, _f64p, _f64p, _f32p, _f32p, _f64p]),
}


def lib():
    """Builds (if needed) and loads the oracle shared library."""
    global _lib
    if _lib is None:
        path = _build.build()
        handle = ctypes.CDLL(path)
        for name, (res, args) in _SIGNATURES.items():
            fn = getattr(handle, name, None)
            if fn is None:
                continue
            fn.restype = res
            fn.argtypes = args
        _lib = handle
    return _lib


def _f32(a, shape_tail=None):
    a = np.ascontiguousarray(np.asarray(a, dtype=np.float32))
    if shape_tail is not None and a.shape[1:] != shape_tail:
        raise ValueError("bad shape %s" % (a.shape,))
    return a


def _ptr(a, t):
    if a is None:
        return ctypes.cast(None, t)
    return a.ctypes.data_as(t)


def _faces(faces):
    return np.ascontiguousarray(np.asarray(faces, dtype=np.int64).reshape(-1, 3))


def mesh_count_faces(faces, num_verts):
    faces = _faces(faces)
    return int(lib().oracle_mesh_count_faces(_ptr(faces, _i64p), faces.shape[0], num_verts))


def mesh_visibility(verts, faces, points, bvh=False):
    """uint8 [P, F]: 1 where face f is visible from wall point p (brute force over
    all faces, or through a CPU BVH with identical results when bvh=True)."""
    verts, points, faces = _f32(verts), _f32(points), _faces(faces)
    out = np.zeros((points.shape[0], faces.shape[0]), np.uint8)
    fn = lib().oracle_mesh_visibility_bvh if bvh else lib().oracle_mesh_visibility
    fn(_ptr(verts, _f32p), verts.shape[0], _ptr(faces, _i64p), faces.shape[0],
       _ptr(points, _f32p), points.shape[0], _ptr(out, _u8p))
    return out


def mesh_visibility_pairs(verts, faces, points, pair_p, pair_f):
    verts, points, faces = _f32(verts), _f32(points), _faces(faces)
    pp = np.ascontiguousarray(pair_p, dtype=np.int64)
    pf = np.ascontiguousarray(pair_f, dtype=np.int64)
    out = np.zeros(pp.shape[0], np.uint8)
    lib().oracle_mesh_visibility_pairs(_ptr(verts, _f32p), verts.shape[0], _ptr(faces, _i64p),
                                       faces.shape[0], _ptr(points, _f32p), _ptr(pp, _i64p),
                                       _ptr(pf, _i64p), pp.shape[0], _ptr(out, _u8p))
    return out


def _material(material, nv):
    if material is None:
        return np.zeros((nv, 0), np.float32)
    m = _f32(material)
    return m.reshape(nv, -1)


def mesh_confocal_forward(verts, faces, material, scan_points, scan_origin, vis, nbins,
                          bin_width, bin_offset, fp64=True):
    """float64 [T, S] transient of one mesh (reference layout [B, T, S] per item)."""
    verts, faces, sp = _f32(verts), _faces(faces), _f32(scan_points)
    mat = _material(material, verts.shape[0])
    so = None if scan_origin is None or len(scan_origin) == 0 else _f32(scan_origin)
    vis = np.ascontiguousarray(vis, dtype=np.uint8)
    assert vis.shape == (sp.shape[0], faces.shape[0])
    out = np.zeros((nbins, sp.shape[0]), np.float64)
    lib().oracle_mesh_confocal_forward(
        _ptr(verts, _f32p), verts.shape[0], _ptr(faces, _i64p), faces.shape[0],
        _ptr(mat, _f32p), mat.shape[1], _ptr(sp, _f32p), sp.shape[0], _ptr(so, _f32p),
        _ptr(vis, _u8p), nbins, ctypes.c_float(bin_width), ctypes.c_float(bin_offset),
        int(fp64), _ptr(out, _f64p))
    return out


def mesh_confocal_grad(verts, faces, material, scan_points, scan_origin, vis, nbins,
                       bin_width, bin_offset, transient_grad, want_verts=True, fp64=True):
    """(verts_grad [V, 3] or [V, 0], material_grad [V, M]) in float64."""
    verts, faces, sp = _f32(verts), _faces(faces), _f32(scan_points)
    mat = _material(material, verts.shape[0])
    so = None if scan_origin is None or len(scan_origin) == 0 else _f32(scan_origin)
    vis = np.ascontiguousarray(vis, dtype=np.uint8)
    tg = np.ascontiguousarray(transient_grad, dtype=np.float64)
    assert tg.shape == (nbins, sp.shape[0])
    nv = verts.shape[0]
    vg = np.zeros((nv, 3 if want_verts else 0), np.float64)
    mg = np.zeros((nv, mat.shape[1]), np.float64)
    lib().oracle_mesh_confocal_grad(
        _ptr(verts, _f32p), nv, _ptr(faces, _i64p), faces.shape[0], _ptr(mat, _f32p),
        mat.shape[1], _ptr(sp, _f32p), sp.shape[0], _ptr(so, _f32p), _ptr(vis, _u8p), nbins,
        ctypes.c_float(bin_width), ctypes.c_float(bin_offset), _ptr(tg, _f64p),
        int(want_verts), int(fp64), _ptr(vg, _f64p), _ptr(mg, _f64p))
    return vg, mg


def mesh_exhaustive_forward(verts, faces, material, scan_points, laser_points, scan_origin,
                            laser_origin, vis_s, vis_l, nbins, bin_width, bin_offset,
                            fp64=True):
    """float64 [T, S, L] transient of one mesh."""
    verts, faces = _f32(verts), _faces(faces)
    sp, lp = _f32(scan_points), _f32(laser_points)
    mat = _material(material, verts.shape[0])
    so = None if scan_origin is None or len(scan_origin) == 0 else _f32(scan_origin)
    lo = None if laser_origin is None or len(laser_origin) == 0 else _f32(laser_origin)
    vs = np.ascontiguousarray(vis_s, dtype=np.uint8)
    vl = np.ascontiguousarray(vis_l, dtype=np.uint8)
    out = np.zeros((nbins, sp.shape[0], lp.shape[0]), np.float64)
    lib().oracle_mesh_exhaustive_forward(
        _ptr(verts, _f32p), verts.shape[0], _ptr(faces, _i64p), faces.shape[0],
        _ptr(mat, _f32p), mat.shape[1], _ptr(sp, _f32p), sp.shape[0], _ptr(lp, _f32p),
        lp.shape[0], _ptr(so, _f32p), _ptr(lo, _f32p), _ptr(vs, _u8p), _ptr(vl, _u8p), nbins,
        ctypes.c_float(bin_width), ctypes.c_float(bin_offset), int(fp64), _ptr(out, _f64p))
    return out


def mesh_exhaustive_grad(verts, faces, material, scan_points, laser_points, scan_origin,
                         laser_origin, vis_s, vis_l, nbins, bin_width, bin_offset,
                         transient_grad, want_verts=True, fp64=True):
    verts, faces = _f32(verts), _faces(faces)
    sp, lp = _f32(scan_points), _f32(laser_points)
    mat = _material(material, verts.shape[0])
    so = None if scan_origin is None or len(scan_origin) == 0 else _f32(scan_origin)
    lo = None if laser_origin is None or len(laser_origin) == 0 else _f32(laser_origin)
    vs = np.ascontiguousarray(vis_s, dtype=np.uint8)
    vl = np.ascontiguousarray(vis_l, dtype=np.uint8)
    tg = np.ascontiguousarray(transient_grad, dtype=np.float64)
    nv = verts.shape[0]
    vg = np.zeros((nv, 3 if want_verts else 0), np.float64)
    mg = np.zeros((nv, mat.shape[1]), np.float64)
    lib().oracle_mesh_exhaustive_grad(
        _ptr(verts, _f32p), nv, _ptr(faces, _i64p), faces.shape[0], _ptr(mat, _f32p),
        mat.shape[1], _ptr(sp, _f32p), sp.shape[0], _ptr(lp, _f32p), lp.shape[0],
        _ptr(so, _f32p), _ptr(lo, _f32p), _ptr(vs, _u8p), _ptr(vl, _u8p), nbins,
        ctypes.c_float(bin_width), ctypes.c_float(bin_offset), _ptr(tg, _f64p),
        int(want_verts), int(fp64), _ptr(vg, _f64p), _ptr(mg, _f64p))
    return vg, mg


# ---------------------------------------------------------------------------
# Volume renderer (one item; layouts as the reference's operators).

def _v3(v):
    return np.ascontiguousarray(np.asarray(v, dtype=np.float32).reshape(3))


def _f64(a):
    return np.ascontiguousarray(np.asarray(a, dtype=np.float64))


def volume_confocal_forward(volume, mp, nbins, origin, size, bin_width, bin_offset, fp64=True):
    """transient [N, T] of volume [X, Y, Z] seen from measurement points [3, N]."""
    v, m = _f32(volume), _f32(mp)
    o, s = _v3(origin), _v3(size)
    out = np.zeros((m.shape[1], nbins), np.float64)
    lib().oracle_volume_confocal_forward(_ptr(v, _f32p), *v.shape, _ptr(m, _f32p), m.shape[1],
                                         nbins, _ptr(o, _f32p), _ptr(s, _f32p), bin_width,
                                         bin_offset, int(fp64), _ptr(out, _f64p))
    return out


def volume_confocal_adjoint(transient, shape, mp, origin, size, bin_width, bin_offset,
                            fp64=True):
    """Exact adjoint of volume_confocal_forward: volume [X, Y, Z] from transient [N, T]."""
    t, m = _f64(transient), _f32(mp)
    o, s = _v3(origin), _v3(size)
    out = np.zeros(tuple(shape), np.float64)
    lib().oracle_volume_confocal_adjoint(_ptr(t, _f64p), *shape, _ptr(m, _f32p), m.shape[1],
                                         t.shape[1], _ptr(o, _f32p), _ptr(s, _f32p), bin_width,
                                         bin_offset, int(fp64), _ptr(out, _f64p))
    return out


def volume_confocal_transposed(transient, shape, mp, origin, size, bin_width, bin_offset,
                               fp64=True):
    """The reference's transposed operator (volume_confocal_grad_volume)."""
    t, m = _f64(transient), _f32(mp)
    o, s = _v3(origin), _v3(size)
    out = np.zeros(tuple(shape), np.float64)
    lib().oracle_volume_confocal_transposed(_ptr(t, _f64p), *shape, _ptr(m, _f32p), m.shape[1],
                                            t.shape[1], _ptr(o, _f32p), _ptr(s, _f32p),
                                            bin_width, bin_offset, int(fp64), _ptr(out, _f64p))
    return out


def volume_confocal_grad_mp(volume, mp, transient_grad, origin, size, bin_width, bin_offset,
                            fp64=True):
    """d loss / d measurement points [3, N]."""
    v, m, g = _f32(volume), _f32(mp), _f64(transient_grad)
    o, s = _v3(origin), _v3(size)
    out = np.zeros((3, m.shape[1]), np.float64)
    lib().oracle_volume_confocal_grad_mp(_ptr(v, _f32p), *v.shape, _ptr(m, _f32p), m.shape[1],
                                         g.shape[1], _ptr(g, _f64p), _ptr(o, _f32p),
                                         _ptr(s, _f32p), bin_width, bin_offset, int(fp64),
                                         _ptr(out, _f64p))
    return out


def volume_exhaustive_forward(volume, scan_points, laser_points, nbins, start, end, bin_width,
                              bin_offset):
    """transient [T, S, L] of volume [D, H, W]; points [3, S] / [3, L]."""
    v, sp, lp = _f32(volume), _f32(scan_points), _f32(laser_points)
    a, e = _v3(start), _v3(end)
    out = np.zeros((nbins, sp.shape[1], lp.shape[1]), np.float64)
    lib().oracle_volume_exhaustive_forward(_ptr(v, _f32p), *v.shape, _ptr(sp, _f32p),
                                           sp.shape[1], _ptr(lp, _f32p), lp.shape[1], nbins,
                                           _ptr(a, _f32p), _ptr(e, _f32p), bin_width, bin_offset,
                                           1, _ptr(out, _f64p))
    return out


def volume_exhaustive_adjoint(transient_grad, shape, scan_points, laser_points, start, end,
                              bin_width, bin_offset):
    g, sp, lp = _f64(transient_grad), _f32(scan_points), _f32(laser_points)
    a, e = _v3(start), _v3(end)
    out = np.zeros(tuple(shape), np.float64)
    lib().oracle_volume_exhaustive_adjoint(_ptr(g, _f64p), *shape, _ptr(sp, _f32p), sp.shape[1],
                                           _ptr(lp, _f32p), lp.shape[1], g.shape[0],
                                           _ptr(a, _f32p), _ptr(e, _f32p), bin_width, bin_offset,
                                           _ptr(out, _f64p))
    return out


# ---------------------------------------------------------------------------
# Backprojection (one item).

def _origin(o, n):
    if o is None:
        return np.zeros((0, 3), np.float32), 0
    o = _f32(o)
    return o, o.shape[0] if o.ndim == 2 and o.shape[1] == 3 else o.shape[-1]


def bp_confocal_velten(transient, scan_points, scan_origin, shape, start, end, bin_width,
                       bin_offset):
    """volume [D, H, W] from transient [T, S]; scan_points / scan_origin [S, 3]."""
    t, sp = _f32(transient), _f32(scan_points)
    so = _f32(scan_origin) if scan_origin is not None else np.zeros((0, 3), np.float32)
    a, e = _v3(start), _v3(end)
    out = np.zeros(tuple(shape), np.float64)
    lib().oracle_bp_confocal_velten(_ptr(t, _f32p), t.shape[0], _ptr(sp, _f32p), sp.shape[0],
                                    _ptr(so, _f32p), so.shape[0], *shape, _ptr(a, _f32p),
                                    _ptr(e, _f32p), bin_width, bin_offset, _ptr(out, _f64p))
    return out


def bp_confocal_velten_adjoint(volume, scan_points, scan_origin, nbins, start, end, bin_width,
                               bin_offset):
    v, sp = _f64(volume), _f32(scan_points)
    so = _f32(scan_origin) if scan_origin is not None else np.zeros((0, 3), np.float32)
    a, e = _v3(start), _v3(end)
    out = np.zeros((nbins, sp.shape[0]), np.float64)
    lib().oracle_bp_confocal_velten_adjoint(_ptr(v, _f64p), *v.shape, _ptr(sp, _f32p),
                                            sp.shape[0], _ptr(so, _f32p), so.shape[0], nbins,
                                            _ptr(a, _f32p), _ptr(e, _f32p), bin_width,
                                            bin_offset, _ptr(out, _f64p))
    return out


def bp_exhaustive_velten(transient, scan_points, laser_points, scan_origin, laser_origin, shape,
                         start, end, bin_width, bin_offset):
    """volume [D, H, W] from transient [T, S, L]; points [S, 3] / [L, 3]."""
    t, sp, lp = _f32(transient), _f32(scan_points), _f32(laser_points)
    so = _f32(scan_origin) if scan_origin is not None else np.zeros((0, 3), np.float32)
    lo = _f32(laser_origin) if laser_origin is not None else np.zeros((0, 3), np.float32)
    a, e = _v3(start), _v3(end)
    out = np.zeros(tuple(shape), np.float64)
    lib().oracle_bp_exhaustive_velten(_ptr(t, _f32p), t.shape[0], _ptr(sp, _f32p), sp.shape[0],
                                      _ptr(lp, _f32p), lp.shape[0], _ptr(so, _f32p),
                                      so.shape[0], _ptr(lo, _f32p), lo.shape[0], *shape,
                                      _ptr(a, _f32p), _ptr(e, _f32p), bin_width, bin_offset,
                                      _ptr(out, _f64p))
    return out


def bp_exhaustive_arellano(transient, scan_points, laser_points, scan_origin, laser_origin,
                           shape, start, end, bin_width, bin_offset):
    """volume [D, H, W] from transient [T, S, L]; points [3, S] / [3, L] (origins [3, n])."""
    t, sp, lp = _f32(transient), _f32(scan_points), _f32(laser_points)
    so = _f32(scan_origin) if scan_origin is not None else np.zeros((3, 0), np.float32)
    lo = _f32(laser_origin) if laser_origin is not None else np.zeros((3, 0), np.float32)
    a, e = _v3(start), _v3(end)
    out = np.zeros(tuple(shape), np.float64)
    lib().oracle_bp_exhaustive_arellano(_ptr(t, _f32p), t.shape[0], _ptr(sp, _f32p), sp.shape[1],
                                        _ptr(lp, _f32p), lp.shape[1], _ptr(so, _f32p),
                                        so.shape[1], _ptr(lo, _f32p), lo.shape[1], *shape,
                                        _ptr(a, _f32p), _ptr(e, _f32p), bin_width, bin_offset,
                                        _ptr(out, _f64p))
    return out


# ---------------------------------------------------------------------------
# RBF to volume (one item).

def rbf2volume_forward(rbf, shape, start, end):
    """volume [1+A, D, H, W] from rbf [N, 4+A]."""
    r = _f32(rbf)
    a, e = _v3(start), _v3(end)
    out = np.zeros((r.shape[1] - 3,) + tuple(shape), np.float64)
    lib().oracle_rbf2volume_forward(_ptr(r, _f32p), r.shape[0], r.shape[1], *shape,
                                    _ptr(a, _f32p), _ptr(e, _f32p), _ptr(out, _f64p))
    return out


def rbf2volume_grad(rbf, volume, volume_grad, start, end):
    """rbf_grad [N, 4+A]."""
    r, v, g = _f32(rbf), _f64(volume), _f64(volume_grad)
    a, e = _v3(start), _v3(end)
    out = np.zeros(r.shape, np.float64)
    lib().oracle_rbf2volume_grad(_ptr(r, _f32p), r.shape[0], r.shape[1], *v.shape[1:],
                                 _ptr(v, _f64p), _ptr(g, _f64p), _ptr(a, _f32p), _ptr(e, _f32p),
                                 _ptr(out, _f64p))
    return out


# ---------------------------------------------------------------------------
# Marching cubes (numpy restatement with its own case-table derivation).

from .isosurface import case_table as marching_cubes_table  # noqa: E402
from .isosurface import marching_cubes, marching_cubes_grad  # noqa: E402,F401


# ---------------------------------------------------------------------------
# f-k migration (numpy restatement).

from .fk import fk_migration, stolt  # noqa: E402,F401


# ---------------------------------------------------------------------------
# Orthographic depth rasteriser (numpy restatement).

from .raster import depth_raster  # noqa: E402,F401


# ---------------------------------------------------------------------------
# Shaded perspective preview rasteriser (numpy restatement).

from .shading import shaded_raster  # noqa: E402,F401
