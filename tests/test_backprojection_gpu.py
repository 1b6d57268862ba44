"""Backprojection on the GPU against the FP64 oracle and the reference's golden
vectors; the Velten adjoint against <B x, y> = <x, B^T y>.

Tolerances (rel-L2): 1e-5 vs the FP64 oracle, 1e-4 vs the reference's FP32
outputs (nearest-bin decisions are shared, so these are summation-order
differences only).
"""
import os

import numpy as np
import pytest
import torch

import oracle
from totri_gb300 import scenes
from totri_gb300.reconstruct import (BackprojectionConfocalVelten,
                                     BackprojectionExhaustiveArellano,
                                     BackprojectionExhaustiveVelten)
from totri_gb300.totri_cpp import reconstruct as K
from totri_gb300.types import BinDef, VolumeDef

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def cu(a):
    return torch.as_tensor(np.ascontiguousarray(a)).cuda()


def test_golden_vectors(cuda_lib):
    g = dict(np.load(os.path.join(GOLDEN, "backprojection.npz")))
    shape = tuple(int(x) for x in g["shape"])
    vd = VolumeDef(tuple(g["start"].tolist()), tuple(g["end"].tolist()), shape)
    v = BackprojectionConfocalVelten.apply(cu(g["transient_confocal"]), cu(g["scan_points"]), vd,
                                           BinDef(0.02, 0.0), cu(g["scan_origin"]))
    assert rel(v.cpu().numpy(), g["volume_confocal"]) < 1e-4
    v = BackprojectionExhaustiveVelten.apply(cu(g["transient_exhaustive"]), cu(g["scan_points"]),
                                             cu(g["laser_points"]), vd, BinDef(0.01, 0.0))
    assert rel(v.cpu().numpy(), g["volume_exhaustive"]) < 1e-4
    v = BackprojectionExhaustiveArellano.apply(
        cu(g["transient_exhaustive"]), cu(g["scan_points"].transpose(0, 2, 1)),
        cu(g["laser_points"].transpose(0, 2, 1)), vd, BinDef(0.01, 0.0))
    assert rel(v.cpu().numpy(), g["volume_arellano"]) < 1e-4


def test_against_oracle_with_origins(cuda_lib):
    rng = np.random.default_rng(7)
    S, L, T, shape = 40, 5, 100, (7, 8, 9)
    st, en = (-0.5, -0.5, 0.5), (0.5, 0.5, 1.5)
    sp = np.stack([rng.uniform(-1, 1, S), rng.uniform(-1, 1, S), np.zeros(S)], 1).astype(np.float32)
    lp = np.stack([rng.uniform(-1, 1, L), rng.uniform(-1, 1, L), np.zeros(L)], 1).astype(np.float32)
    so = np.tile(np.array([[0.1, 0.2, -1.5]], np.float32), (S, 1))
    lo = np.tile(np.array([[-0.3, 0.0, -1.0]], np.float32), (L, 1))
    trc = rng.random((1, T, S)).astype(np.float32)
    tre = rng.random((1, T, S, L)).astype(np.float32)
    vd = VolumeDef(st, en, shape)
    v = BackprojectionConfocalVelten.apply(cu(trc), cu(sp[None]), vd, BinDef(0.02, 0.05),
                                           cu(so[None]))
    ref = oracle.bp_confocal_velten(trc[0], sp, so, shape, st, en, 0.02, 0.05)
    assert rel(v[0].cpu().numpy(), ref) < 1e-5
    v = BackprojectionExhaustiveVelten.apply(cu(tre), cu(sp[None]), cu(lp[None]), vd,
                                             BinDef(0.01, 0.0), cu(so[None]), cu(lo[None]))
    ref = oracle.bp_exhaustive_velten(tre[0], sp, lp, so, lo, shape, st, en, 0.01, 0.0)
    assert rel(v[0].cpu().numpy(), ref) < 1e-5
    v = BackprojectionExhaustiveArellano.apply(cu(tre), cu(sp.T[None]), cu(lp.T[None]), vd,
                                               BinDef(0.01, 0.0), cu(so.T[None]), cu(lo.T[None]))
    ref = oracle.bp_exhaustive_arellano(tre[0], sp.T, lp.T, so.T, lo.T, shape, st, en, 0.01, 0.0)
    assert rel(v[0].cpu().numpy(), ref) < 1e-5


def test_velten_adjoint_full_size(cuda_lib):
    """128^3 voxels x 128x128 scan points x 1024 bins: <B x, y> = <x, B^T y>, and
    the forward against the oracle on a 64-point subset of the scan."""
    s = scenes.volume_scene()
    vd, bd = s["volume_def"], s["bin_def"]
    sp = s["scan_points"].cuda()
    S = sp.shape[1]
    gen = torch.Generator(device="cuda").manual_seed(11)
    x = torch.rand((1, bd.num, S), device="cuda", generator=gen)
    bx = BackprojectionConfocalVelten.apply(x, sp, vd, bd)
    # non-negative y: the identity is tested without cancellation in the sums,
    # so FP32 accumulation error stays relative to |<Bx, y>|
    y = torch.rand(bx.shape, device="cuda", generator=gen)
    bty = torch.empty_like(x)
    K.backprojection_confocal_velten_adjoint(y, sp, torch.empty_like(sp[:, :0]), bty, vd.start,
                                             vd.end, bd.width, bd.offset)
    lhs = float((bx.double() * y.double()).sum())
    rhs = float((x.double() * bty.double()).sum())
    assert abs(lhs - rhs) <= 1e-5 * abs(lhs)
    sub = np.linspace(0, S - 1, 64).astype(np.int64)
    xs = x[:, :, sub].contiguous()
    v = BackprojectionConfocalVelten.apply(xs, sp[:, sub].contiguous(), vd, bd)
    ref = oracle.bp_confocal_velten(xs[0].cpu().numpy(), sp[0, sub].cpu().numpy(), None,
                                    vd.resolution, vd.start, vd.end, bd.width, bd.offset)
    assert rel(v[0].cpu().numpy(), ref) < 1e-5


@pytest.mark.parametrize("offset,origin", [(0.0, False), (0.137, True)])
def test_velten_bins_exact(cuda_lib, offset, origin):
    """Bin decisions bit for bit: with transient[t, s] = t + 1 every voxel sums
    its scan points' bins as integers (exact in FP32 below 2^24), so one bin
    taken differently from the oracle changes a voxel by exactly 1. Covers the
    filtered fast path and its exact fallback, forward and adjoint."""
    g = np.random.default_rng(21)
    T, res = 700, (40, 36, 44)
    sp = scenes.wall_grid(24)[0].numpy()
    S = sp.shape[0]
    tr = np.broadcast_to((np.arange(T, dtype=np.float32) + 1)[:, None], (T, S)).copy()
    so = (sp + g.uniform(-0.3, 0.3, sp.shape).astype(np.float32)) if origin else None
    st, en, bw = (-0.5, -0.4, 0.6), (0.45, 0.5, 1.4), 0.0043
    ref = oracle.bp_confocal_velten(tr, sp, so, res, st, en, bw, offset)
    vol = torch.empty((1,) + res, device="cuda")
    so_t = torch.from_numpy(so)[None].cuda() if origin else torch.empty((1, 0, 3), device="cuda")
    K.backprojection_confocal_velten_forward(torch.from_numpy(tr)[None].cuda(),
                                             torch.from_numpy(sp)[None].cuda(), so_t, vol, st,
                                             en, bw, offset)
    assert np.array_equal(vol[0].double().cpu().numpy(), ref)
    from totri_gb300 import autotune
    for grp in (1, 2):  # one bin window per tile, group windows
        autotune.set_tile("backprojection.velten.groups", grp)
        v2 = torch.empty_like(vol)
        K.backprojection_confocal_velten_forward(torch.from_numpy(tr)[None].cuda(),
                                                 torch.from_numpy(sp)[None].cuda(), so_t, v2, st,
                                                 en, bw, offset)
        autotune.set_tile("backprojection.velten.groups", 0)
        assert np.array_equal(v2[0].double().cpu().numpy(), ref)
    # adjoint: a one-voxel volume of value 1 gives 1 exactly at its bin for every scan point
    one = np.zeros(res, np.float64)
    one[17, 5, 30] = 1.0
    adj_ref = oracle.bp_confocal_velten_adjoint(one, sp, so, T, st, en, bw, offset)
    adj = torch.empty((1, T, S), device="cuda")
    K.backprojection_confocal_velten_adjoint(torch.from_numpy(one.astype(np.float32))[None].cuda(),
                                             torch.from_numpy(sp)[None].cuda(), so_t, adj, st, en,
                                             bw, offset)
    assert np.array_equal(adj[0].double().cpu().numpy(), adj_ref)


def test_velten_tiled_equals_untiled(cuda_lib):
    """The shared-memory tiled Velten kernel sums the same values in the same
    order as the one-voxel-per-thread kernel: identical volumes for 1, 2 and
    4 voxels per thread, bins of two voxels at a time from paired FP32
    instructions (the default) or one at a time ("backprojection.velten.pair"
    = 2), with registers capped for 6 or 5 CTAs per SM or not
    ("backprojection.velten.occupancy" = 5, 1), and with one bin window per tile
    or group windows ("backprojection.velten.groups" = 1, 2), including grids
    that are not a multiple of the voxel block. The scans cover every staging
    of a tile's bin rows (by a CPU model of the kernel's choice, for 4 voxels
    per thread): with group windows, random points give per-point windows, the
    64x64 wall grid with 2,048 bins into 96^3 voxels gives windows per 8 and
    per 4 points, and 4,096 bins into 64^3 voxels gives per-point windows cut
    at their first rows, the rest read from global memory; with one window
    per tile, the fine-bin scans overflow it and read from global memory."""
    from totri_gb300 import autotune
    g = np.random.default_rng(5)
    grid = scenes.wall_grid(64)[0].numpy()
    for res, S, T, bw in (((37, 29, 50), 300, 900, 0.004), ((16, 16, 16), 1000, 256, 0.05),
                          ((21, 9, 11), 77, 400, 0.01), ((96, 96, 96), None, 2048, 0.0025),
                          ((64, 64, 64), None, 4096, 0.00125)):
        pts = grid if S is None else np.stack([g.uniform(-1, 1, S), g.uniform(-1, 1, S),
                                               np.zeros(S)], -1)
        S = pts.shape[0]
        tr = torch.from_numpy(g.random((1, T, S), dtype=np.float32)).cuda()
        sp = torch.from_numpy(pts.astype(np.float32))[None].cuda()
        out = []
        keys = ("mode", "vz", "occupancy", "groups", "pair")
        variants = [(1, 0, 0, 0, 0)] + [
            (0, vz, occ, grp, pair)
            for vz, occ, pair in ((1, 0, 0), (2, 0, 0), (2, 0, 2), (4, 0, 0), (4, 0, 2),
                                  (4, 5, 0), (4, 1, 2))
            for grp in (1, 2)]
        try:
            for values in variants:
                for key, value in zip(keys, values):
                    autotune.set_tile("backprojection.velten." + key, value)
                v = torch.empty((1,) + res, device="cuda")
                K.backprojection_confocal_velten_forward(
                    tr, sp, torch.empty((1, 0, 3), device="cuda"), v, (-0.5, -0.4, 0.5),
                    (0.5, 0.45, 1.5), bw, 0.01)
                out.append(v)
        finally:
            for key in keys:
                autotune.set_tile("backprojection.velten." + key, 0)
        for o in out[1:]:
            assert torch.equal(out[0], o)
