"""Non-finite inputs (NaN and Inf) through every C-ABI operator: each call
returns, leaves the device usable, and gives the output the FP64 oracle gives
for the same inputs (the same IEEE decisions: a NaN or infinite vertex makes
its faces hit nothing, a NaN point takes no samples, a NaN value propagates to
the outputs it is summed into), never a hang or a fault.

Comparison: the positions of NaN outputs must be the same; the finite outputs
within the operator's usual rel-L2 bound (1e-5; 1e-4 for gradients).
"""
import numpy as np
import pytest
import torch

import oracle
from totri_gb300 import scenes
from totri_gb300.render import MeshRenderExhaustive
from totri_gb300.totri_cpp import reconstruct as K
from totri_gb300.totri_cpp import render as R
from totri_gb300.totri_cpp import util as U

from mesh_util import np_scene, rel_l2, unpack_mask

pytestmark = pytest.mark.gpu


def cu(a):
    return torch.as_tensor(np.ascontiguousarray(a)).cuda()


def same(got, ref, tol=1e-5):
    got = np.asarray(got, np.float64)
    ref = np.asarray(ref, np.float64)
    assert np.array_equal(np.isnan(got), np.isnan(ref))
    assert np.array_equal(np.isinf(got), np.isinf(ref))
    fin = np.isfinite(ref)
    assert rel_l2(got[fin], ref[fin]) < tol


def _bad_mesh(seed):
    s = scenes.confocal_small(seed=seed)
    v = s["verts"].clone()
    v[0, 7, 1] = float("nan")
    v[0, 40, 2] = float("inf")
    v[0, 41, 0] = -float("inf")
    return s, v


def test_mesh_confocal_with_nan_and_inf_vertices(cuda_lib):
    s, v = _bad_mesh(3)
    n = np_scene(s)
    n["verts"] = v[0].numpy()
    bd = s["bin_def"]
    F = n["faces"].shape[0]
    d_v, d_f, d_c, d_p = v.cuda(), s["faces"].cuda(), s["colors"].cuda(), s["scan_points"].cuda()
    vis = oracle.mesh_visibility(n["verts"], n["faces"], n["scan_points"])
    got = unpack_mask(R.mesh_visibility(d_v, d_f, d_p)[0].cpu().numpy(), F)
    assert np.array_equal(got, vis)
    assert not vis[:, (n["faces"] == 7).any(1)].any()  # a NaN vertex's faces hit nothing
    empty = torch.empty_like(d_p[:, :0])
    out = torch.full((1, bd.num, d_p.shape[1]), 5.0, device="cuda")
    R.mesh_confocal_forward(d_v, d_f, d_c, d_p, empty, out, bd.width, bd.offset, 0)
    ref = oracle.mesh_confocal_forward(n["verts"], n["faces"], n["colors"], n["scan_points"],
                                       None, vis, bd.num, bd.width, bd.offset)
    same(out[0].cpu().numpy(), ref)
    tg = np.random.default_rng(0).standard_normal(ref.shape).astype(np.float32)
    vg, mg = torch.empty_like(d_v), torch.empty_like(d_c)
    R.mesh_confocal_grad_verts(d_v, d_f, d_c, d_p, empty, cu(tg[None]), vg, mg, bd.width,
                               bd.offset, 0)
    rv, rm = oracle.mesh_confocal_grad(n["verts"], n["faces"], n["colors"], n["scan_points"],
                                       None, vis, bd.num, bd.width, bd.offset, tg)
    same(vg[0].cpu().numpy(), rv, 1e-4)
    same(mg[0].cpu().numpy(), rm, 1e-4)


def test_mesh_confocal_with_nonfinite_points_and_bins(cuda_lib):
    s = scenes.confocal_small(seed=4)
    n = np_scene(s)
    bd = s["bin_def"]
    p = s["scan_points"].clone()
    p[0, 3] = float("nan")
    p[0, 9, 0] = float("inf")
    n["scan_points"] = p[0].numpy()
    d_v, d_f, d_c, d_p = s["verts"].cuda(), s["faces"].cuda(), s["colors"].cuda(), p.cuda()
    F = n["faces"].shape[0]
    vis = oracle.mesh_visibility(n["verts"], n["faces"], n["scan_points"])
    assert np.array_equal(unpack_mask(R.mesh_visibility(d_v, d_f, d_p)[0].cpu().numpy(), F), vis)
    empty = torch.empty_like(d_p[:, :0])
    for bw in (bd.width, float("nan"), 0.0):
        out = torch.full((1, bd.num, d_p.shape[1]), 5.0, device="cuda")
        R.mesh_confocal_forward(d_v, d_f, d_c, d_p, empty, out, bw, bd.offset, 0)
        ref = oracle.mesh_confocal_forward(n["verts"], n["faces"], n["colors"], n["scan_points"],
                                           None, vis, bd.num, bw, bd.offset)
        same(out[0].cpu().numpy(), ref)


def test_mesh_exhaustive_with_nonfinite_inputs(cuda_lib):
    s, v = _bad_mesh(5)
    n = np_scene(s)
    n["verts"] = v[0].numpy()
    sp = scenes.wall_grid(5)
    lp = scenes.wall_grid(3) * 0.8
    sp[0, 2] = float("nan")
    lp[0, 4, 1] = float("inf")
    spn, lpn = sp[0].numpy(), lp[0].numpy()
    from totri_gb300.types import BinDef
    bd = BinDef(0.02, 0.0, 300)
    verts = v.cuda().requires_grad_(True)
    colors = s["colors"].cuda().requires_grad_(True)
    tr = MeshRenderExhaustive.apply(verts, s["faces"].cuda(), sp.cuda(), lp.cuda(), bd, colors)
    vs = oracle.mesh_visibility(n["verts"], n["faces"], spn)
    vl = oracle.mesh_visibility(n["verts"], n["faces"], lpn)
    ref = oracle.mesh_exhaustive_forward(n["verts"], n["faces"], n["colors"], spn, lpn, None,
                                         None, vs, vl, bd.num, bd.width, bd.offset)
    same(tr[0].detach().cpu().numpy(), ref)
    w = torch.randn_like(tr)
    (tr * w).sum().backward()
    rv, rm = oracle.mesh_exhaustive_grad(n["verts"], n["faces"], n["colors"], spn, lpn, None,
                                         None, vs, vl, bd.num, bd.width, bd.offset,
                                         w[0].cpu().numpy())
    same(verts.grad[0].cpu().numpy(), rv, 1e-4)
    same(colors.grad[0].cpu().numpy(), rm, 1e-4)


def test_volume_and_backprojection_with_nonfinite_inputs(cuda_lib):
    g = np.random.default_rng(8)
    X, N, T = 10, 30, 80
    vol = ((g.random((X, X, X)) < 0.15) * g.random((X, X, X))).astype(np.float32)
    vol[3, 4, 5] = np.nan
    vol[6, 1, 2] = np.inf
    mp = np.stack([g.uniform(-1, 1, N), g.uniform(-1, 1, N), np.zeros(N)]).astype(np.float32)
    mp[:, 4] = np.nan
    org, size, bw, bo = (-0.5, -0.5, 0.5), (1.0, 1.0, 1.0), 0.03, 0.0
    out = torch.full((N, T), 3.0, device="cuda")
    R.volume_confocal_forward(cu(vol), cu(mp), out, org, size, bw, bo)
    same(out.cpu().numpy(), oracle.volume_confocal_forward(vol, mp, T, org, size, bw, bo))
    y = g.standard_normal((N, T)).astype(np.float32)
    y[7, 20] = np.nan
    adj = torch.empty(vol.shape, device="cuda")
    R.volume_confocal_adjoint(adj, cu(mp), cu(y), org, size, bw, bo)
    same(adj.cpu().numpy(), oracle.volume_confocal_adjoint(y, vol.shape, mp, org, size, bw, bo))
    tr = torch.empty(vol.shape, device="cuda")
    R.volume_confocal_grad_volume(tr, cu(mp), cu(y), org, size, bw, bo)
    same(tr.cpu().numpy(), oracle.volume_confocal_transposed(y, vol.shape, mp, org, size, bw, bo))

    S, shape = 25, (6, 7, 8)
    st, en = (-0.5, -0.5, 0.5), (0.5, 0.5, 1.5)
    sp = np.stack([g.uniform(-1, 1, S), g.uniform(-1, 1, S), np.zeros(S)], 1).astype(np.float32)
    sp[6] = np.nan
    trc = g.random((T, S)).astype(np.float32)
    trc[10, 3] = np.inf
    v = torch.empty((1,) + shape, device="cuda")
    K.backprojection_confocal_velten_forward(cu(trc[None]), cu(sp[None]),
                                             torch.empty((1, 0, 3), device="cuda"), v, st, en,
                                             0.02, 0.0)
    same(v[0].cpu().numpy(), oracle.bp_confocal_velten(trc, sp, None, shape, st, en, 0.02, 0.0))


def test_rbf_with_nonfinite_gaussians(cuda_lib):
    g = np.random.default_rng(9)
    N = 60
    rbf = np.concatenate([g.uniform(-0.5, 0.5, (N, 3)) + np.array([0, 0, 1.0]),
                          g.uniform(0.02, 0.08, (N, 1)), g.random((N, 1))], 1).astype(np.float32)
    rbf[3, 0] = np.nan
    rbf[8, 3] = np.inf
    rbf[12, 4] = np.inf
    shape, start, end = (9, 8, 7), (-0.5, -0.5, 0.5), (0.5, 0.5, 1.5)
    vol = torch.empty((1, 2) + shape, device="cuda")
    U.rbf2volume_gaussian_forward(cu(rbf[None]), vol, start, end)
    ref = oracle.rbf2volume_forward(rbf, shape, start, end)
    same(vol[0].cpu().numpy(), ref)


def test_device_still_answers(cuda_lib):
    """After all of the above, a plain render still matches the oracle."""
    s = scenes.confocal_small(seed=6)
    n = np_scene(s)
    bd = s["bin_def"]
    vis = oracle.mesh_visibility(n["verts"], n["faces"], n["scan_points"])
    out = torch.empty((1, bd.num, n["scan_points"].shape[0]), device="cuda")
    R.mesh_confocal_forward(s["verts"].cuda(), s["faces"].cuda(), s["colors"].cuda(),
                            s["scan_points"].cuda(), torch.empty((1, 0, 3), device="cuda"), out,
                            bd.width, bd.offset, 0)
    ref = oracle.mesh_confocal_forward(n["verts"], n["faces"], n["colors"], n["scan_points"],
                                       None, vis, bd.num, bd.width, bd.offset)
    assert rel_l2(out[0].cpu().numpy(), ref) < 1e-5


def test_volume_with_degenerate_bin_width(cuda_lib):
    """A zero or NaN bin width: every bin is walked (zero: all bins share one
    centre, the offset), matching the oracle; no hang, no fault."""
    g = np.random.default_rng(10)
    X, N, T = 8, 20, 40
    vol = ((g.random((X, X, X)) < 0.2) * g.random((X, X, X))).astype(np.float32)
    mp = np.stack([g.uniform(-1, 1, N), g.uniform(-1, 1, N), np.zeros(N)]).astype(np.float32)
    org, size = (-0.5, -0.5, 0.5), (1.0, 1.0, 1.0)
    y = g.standard_normal((N, T)).astype(np.float32)
    for bw, bo in ((0.0, 1.1), (float("nan"), 0.0), (float("inf"), 0.0), (0.03, float("nan"))):
        out = torch.full((N, T), 3.0, device="cuda")
        R.volume_confocal_forward(cu(vol), cu(mp), out, org, size, bw, bo)
        same(out.cpu().numpy(), oracle.volume_confocal_forward(vol, mp, T, org, size, bw, bo))
        adj = torch.full(vol.shape, 3.0, device="cuda")
        R.volume_confocal_adjoint(adj, cu(mp), cu(y), org, size, bw, bo)
        same(adj.cpu().numpy(),
             oracle.volume_confocal_adjoint(y, vol.shape, mp, org, size, bw, bo))
