"""Exhaustive (laser + detector) mesh path on the GPU against the CPU oracle and
the reference's golden vectors.

Tolerances (rel-L2): transients and gradients 1e-5 vs the FP64 oracle (masks
exact); 1e-4 / 1e-3 vs the reference's FP32 forward / gradient (its own FP32
bin coordinates move its gradient by up to ~1e-4 from the FP64 value).
"""
import os

import numpy as np
import pytest
import torch

import oracle
from totri_gb300 import scenes
from totri_gb300.render import MeshRenderExhaustive
from totri_gb300.totri_cpp import render as R
from totri_gb300.types import BinDef

from mesh_util import np_scene, rel_l2, unpack_mask

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def case(seed=0, s_res=6, l_res=3, nb=300, bw=0.02):
    s = scenes.confocal_small(seed=seed)
    sp = scenes.wall_grid(s_res)
    lp = scenes.wall_grid(l_res) * 0.8
    return s, sp, lp, BinDef(bw, 0.0, nb)


def test_forward_and_grad_match_oracle(cuda_lib):
    s, sp, lp, bd = case()
    n = np_scene(s)
    spn, lpn = sp[0].numpy(), lp[0].numpy()
    verts = s["verts"].cuda().requires_grad_(True)
    colors = s["colors"].cuda().requires_grad_(True)
    tr = MeshRenderExhaustive.apply(verts, s["faces"].cuda(), sp.cuda(), lp.cuda(), bd, colors)
    vs = oracle.mesh_visibility(n["verts"], n["faces"], spn)
    vl = oracle.mesh_visibility(n["verts"], n["faces"], lpn)
    ref = oracle.mesh_exhaustive_forward(n["verts"], n["faces"], n["colors"], spn, lpn, None,
                                         None, vs, vl, bd.num, bd.width, bd.offset)
    assert rel_l2(tr[0].detach().cpu().numpy(), ref) < 1e-5
    w = torch.randn_like(tr)
    (tr * w).sum().backward()
    rv, rm = oracle.mesh_exhaustive_grad(n["verts"], n["faces"], n["colors"], spn, lpn, None,
                                         None, vs, vl, bd.num, bd.width, bd.offset,
                                         w[0].cpu().numpy())
    assert rel_l2(verts.grad[0].cpu().numpy(), rv) < 1e-5
    assert rel_l2(colors.grad[0].cpu().numpy(), rm) < 1e-5


def test_masks_are_the_confocal_masks(cuda_lib):
    s, sp, lp, bd = case(seed=3)
    n = np_scene(s)
    F = n["faces"].shape[0]
    pts = torch.cat([sp, lp], dim=1).cuda()
    m = unpack_mask(R.mesh_visibility(s["verts"].cuda(), s["faces"].cuda(), pts)[0].cpu().numpy(),
                    F)
    assert np.array_equal(m, oracle.mesh_visibility(n["verts"], n["faces"], pts[0].cpu().numpy()))


def test_with_origins_matches_oracle(cuda_lib):
    s, sp, lp, bd = case(seed=5, nb=600)
    n = np_scene(s)
    so = torch.tensor([[0.2, 0.1, -1.0]]).expand(1, sp.shape[1], 3)
    lo = torch.tensor([[-0.4, 0.3, -2.0]])
    out = torch.empty((1, bd.num, sp.shape[1], lp.shape[1]), device="cuda")
    R.mesh_exhaustive_forward(s["verts"].cuda(), s["faces"].cuda(), s["colors"].cuda(), sp.cuda(),
                              lp.cuda(), so.cuda(), lo[:, None, :].expand(1, lp.shape[1], 3).cuda(),
                              out, bd.width, bd.offset, 0)
    spn, lpn = sp[0].numpy(), lp[0].numpy()
    vs = oracle.mesh_visibility(n["verts"], n["faces"], spn)
    vl = oracle.mesh_visibility(n["verts"], n["faces"], lpn)
    ref = oracle.mesh_exhaustive_forward(n["verts"], n["faces"], n["colors"], spn, lpn,
                                         so[0].numpy(), np.repeat(lo.numpy(), lpn.shape[0], 0),
                                         vs, vl, bd.num, bd.width, bd.offset)
    assert rel_l2(out[0].cpu().numpy(), ref) < 1e-5


def test_matches_reference_golden(cuda_lib):
    g = dict(np.load(os.path.join(GOLDEN, "mesh_exhaustive.npz")))
    nb, bw, bo = int(g["bin"][0]), float(g["bin"][1]), float(g["bin"][2])
    verts = torch.as_tensor(g["verts"])[None].cuda()
    faces = torch.as_tensor(g["faces"])[None].cuda()
    colors = torch.as_tensor(g["colors"])[None].cuda()
    sp = torch.as_tensor(g["scan_points"])[None].cuda()
    lp = torch.as_tensor(g["laser_points"])[None].cuda()
    e = torch.empty_like(sp[:, :0])
    out = torch.empty((1, nb, sp.shape[1], lp.shape[1]), device="cuda")
    R.mesh_exhaustive_forward(verts, faces, colors, sp, lp, e, torch.empty_like(lp[:, :0]), out,
                              bw, bo, 0)
    assert rel_l2(out[0].cpu().numpy(), g["transient"]) < 1e-4
    vg, mg = torch.empty_like(verts), torch.empty_like(colors)
    R.mesh_exhaustive_grad_verts(verts, faces, colors, sp, lp, e, torch.empty_like(lp[:, :0]),
                                 torch.as_tensor(g["transient_grad"].astype(np.float32))[None]
                                 .cuda(), vg, mg, bw, bo, 0)
    assert rel_l2(vg[0].cpu().numpy(), g["verts_grad"]) < 1e-3
    assert rel_l2(mg[0].cpu().numpy(), g["colors_grad"]) < 1e-3


def test_filtered_fast_path_keeps_exact_bins(cuda_lib):
    """The exhaustive kernels decide vertex order and bins from fast lengths
    only where a proven margin says the exact chain decides the same. With the
    fast path off every triple takes the exact chain: transients and gradients
    agree to FP32 rounding."""
    from totri_gb300 import autotune
    s, sp, lp, bd = case(seed=4, s_res=8, l_res=4, nb=400, bw=0.0123)
    d = [s[k].cuda() for k in ("verts", "faces", "colors")]
    so = torch.empty((1, 0, 3), device="cuda")
    out = []
    for exact in (0, 1):
        autotune.set_tile("mesh.exhaustive.exact", exact)
        try:
            tr = torch.empty((1, bd.num, sp.shape[1], lp.shape[1]), device="cuda")
            R.mesh_exhaustive_forward(*d, sp.cuda(), lp.cuda(), so, so, tr, bd.width, 0.031, 0)
            vg, mg = torch.empty_like(d[0]), torch.empty_like(d[2])
            R.mesh_exhaustive_grad_verts(*d, sp.cuda(), lp.cuda(), so, so, tr, vg, mg, bd.width,
                                         0.031, 0)
            out.append((tr.cpu(), vg.cpu(), mg.cpu()))
        finally:
            autotune.set_tile("mesh.exhaustive.exact", 0)
    (a, va, ma), (b, vb, mb) = out
    # values differ by the few ulps of the bin coordinates (a partial bin's
    # width (b + 1 - c) moves by one ulp of c, ~1e-4 of that bin's share);
    # a bin or order taken differently would move whole tent pieces
    assert rel_l2(a.numpy(), b.numpy()) < 1e-5
    assert float((a - b).abs().max()) <= 2e-4 * float(b.abs().max())
    # gradients: FP32 cancellation amplifies the few-ulp value differences
    assert rel_l2(va.numpy(), vb.numpy()) < 1e-4
    assert rel_l2(ma.numpy(), mb.numpy()) < 1e-4
