"""Confocal mesh path on the GPU against the CPU oracle.

Tolerances (from the path's contract): visibility masks and bin decisions are
exact (masks compared bit for bit); transients and vertex/albedo gradients
within rel-L2 1e-5 of the FP64 oracle (the gradient kernel places the tent
corners relative to their first bin from double-float path lengths; plain
FP32 bin coordinates, as in the reference and the oracle's FP32 mode, leave
errors of order 1e-4).
"""
import numpy as np
import pytest
import torch

import oracle
from totri_gb300 import scenes
from totri_gb300.render import MeshRenderConfocal
from totri_gb300.totri_cpp import render as R

from mesh_util import np_scene, rel_l2, unpack_mask

pytestmark = pytest.mark.gpu

FWD_TOL = 1e-5
GRAD_TOL = 1e-5


def _dev(s):
    return {k: (v.cuda() if torch.is_tensor(v) else v) for k, v in s.items()}


def _oracle_forward(n, vis, bin_def, origin=None):
    return oracle.mesh_confocal_forward(n["verts"], n["faces"], n["colors"], n["scan_points"],
                                        origin, vis, bin_def.num, bin_def.width,
                                        bin_def.offset, fp64=True)


def test_visibility_matches_brute_force_small(cuda_lib):
    s = scenes.confocal_small()
    d, n = _dev(s), np_scene(s)
    F = n["faces"].shape[0]
    ref = oracle.mesh_visibility(n["verts"], n["faces"], n["scan_points"])
    bf = R.mesh_visibility(d["verts"], d["faces"], d["scan_points"], brute_force=True)
    bvh = R.mesh_visibility(d["verts"], d["faces"], d["scan_points"])
    assert np.array_equal(unpack_mask(bf[0].cpu().numpy(), F), ref)
    assert np.array_equal(unpack_mask(bvh[0].cpu().numpy(), F), ref)
    assert 0.2 < ref.mean() < 0.6


def test_forward_small_matches_oracle(cuda_lib):
    s = scenes.confocal_small()
    d, n = _dev(s), np_scene(s)
    bd = s["bin_def"]
    vis = oracle.mesh_visibility(n["verts"], n["faces"], n["scan_points"])
    ref = _oracle_forward(n, vis, bd)
    out = torch.full((1, bd.num, n["scan_points"].shape[0]), 7.0, device="cuda")
    R.mesh_confocal_forward(d["verts"], d["faces"], d["colors"], d["scan_points"],
                            torch.empty_like(d["scan_points"][:, :0]), out, bd.width,
                            bd.offset, 0)
    got = out[0].double().cpu().numpy()
    assert rel_l2(got, ref) < FWD_TOL
    # bins where the oracle has no contribution stay exactly zero
    assert np.all(got[ref == 0] == 0)


def test_forward_with_origin_and_int64_faces(cuda_lib):
    s = scenes.confocal_small(seed=5)
    d, n = _dev(s), np_scene(s)
    bd = s["bin_def"]
    origin = torch.tensor([[0.3, -0.2, -1.0]])
    so = origin[:, None, :].expand(1, n["scan_points"].shape[0], 3)
    vis = oracle.mesh_visibility(n["verts"], n["faces"], n["scan_points"])
    ref = oracle.mesh_confocal_forward(n["verts"], n["faces"], n["colors"], n["scan_points"],
                                       so[0].numpy(), vis, 1024, bd.width, bd.offset, fp64=True)
    out = torch.empty((1, 1024, n["scan_points"].shape[0]), device="cuda")
    R.mesh_confocal_forward(d["verts"], d["faces"].long(), d["colors"], d["scan_points"],
                            so.cuda(), out, bd.width, bd.offset, 0)
    assert rel_l2(out[0].double().cpu().numpy(), ref) < FWD_TOL


def test_grad_small_matches_oracle(cuda_lib):
    s = scenes.confocal_small(seed=3)
    d, n = _dev(s), np_scene(s)
    bd = s["bin_def"]
    S = n["scan_points"].shape[0]
    vis = oracle.mesh_visibility(n["verts"], n["faces"], n["scan_points"])
    tg = np.random.default_rng(0).standard_normal((bd.num, S)).astype(np.float32)
    rv, rm = oracle.mesh_confocal_grad(n["verts"], n["faces"], n["colors"], n["scan_points"],
                                       None, vis, bd.num, bd.width, bd.offset, tg, fp64=True)
    vg = torch.full_like(d["verts"], 3.0)
    mg = torch.full_like(d["colors"], 3.0)
    R.mesh_confocal_grad_verts(d["verts"], d["faces"], d["colors"], d["scan_points"],
                               torch.empty_like(d["scan_points"][:, :0]),
                               torch.from_numpy(tg)[None].cuda(), vg, mg, bd.width, bd.offset, 0)
    assert rel_l2(vg[0].double().cpu().numpy(), rv) < GRAD_TOL
    assert rel_l2(mg[0].double().cpu().numpy(), rm) < GRAD_TOL


def test_autograd_reuse_matches_plain_calls(cuda_lib):
    s = scenes.confocal_small(seed=4)
    d = _dev(s)
    bd = s["bin_def"]
    verts = d["verts"].clone().requires_grad_(True)
    colors = d["colors"].clone().requires_grad_(True)
    tr = MeshRenderConfocal.apply(verts, d["faces"], d["scan_points"], bd, colors)
    g = torch.randn_like(tr)
    tr.backward(g)
    out = torch.empty_like(tr)
    R.mesh_confocal_forward(d["verts"], d["faces"], d["colors"], d["scan_points"],
                            torch.empty_like(d["scan_points"][:, :0]), out, bd.width, bd.offset, 0)
    vg = torch.empty_like(d["verts"])
    mg = torch.empty_like(d["colors"])
    R.mesh_confocal_grad_verts(d["verts"], d["faces"], d["colors"], d["scan_points"],
                               torch.empty_like(d["scan_points"][:, :0]), g, vg, mg, bd.width,
                               bd.offset, 0)
    # shared-memory atomics add in a run-dependent order: equal up to FP32 rounding
    assert rel_l2(tr.detach().cpu().numpy(), out.cpu().numpy()) < 1e-6
    assert rel_l2(verts.grad.cpu().numpy(), vg.cpu().numpy()) < 1e-5
    assert rel_l2(colors.grad.cpu().numpy(), mg.cpu().numpy()) < 1e-5


def test_padded_and_empty_faces(cuda_lib):
    s = scenes.confocal_small(seed=6)
    d, n = _dev(s), np_scene(s)
    bd = s["bin_def"]
    faces = d["faces"].clone()
    faces[0, 200, 1] = -1  # the list ends at face 200
    faces[0, 250, 0] = -5
    vis = oracle.mesh_visibility(n["verts"], faces[0].cpu().numpy(), n["scan_points"])
    assert vis[:, 200:].sum() == 0
    ref = oracle.mesh_confocal_forward(n["verts"], faces[0].cpu().numpy(), n["colors"],
                                       n["scan_points"], None, vis, bd.num, bd.width,
                                       bd.offset, fp64=True)
    out = torch.empty((1, bd.num, n["scan_points"].shape[0]), device="cuda")
    R.mesh_confocal_forward(d["verts"], faces, d["colors"], d["scan_points"],
                            torch.empty_like(d["scan_points"][:, :0]), out, bd.width, bd.offset, 0)
    assert rel_l2(out[0].double().cpu().numpy(), ref) < FWD_TOL
    empty = torch.full_like(out, 5.0)
    R.mesh_confocal_forward(d["verts"], faces[:, :0], d["colors"], d["scan_points"],
                            torch.empty_like(d["scan_points"][:, :0]), empty, bd.width,
                            bd.offset, 0)
    assert float(empty.abs().max()) == 0.0


def test_batch_of_two_meshes(cuda_lib):
    a = scenes.confocal_small(seed=7)
    b = scenes.confocal_small(seed=8)
    bd = a["bin_def"]
    verts = torch.cat([a["verts"], b["verts"]]).cuda()
    colors = torch.cat([a["colors"], b["colors"]]).cuda()
    sp = torch.cat([a["scan_points"], b["scan_points"]]).cuda()
    tr = MeshRenderConfocal.apply(verts, a["faces"].cuda().expand(2, -1, -1), sp, bd, colors)
    for i, s in enumerate((a, b)):
        n = np_scene(s)
        vis = oracle.mesh_visibility(n["verts"], n["faces"], n["scan_points"])
        ref = _oracle_forward(n, vis, bd)
        assert rel_l2(tr[i].double().cpu().numpy(), ref) < FWD_TOL


def test_differentiable_workload_visibility_and_forward(cuda_lib):
    """Full-size differentiable scene (20,480 faces x 4,096 scan points): BVH masks
    equal the GPU brute-force masks everywhere and the oracle on a sample of pairs;
    the forward matches the FP64 oracle evaluated on those masks."""
    s = scenes.confocal_differentiable()
    d, n = _dev(s), np_scene(s)
    bd = s["bin_def"]
    F = n["faces"].shape[0]
    bvh = unpack_mask(R.mesh_visibility(d["verts"], d["faces"], d["scan_points"])[0]
                      .cpu().numpy(), F)
    bf = unpack_mask(R.mesh_visibility(d["verts"], d["faces"], d["scan_points"],
                                       brute_force=True)[0].cpu().numpy(), F)
    assert np.array_equal(bvh, bf)
    g = np.random.default_rng(1)
    pp = g.integers(0, n["scan_points"].shape[0], 3000)
    pf = g.integers(0, F, 3000)
    ref = oracle.mesh_visibility_pairs(n["verts"], n["faces"], n["scan_points"], pp, pf)
    assert np.array_equal(bvh[pp, pf], ref)
    out = torch.empty((1, bd.num, n["scan_points"].shape[0]), device="cuda")
    R.mesh_confocal_forward(d["verts"], d["faces"], d["colors"], d["scan_points"],
                            torch.empty_like(d["scan_points"][:, :0]), out, bd.width, bd.offset, 0)
    ref = _oracle_forward(n, bvh, bd)
    assert rel_l2(out[0].double().cpu().numpy(), ref) < FWD_TOL


def test_filtered_fast_path_keeps_exact_bins(cuda_lib):
    """The splat takes vertex order and bins from fast lengths only where a
    proven margin says the exact chain decides the same; with the fast path off
    (every pair exact) the full-size transient agrees to FP32 rounding. The
    gradient always runs the exact chain, so it is unchanged."""
    from totri_gb300 import autotune
    s = scenes.confocal_differentiable()
    d = _dev(s)
    bd = s["bin_def"]
    empty = torch.empty_like(d["scan_points"][:, :0])
    tg = torch.randn((1, bd.num, d["scan_points"].shape[1]), device="cuda",
                     generator=torch.Generator(device="cuda").manual_seed(3))
    out = []
    for exact in (0, 1):
        autotune.set_tile("mesh.confocal.exact", exact)
        try:
            tr = torch.empty((1, bd.num, d["scan_points"].shape[1]), device="cuda")
            R.mesh_confocal_forward(d["verts"], d["faces"], d["colors"], d["scan_points"], empty,
                                    tr, bd.width, 0.0137, 0)
            vg, mg = torch.empty_like(d["verts"]), torch.empty_like(d["colors"])
            R.mesh_confocal_grad_verts(d["verts"], d["faces"], d["colors"], d["scan_points"],
                                       empty, tg, vg, mg, bd.width, 0.0137, 0)
            out.append((tr.cpu(), vg.cpu(), mg.cpu()))
        finally:
            autotune.set_tile("mesh.confocal.exact", 0)
    (a, va, ma), (b, vb, mb) = out
    # values differ by the few ulps of the bin coordinates (a partial bin's
    # width (b + 1 - c) moves by one ulp of c, ~1e-4 of that bin's share);
    # a bin or order taken differently would move whole tent pieces
    assert rel_l2(a.numpy(), b.numpy()) < 1e-5
    assert float((a - b).abs().max()) <= 2e-4 * float(b.abs().max())
    # the gradient takes the exact chain either way (atomic order only)
    assert rel_l2(va.numpy(), vb.numpy()) < 1e-5
    assert rel_l2(ma.numpy(), mb.numpy()) < 1e-5


@pytest.mark.parametrize("ts", [1, 4, 8, 16])
def test_compact_splat_matches_pair_per_thread(cuda_lib, ts):
    """The compacted splat (visible pairs queued per warp) sums the same
    contributions as the pair-per-thread splat, at every scan tile width; only
    the order of the shared-memory atomics differs. The small scene with
    padded faces checks it against the FP64 oracle as well."""
    from totri_gb300 import autotune
    s = scenes.confocal_differentiable()
    d = _dev(s)
    bd = s["bin_def"]
    empty = torch.empty_like(d["scan_points"][:, :0])
    out = []
    for mode in (0, 1):
        autotune.set_tile("mesh.confocal.splat.mode", mode)
        autotune.set_tile("mesh.confocal.splat.ts", ts)
        try:
            tr = torch.empty((1, bd.num, d["scan_points"].shape[1]), device="cuda")
            R.mesh_confocal_forward(d["verts"], d["faces"], d["colors"], d["scan_points"], empty,
                                    tr, bd.width, bd.offset, 0)
            out.append(tr.cpu().numpy())
        finally:
            autotune.set_tile("mesh.confocal.splat.mode", 0)
            autotune.set_tile("mesh.confocal.splat.ts", 0)
    assert rel_l2(out[1], out[0]) < 1e-6
    assert np.array_equal(out[1] == 0, out[0] == 0)

    sm = scenes.confocal_small(seed=6)
    n = np_scene(sm)
    bd = sm["bin_def"]
    ds = _dev(sm)
    ds["faces"][0, 201, 2] = -1  # the list ends at face 201, inside a 32-face chunk
    n["faces"] = ds["faces"][0].cpu().numpy()
    vis = oracle.mesh_visibility(n["verts"], n["faces"], n["scan_points"])
    ref = _oracle_forward(n, vis, bd)
    autotune.set_tile("mesh.confocal.splat.mode", 1)
    autotune.set_tile("mesh.confocal.splat.ts", ts)
    try:
        tr = torch.empty((1, bd.num, n["scan_points"].shape[0]), device="cuda")
        R.mesh_confocal_forward(ds["verts"], ds["faces"], ds["colors"], ds["scan_points"],
                                torch.empty_like(ds["scan_points"][:, :0]), tr, bd.width,
                                bd.offset, 0)
    finally:
        autotune.set_tile("mesh.confocal.splat.mode", 0)
        autotune.set_tile("mesh.confocal.splat.ts", 0)
    assert rel_l2(tr[0].double().cpu().numpy(), ref) < FWD_TOL


_SEED_CASES = [  # (mesh.visibility.seed, mesh.visibility.seed.steps, mesh.visibility.chunks)
    (1, 0, 0),   # surface walk off
    (0, 0, 0),   # defaults: faces seen from behind, 48 steps, chunks by grid size
    (2, 4, 3),   # every target, short walks, 3 chunks per block
    (3, 64, 16),
    (0, 1, 1),
]


def _with_seed(case, fn):
    from totri_gb300 import autotune
    keys = ("mesh.visibility.seed", "mesh.visibility.seed.steps", "mesh.visibility.chunks")
    for k, v in zip(keys, case):
        autotune.set_tile(k, v)
    try:
        return fn()
    finally:
        for k in keys:
            autotune.set_tile(k, 0)


# visibility kernels: the 4-wide BVH searches (the default) at 4 and 5 CTAs
# per SM, the binary searches at 5, 4 and 3, and the queued searches at 5 and 4
_KERNELS = [{}, {"mesh.visibility.occupancy": 5},
            {"mesh.visibility.wide": 2}, {"mesh.visibility.wide": 2, "mesh.visibility.occupancy": 4},
            {"mesh.visibility.wide": 2, "mesh.visibility.occupancy": 1},
            {"mesh.visibility.queue": 1},
            {"mesh.visibility.queue": 1, "mesh.visibility.occupancy": 4}]


@pytest.fixture(scope="module")
def differentiable_brute_force(cuda_lib):
    """The full-size workload on the device and its GPU brute-force masks."""
    d = _dev(scenes.confocal_differentiable())
    return d, R.mesh_visibility(d["verts"], d["faces"], d["scan_points"], brute_force=True)


@pytest.mark.parametrize("kernel", _KERNELS)
def test_seeded_visibility_equals_brute_force(differentiable_brute_force, kernel):
    """The surface walk from the last occluder of each wall point can only
    prove 'not visible' with the exact leaf test, and the queued BVH searches
    run the same search per ray, so the masks equal the brute-force masks bit
    for bit whatever the walk's settings; full-size 20,480-face workload."""
    d, bf = differentiable_brute_force
    for case in _SEED_CASES:
        got = _with_keys(kernel, lambda: _with_seed(case, lambda: R.mesh_visibility(
            d["verts"], d["faces"], d["scan_points"])))
        assert torch.equal(got, bf), (kernel, case)


def _with_keys(keys, fn):
    from totri_gb300 import autotune
    for k, v in keys.items():
        autotune.set_tile(k, v)
    try:
        return fn()
    finally:
        for k in keys:
            autotune.set_tile(k, 0)


def test_shaft_visibility_equals_brute_force(differentiable_brute_force):
    """The shaft search (one warp-wide BVH walk per target over the hull of
    the warp's wall points and the target's hit box, then exact tests of its
    candidates per lane) gives the brute-force masks bit for bit: with the
    surface walk on or off, with the candidate list capped to force the
    per-lane fallback, and with the wall 40 m away."""
    d, bf = differentiable_brute_force
    for seed, cap in ((0, 0), (1, 0), (0, 1), (2, 5)):
        got = _with_keys({"mesh.visibility.mode": 7, "mesh.visibility.seed": seed,
                          "mesh.visibility.shaft.cap": cap},
                         lambda: R.mesh_visibility(d["verts"], d["faces"], d["scan_points"]))
        assert torch.equal(got, bf), (seed, cap)
    far = d["scan_points"].clone()
    far[..., 2] = -40.0
    far[..., :2] *= 20.0
    bf = R.mesh_visibility(d["verts"], d["faces"], far, brute_force=True)
    got = _with_keys({"mesh.visibility.mode": 7},
                     lambda: R.mesh_visibility(d["verts"], d["faces"], far))
    assert torch.equal(got, bf)


@pytest.mark.parametrize("kernel", _KERNELS)
def test_seeded_visibility_without_or_with_odd_adjacency(cuda_lib, kernel):
    """Edge adjacency only steers the walk: a triangle soup (no shared vertex
    indices), non-manifold fins (three faces on one edge) and degenerate faces
    leave the masks equal to the oracle's."""
    s = scenes.confocal_small(seed=4)
    v, f = s["verts"][0], s["faces"][0]
    soup_v = v[f.reshape(-1).long()].reshape(1, -1, 3).contiguous()
    soup_f = torch.arange(soup_v.shape[1], dtype=f.dtype).reshape(1, -1, 3)
    fins = torch.stack([f[:40, 0], f[:40, 1], f[40:80, 2]], 1)  # reuse edges of 40 faces
    degen = torch.stack([f[80:90, 0], f[80:90, 0], f[80:90, 1]], 1)
    odd_f = torch.cat([f, fins, degen])[None].contiguous()
    pts = s["scan_points"]
    for verts, faces in ((soup_v, soup_f), (v[None].contiguous(), odd_f)):
        ref = oracle.mesh_visibility(verts[0].numpy(), faces[0].numpy(), pts[0].numpy())
        F = faces.shape[1]
        for case in _SEED_CASES:
            got = _with_keys(kernel, lambda: _with_seed(case, lambda: R.mesh_visibility(
                verts.cuda(), faces.cuda(), pts.cuda())))
            assert np.array_equal(unpack_mask(got[0].cpu().numpy(), F), ref), (kernel, case)


def test_unoccluded_render_and_gradient_match_oracle_without_visibility(cuda_lib):
    """The unoccluded three-bounce render of the config-0 scene (level-2
    icosphere, 32x32 scan, 512 bins): every (scan point, face) pair counts, as
    the FP64 oracle with an all-ones mask computes it; through the C ABI and
    through MeshRenderConfocal.apply(..., visibility=False) forward and
    backward (whose gradient reuses the forward's all-visible masks)."""
    s = scenes.confocal_small()
    d, n = _dev(s), np_scene(s)
    bd = s["bin_def"]
    S, F = n["scan_points"].shape[0], n["faces"].shape[0]
    ones = np.ones((S, F), np.uint8)
    ref = _oracle_forward(n, ones, bd)
    vis = oracle.mesh_visibility(n["verts"], n["faces"], n["scan_points"])
    assert np.abs(ref).sum() > 1.2 * np.abs(_oracle_forward(n, vis, bd)).sum()  # occlusion matters
    empty = torch.empty_like(d["scan_points"][:, :0])
    out = torch.full((1, bd.num, S), 7.0, device="cuda")
    R.mesh_confocal_forward_unoccluded(d["verts"], d["faces"], d["colors"], d["scan_points"],
                                       empty, out, bd.width, bd.offset, 0)
    assert rel_l2(out[0].double().cpu().numpy(), ref) < FWD_TOL
    tg = np.random.default_rng(4).standard_normal(ref.shape)
    rv, rm = oracle.mesh_confocal_grad(n["verts"], n["faces"], n["colors"], n["scan_points"],
                                       None, ones, bd.num, bd.width, bd.offset, tg)
    vg, mg = torch.empty_like(d["verts"]), torch.empty_like(d["colors"])
    R.mesh_confocal_grad_verts_unoccluded(d["verts"], d["faces"], d["colors"], d["scan_points"],
                                          empty, torch.tensor(tg, dtype=torch.float32)[None].cuda(),
                                          vg, mg, bd.width, bd.offset, 0)
    assert rel_l2(vg[0].double().cpu().numpy(), rv) < GRAD_TOL
    assert rel_l2(mg[0].double().cpu().numpy(), rm) < GRAD_TOL
    verts = d["verts"].clone().requires_grad_(True)
    colors = d["colors"].clone().requires_grad_(True)
    tr = MeshRenderConfocal.apply(verts, d["faces"], d["scan_points"], bd, colors, None, False)
    assert rel_l2(tr[0].detach().double().cpu().numpy(), ref) < FWD_TOL
    (tr * torch.tensor(tg, dtype=torch.float32)[None].cuda()).sum().backward()
    assert rel_l2(verts.grad[0].double().cpu().numpy(), rv) < GRAD_TOL
    assert rel_l2(colors.grad[0].double().cpu().numpy(), rm) < GRAD_TOL
