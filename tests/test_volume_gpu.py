"""Volume renderer on the GPU against the FP64 oracle, the reference's golden
vectors, and the adjoint identity <A x, y> = <x, A^T y>.

Tolerances (rel-L2): forwards/adjoints 1e-5 vs the FP64 oracle; 1e-4 vs the
reference's FP32 outputs; measurement-point gradient 1e-4 vs the oracle.
"""
import os

import numpy as np
import pytest
import torch

import oracle
from totri_gb300 import scenes
from totri_gb300.render import VolumeRenderConfocal, VolumeRenderExhaustive
from totri_gb300.totri_cpp import render as R
from totri_gb300.types import BinDef, VolumeDef

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def cu(a):
    return torch.as_tensor(np.ascontiguousarray(a)).cuda()


def small_case(seed=0, X=12, N=40, T=96):
    g = np.random.default_rng(seed)
    vol = ((g.random((X, X, X)) < 0.1) * g.random((X, X, X))).astype(np.float32)
    mp = np.stack([g.uniform(-1, 1, N), g.uniform(-1, 1, N), np.zeros(N)]).astype(np.float32)
    return vol, mp, (-0.5, -0.5, 0.5), (1.0, 1.0, 1.0), T, 0.03, 0.0


def test_confocal_forward_adjoint_and_points_grad(cuda_lib):
    vol, mp, org, size, T, bw, bo = small_case()
    out = torch.full((mp.shape[1], T), 3.0, device="cuda")
    R.volume_confocal_forward(cu(vol), cu(mp), out, org, size, bw, bo)
    ref = oracle.volume_confocal_forward(vol, mp, T, org, size, bw, bo)
    assert rel(out.cpu().numpy(), ref) < 1e-5
    y = np.random.default_rng(1).standard_normal((mp.shape[1], T)).astype(np.float32)
    adj = torch.empty(vol.shape, device="cuda")
    R.volume_confocal_adjoint(adj, cu(mp), cu(y), org, size, bw, bo)
    assert rel(adj.cpu().numpy(), oracle.volume_confocal_adjoint(y, vol.shape, mp, org, size, bw,
                                                                 bo)) < 1e-5
    tr = torch.empty(vol.shape, device="cuda")
    R.volume_confocal_grad_volume(tr, cu(mp), cu(y), org, size, bw, bo)
    assert rel(tr.cpu().numpy(),
               oracle.volume_confocal_transposed(y, vol.shape, mp, org, size, bw, bo)) < 1e-5
    gm = torch.empty((3, mp.shape[1]), device="cuda")
    R.volume_confocal_grad_measurement_points(gm, cu(vol), cu(mp), cu(y), org, size, bw, bo)
    assert rel(gm.cpu().numpy(), oracle.volume_confocal_grad_mp(vol, mp, y, org, size, bw,
                                                                bo)) < 1e-4


def test_confocal_matches_reference_golden(cuda_lib):
    g = dict(np.load(os.path.join(GOLDEN, "volume_confocal.npz")))
    T, bw, bo = int(g["bin"][0]), float(g["bin"][1]), float(g["bin"][2])
    out = torch.empty((g["mp"].shape[1], T), device="cuda")
    R.volume_confocal_forward(cu(g["volume"]), cu(g["mp"]), out, g["origin"], g["size"], bw, bo)
    assert rel(out.cpu().numpy(), g["transient"]) < 1e-4
    tv = torch.empty(g["volume"].shape, device="cuda")
    R.volume_confocal_grad_volume(tv, cu(g["mp"]), cu(g["transient_grad"]), g["origin"],
                                  g["size"], bw, bo)
    assert rel(tv.cpu().numpy(), g["grad_volume"]) < 1e-4
    gm = torch.empty_like(cu(g["mp"]))
    R.volume_confocal_grad_measurement_points(gm, cu(g["volume"]), cu(g["mp"]),
                                              cu(g["transient_grad"]), g["origin"], g["size"],
                                              bw, bo)
    assert rel(gm.cpu().numpy(), g["grad_mp"]) < 1e-4


def test_confocal_autograd_uses_exact_adjoint(cuda_lib):
    vol, mp, org, size, T, bw, bo = small_case(seed=2)
    v = cu(vol).requires_grad_(True)
    p = cu(mp).requires_grad_(True)
    tr = VolumeRenderConfocal.apply(v, p, org, size, T, bw, bo)
    w = torch.randn_like(tr)
    (tr * w).sum().backward()
    adj = oracle.volume_confocal_adjoint(w.cpu().numpy(), vol.shape, mp, org, size, bw, bo)
    assert rel(v.grad.cpu().numpy(), adj) < 1e-5
    assert p.grad is not None and torch.isfinite(p.grad).all()


def test_confocal_full_size_adjoint_identity_and_sampled_points(cuda_lib):
    """128^3 voxels (2% occupied), 128x128 scan points, 1024 bins: the adjoint
    identity on the whole operator (FP64 reductions), and 12 transient rows
    against the FP64 oracle."""
    s = scenes.volume_scene()
    vd, bd = s["volume_def"], s["bin_def"]
    org = vd.start
    size = tuple(e - a for a, e in zip(vd.start, vd.end))
    vol = s["volume"].cuda()
    mp = s["scan_points"][0].T.contiguous().cuda()
    N, T = mp.shape[1], bd.num
    out = torch.empty((N, T), device="cuda")
    R.volume_confocal_forward(vol, mp, out, org, size, bd.width, bd.offset)
    # non-negative y: no cancellation in <Ax, y>, so the FP32 error stays relative
    y = torch.rand((N, T), device="cuda", generator=torch.Generator(device="cuda").manual_seed(12))
    adj = torch.empty_like(vol)
    R.volume_confocal_adjoint(adj, mp, y, org, size, bd.width, bd.offset)
    lhs = (out.double() * y.double()).sum().item()
    rhs = (vol.double() * adj.double()).sum().item()
    assert abs(lhs - rhs) <= 1e-5 * max(abs(lhs), abs(rhs))
    rows = np.random.default_rng(3).choice(N, 12, replace=False)
    ref = oracle.volume_confocal_forward(s["volume"].numpy(), mp[:, rows].cpu().numpy(), T, org,
                                         size, bd.width, bd.offset)
    assert rel(out[rows].cpu().numpy(), ref) < 1e-5


def exhaustive_case(seed=4):
    g = np.random.default_rng(seed)
    D, H, W, S, L, T = 6, 5, 7, 9, 4, 64
    vol = ((g.random((1, D, H, W)) < 0.3) * g.random((1, D, H, W))).astype(np.float32)
    sp = np.stack([g.uniform(-1, 1, S), g.uniform(-1, 1, S), np.zeros(S)])[None].astype(np.float32)
    lp = np.stack([g.uniform(-1, 1, L), g.uniform(-1, 1, L), np.zeros(L)])[None].astype(np.float32)
    return vol, sp, lp, T, (-0.5, -0.5, 0.5), (0.5, 0.5, 1.5), 0.05


def test_exhaustive_forward_and_adjoint(cuda_lib):
    vol, sp, lp, T, st, en, bw = exhaustive_case()
    vd = VolumeDef(st, en, vol.shape[1:])
    bd = BinDef(bw, 0.0, T)
    v = cu(vol).requires_grad_(True)
    tr = VolumeRenderExhaustive.apply(v, cu(sp), cu(lp), vd, bd)
    ref = oracle.volume_exhaustive_forward(vol[0], sp[0], lp[0], T, st, en, bw, 0.0)
    assert rel(tr[0].detach().cpu().numpy(), ref) < 1e-5
    g = dict(np.load(os.path.join(GOLDEN, "volume_exhaustive.npz")))
    out = torch.empty(g["transient"].shape, device="cuda")
    empty = torch.empty((1, 3, 0), device="cuda")
    R.volume_render_exhaustive_forward(cu(g["volume"]), cu(g["scan_points"]),
                                       cu(g["laser_points"]), empty, empty, out, g["start"],
                                       g["end"], float(g["bin"][1]), float(g["bin"][2]))
    assert rel(out.cpu().numpy(), g["transient"]) < 1e-4
    w = torch.randn_like(tr)
    (tr * w).sum().backward(retain_graph=True)
    adj = oracle.volume_exhaustive_adjoint(w[0].cpu().numpy(), vol.shape[1:], sp[0], lp[0], st,
                                           en, bw, 0.0)
    assert rel(v.grad[0].cpu().numpy(), adj) < 1e-5
    # adjoint identity with a non-negative cotangent (no cancellation in the sums)
    wp = torch.rand(tr.shape, device="cuda", generator=torch.Generator(device="cuda").manual_seed(13))
    v.grad = None
    (tr * wp).sum().backward()
    lhs = float((tr.detach().double() * wp.double()).sum())
    rhs = float((v.detach().double() * v.grad.double()).sum())
    assert abs(lhs - rhs) <= 1e-5 * abs(lhs)


def test_filtered_samples_keep_exact_cells(cuda_lib):
    """The confocal forward and adjoint take each sample's cell (floor of the
    depth coordinate) from a fast root only outside a proven rounding margin;
    with the fast path off every sample takes the exact chain. Volumes and
    transients agree to FP32 rounding: a cell taken differently would move a
    whole sample's weight to the neighbouring voxel."""
    from totri_gb300 import autotune
    s = scenes.volume_scene(res=64, scan_res=32, nbins=512)
    vd, bd = s["volume_def"], s["bin_def"]
    size = tuple(e - a for a, e in zip(vd.start, vd.end))
    vol = s["volume"].cuda()
    mp = s["scan_points"][0].T.contiguous().cuda()
    y = torch.rand((mp.shape[1], bd.num), device="cuda",
                   generator=torch.Generator(device="cuda").manual_seed(9))
    out = []
    for exact in (0, 1):
        autotune.set_tile("volume.exact", exact)
        try:
            tr = torch.empty((mp.shape[1], bd.num), device="cuda")
            R.volume_confocal_forward(vol, mp, tr, vd.start, size, bd.width, bd.offset)
            adj = torch.empty_like(vol)
            R.volume_confocal_adjoint(adj, mp, y, vd.start, size, bd.width, bd.offset)
            out.append((tr.cpu(), adj.cpu()))
        finally:
            autotune.set_tile("volume.exact", 0)
    (ta, aa), (tb, ab) = out
    for a, b in ((ta, tb), (aa, ab)):
        assert rel(a.numpy(), b.numpy()) < 1e-5
        assert float((a - b).abs().max()) <= 2e-4 * float(b.abs().max())


def column_case(Z, seed, bo=0.0, N=36, lift=False):
    """A 6 x 5 x Z volume over [-0.5, 0.5]^2 x [0.5, 1.5] m, N points on
    [-1, 1]^2 (heights 0, or up to 1.2 m with lift, so that some columns
    start below a point), 0.01 m bins to 3 m past the offset."""
    g = np.random.default_rng(seed)
    vol = ((g.random((6, 5, Z)) < 0.3) * g.random((6, 5, Z))).astype(np.float32)
    wz = g.uniform(0.0, 1.2, N) if lift else np.zeros(N)
    mp = np.stack([g.uniform(-1, 1, N), g.uniform(-1, 1, N), wz]).astype(np.float32)
    T = int(round((3.0 - bo) / 0.01))
    return vol, mp, (-0.5, -0.5, 0.5), (1.0, 1.0, 1.0), T, 0.01, bo


@pytest.mark.parametrize("Z", [1, 19, 32, 40, 100, 128, 200, 256, 300])
@pytest.mark.parametrize("mode", [0, 1, 2])
def test_adjoint_kernels_match_oracle(cuda_lib, Z, mode):
    """The three adjoint kernels ("volume.adjoint.mode": 0 lanes over 32
    columns, the default; 1 shared-memory atomics; 2 lane-owned cells, for
    columns of up to 256 cells, else the atomic kernel) against the FP64 exact
    adjoint, at column depths that take every cells-per-lane variant and its
    edges, on a 6 x 5 column grid (a partial 8 x 4 tile), with points below
    and inside the volume's height range."""
    from totri_gb300 import autotune
    vol, mp, org, size, T, bw, bo = column_case(Z, seed=Z, lift=True)
    y = np.random.default_rng(Z + 1).standard_normal((mp.shape[1], T)).astype(np.float32)
    ref = oracle.volume_confocal_adjoint(y, vol.shape, mp, org, size, bw, bo)
    autotune.set_tile("volume.adjoint.mode", mode)
    try:
        adj = torch.full(vol.shape, 7.0, device="cuda")
        R.volume_confocal_adjoint(adj, cu(mp), cu(y), org, size, bw, bo)
    finally:
        autotune.set_tile("volume.adjoint.mode", 0)
    got = adj.cpu().numpy()
    if Z == 1:  # a single cell has no interpolation pair: no samples
        assert not got.any() and not ref.any()
        return
    # the interpolation weight z_hat - floor(z_hat) keeps the FP32 rounding of
    # z_hat in [0, Z) (the reference's arithmetic), an absolute error that
    # grows with the column depth: 1e-5 up to 200 cells, in proportion beyond
    assert rel(got, ref) < 1e-5 * max(1.0, Z / 200.0)


@pytest.mark.parametrize("mode", [0, 1, 2])
def test_negative_bin_offset(cuda_lib, mode):
    """With a negative bin offset the first bins have negative centres; their
    samples (the centre squared, as the reference computes them) reach the
    volume when |offset| exceeds a point's horizontal distance to a column.
    Forward, adjoint (both kernels) and measurement-point gradient against the
    FP64 oracle, which walks every bin."""
    from totri_gb300 import autotune
    vol, mp, org, size, T, bw, bo = column_case(48, seed=5, bo=-1.0)
    out = torch.full((mp.shape[1], T), 3.0, device="cuda")
    R.volume_confocal_forward(cu(vol), cu(mp), out, org, size, bw, bo)
    ref = oracle.volume_confocal_forward(vol, mp, T, org, size, bw, bo)
    assert np.abs(ref[:, :100]).sum() > 0.05 * np.abs(ref).sum()  # negative centres count
    assert rel(out.cpu().numpy(), ref) < 1e-5
    y = np.random.default_rng(6).standard_normal((mp.shape[1], T)).astype(np.float32)
    autotune.set_tile("volume.adjoint.mode", mode)
    try:
        adj = torch.empty(vol.shape, device="cuda")
        R.volume_confocal_adjoint(adj, cu(mp), cu(y), org, size, bw, bo)
    finally:
        autotune.set_tile("volume.adjoint.mode", 0)
    assert rel(adj.cpu().numpy(),
               oracle.volume_confocal_adjoint(y, vol.shape, mp, org, size, bw, bo)) < 1e-5
    gm = torch.empty((3, mp.shape[1]), device="cuda")
    R.volume_confocal_grad_measurement_points(gm, cu(vol), cu(mp), cu(y), org, size, bw, bo)
    assert rel(gm.cpu().numpy(), oracle.volume_confocal_grad_mp(vol, mp, y, org, size, bw,
                                                                bo)) < 1e-4


def test_adjoint_kernels_full_size_agree(cuda_lib):
    """128^3 voxels x 128x128 points x 1024 bins: the three adjoint kernels
    agree to FP32 summation order (the same samples, each decided by the
    exact chain)."""
    from totri_gb300 import autotune
    s = scenes.volume_scene()
    vd, bd = s["volume_def"], s["bin_def"]
    size = tuple(e - a for a, e in zip(vd.start, vd.end))
    mp = s["scan_points"][0].T.contiguous().cuda()
    y = torch.randn((mp.shape[1], bd.num), device="cuda",
                    generator=torch.Generator(device="cuda").manual_seed(21))
    out = []
    for mode in (0, 1, 2):
        autotune.set_tile("volume.adjoint.mode", mode)
        try:
            adj = torch.empty((128, 128, 128), device="cuda")
            R.volume_confocal_adjoint(adj, mp, y, vd.start, size, bd.width, bd.offset)
            out.append(adj.cpu().numpy())
        finally:
            autotune.set_tile("volume.adjoint.mode", 0)
    assert rel(out[0], out[1]) < 1e-5
    assert rel(out[2], out[1]) < 1e-5


@pytest.mark.parametrize("warps", [1, 3, 8])
def test_adjoint_columns_kernel_block_shapes(cuda_lib, warps):
    """The lanes-over-columns adjoint with 1, 3 and 8 warps per CTA (its
    point groups and per-warp column copies) against the FP64 exact adjoint,
    on a 13 x 9 column grid (partial tiles in both directions)."""
    from totri_gb300 import autotune
    g = np.random.default_rng(warps)
    vol = np.zeros((13, 9, 70), np.float32)
    N = 150
    mp = np.stack([g.uniform(-1, 1, N), g.uniform(-1, 1, N), g.uniform(0, 0.8, N)]).astype(
        np.float32)
    org, size, T, bw, bo = (-0.5, -0.5, 0.5), (1.0, 1.0, 1.0), 300, 0.01, 0.0
    y = g.standard_normal((N, T)).astype(np.float32)
    ref = oracle.volume_confocal_adjoint(y, vol.shape, mp, org, size, bw, bo)
    autotune.set_tile("volume.adjoint.warps", warps)
    try:
        adj = torch.full(vol.shape, 5.0, device="cuda")
        R.volume_confocal_adjoint(adj, cu(mp), cu(y), org, size, bw, bo)
    finally:
        autotune.set_tile("volume.adjoint.warps", 0)
    assert rel(adj.cpu().numpy(), ref) < 1e-5


@pytest.mark.parametrize("slabs", [1, 2, 3, 7])
def test_adjoint_columns_kernel_slabs(cuda_lib, slabs):
    """The lanes-over-columns adjoint with its columns whole or split into z
    slabs of cells, a CTA per slab ("volume.adjoint.slabs"; slabs that do not
    divide the column, sample pairs straddling two slabs), against the FP64
    exact adjoint: lifted points (columns that start below a point) and a
    negative bin offset."""
    from totri_gb300 import autotune
    for Z, bo in ((100, 0.0), (48, -1.0), (19, 0.0)):
        vol, mp, org, size, T, bw, bo = column_case(Z, seed=Z + slabs, bo=bo, lift=True)
        y = np.random.default_rng(Z + 3).standard_normal((mp.shape[1], T)).astype(np.float32)
        ref = oracle.volume_confocal_adjoint(y, vol.shape, mp, org, size, bw, bo)
        autotune.set_tile("volume.adjoint.slabs", slabs)
        try:
            adj = torch.full(vol.shape, 7.0, device="cuda")
            R.volume_confocal_adjoint(adj, cu(mp), cu(y), org, size, bw, bo)
        finally:
            autotune.set_tile("volume.adjoint.slabs", 0)
        assert rel(adj.cpu().numpy(), ref) < 1e-5


@pytest.mark.parametrize("seed", range(8))
def test_forward_keeps_every_sample_of_sparse_volumes(cuda_lib, seed):
    """Three occupied voxels and 400 points: each transient bin holds one or
    two samples, so a sample missing from a (voxel, point) pair's walked bins
    (bin_range widens its span by a rounding bound, a small fraction of a bin)
    would move the result by a percent, far past the 1e-5 bound. Points on and
    off the occupied columns (including straight below them), below and
    inside the volume's height; bin widths of 1 mm to 2 cm, with and without a
    negative bin offset; forward and measurement-point gradient against the
    FP64 oracle."""
    g = np.random.default_rng(100 + seed)
    X, Y, Z = 7, 6, int(g.integers(20, 140))
    vol = np.zeros((X, Y, Z), np.float32)
    cols = []
    for _ in range(3):
        ix, iy = int(g.integers(X)), int(g.integers(Y))
        vol[ix, iy, g.integers(Z)] = g.uniform(0.5, 1.5)
        cols.append((ix, iy))
    org, size = (-0.5, -0.5, 0.5), (1.0, 1.0, 1.0)
    N = 400
    px, py = g.uniform(-1, 1, N), g.uniform(-1, 1, N)
    for j, (ix, iy) in enumerate(cols):  # straight below an occupied column
        px[j] = org[0] + (ix + 0.5) * size[0] / X
        py[j] = org[1] + (iy + 0.5) * size[1] / Y
    wz = np.where(g.random(N) < 0.3, g.uniform(0, 1.2, N), 0.0)
    mp = np.stack([px, py, wz]).astype(np.float32)
    bw = (0.001, 0.003, 0.01, 0.02)[seed % 4]
    bo = -0.5 if seed % 2 else 0.0
    T = int(round((3.2 - bo) / bw))
    ref = oracle.volume_confocal_forward(vol, mp, T, org, size, bw, bo)
    assert (ref > 0).sum() > 100
    out = torch.full((N, T), 3.0, device="cuda")
    R.volume_confocal_forward(cu(vol), cu(mp), out, org, size, bw, bo)
    assert rel(out.cpu().numpy(), ref) < 1e-5
    y = np.random.default_rng(seed).standard_normal((N, T)).astype(np.float32)
    gm = torch.empty((3, N), device="cuda")
    R.volume_confocal_grad_measurement_points(gm, cu(vol), cu(mp), cu(y), org, size, bw, bo)
    assert rel(gm.cpu().numpy(), oracle.volume_confocal_grad_mp(vol, mp, y, org, size, bw,
                                                                bo)) < 1e-4


@pytest.mark.parametrize("seed", range(4))
def test_adjoint_keeps_every_sample_of_sparse_cotangents(cuda_lib, seed):
    """A cotangent with a few nonzero bins: each cell of the adjoint then sums
    a handful of samples, so one missing from a lane's walked bins (its span is
    widened by a rounding bound, a small fraction of a bin) would show far past
    the 1e-5 bound. Whole columns and slabs, lifted points, a negative bin
    offset; against the FP64 exact adjoint."""
    from totri_gb300 import autotune
    vol, mp, org, size, T, bw, bo = column_case(int(60 + 30 * seed), seed=200 + seed,
                                                bo=-0.5 if seed % 2 else 0.0, lift=True)
    g = np.random.default_rng(300 + seed)
    y = np.zeros((mp.shape[1], T), np.float32)
    hot = g.random(y.shape) < 0.01
    y[hot] = g.standard_normal(hot.sum()).astype(np.float32)
    ref = oracle.volume_confocal_adjoint(y, vol.shape, mp, org, size, bw, bo)
    assert (ref != 0).sum() > 50
    for slabs in (1, 3):
        autotune.set_tile("volume.adjoint.slabs", slabs)
        try:
            adj = torch.full(vol.shape, 7.0, device="cuda")
            R.volume_confocal_adjoint(adj, cu(mp), cu(y), org, size, bw, bo)
        finally:
            autotune.set_tile("volume.adjoint.slabs", 0)
        assert rel(adj.cpu().numpy(), ref) < 1e-5
