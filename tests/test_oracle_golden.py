"""The CPU oracle against golden vectors from the reference's own code.

tests/golden/*.npz hold seeded inputs and the outputs of the reference's kernel
sources compiled for the CPU (tests/golden/make_golden.py). The reference
computes in FP32; the oracle in FP64 with FP32 discrete decisions.
Tolerances (rel-L2): forwards and volume/backprojection/RBF gradients 1e-5;
mesh vertex gradients 1e-4 (the reference's FP32 gradient formula cancels).
"""
import os

import numpy as np
import pytest

import oracle

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load(name):
    return dict(np.load(os.path.join(GOLDEN, name + ".npz")))


def rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def test_mesh_confocal_golden():
    g = load("mesh_confocal")
    nb, bw, bo = int(g["bin"][0]), float(g["bin"][1]), float(g["bin"][2])
    vis = oracle.mesh_visibility(g["verts"], g["faces"], g["scan_points"])
    assert np.array_equal(vis, g["vis"])  # our FP32 visibility semantics are stable
    tr = oracle.mesh_confocal_forward(g["verts"], g["faces"], g["colors"], g["scan_points"], None,
                                      vis, nb, bw, bo)
    assert rel(tr, g["transient"]) < 1e-5
    tro = oracle.mesh_confocal_forward(g["verts"], g["faces"], g["colors"], g["scan_points"],
                                       g["scan_origin"], vis, 1024, bw, bo)
    assert rel(tro, g["transient_origin"]) < 1e-5
    sub = g["grad_points"]
    vg, mg = oracle.mesh_confocal_grad(g["verts"], g["faces"], g["colors"], g["scan_points"][sub],
                                       None, vis[sub], nb, bw, bo,
                                       g["transient_grad"].astype(np.float64))
    assert rel(vg, g["verts_grad"]) < 1e-4
    assert rel(mg, g["colors_grad"]) < 1e-5


def test_mesh_exhaustive_golden():
    g = load("mesh_exhaustive")
    nb, bw, bo = int(g["bin"][0]), float(g["bin"][1]), float(g["bin"][2])
    tr = oracle.mesh_exhaustive_forward(g["verts"], g["faces"], g["colors"], g["scan_points"],
                                        g["laser_points"], None, None, g["vis_s"], g["vis_l"],
                                        nb, bw, bo)
    assert rel(tr, g["transient"]) < 1e-5
    vg, mg = oracle.mesh_exhaustive_grad(g["verts"], g["faces"], g["colors"], g["scan_points"],
                                         g["laser_points"], None, None, g["vis_s"], g["vis_l"],
                                         nb, bw, bo, g["transient_grad"].astype(np.float64))
    assert rel(vg, g["verts_grad"]) < 1e-4
    assert rel(mg, g["colors_grad"]) < 1e-5


def test_volume_confocal_golden():
    g = load("volume_confocal")
    T, bw, bo = int(g["bin"][0]), float(g["bin"][1]), float(g["bin"][2])
    tr = oracle.volume_confocal_forward(g["volume"], g["mp"], T, g["origin"], g["size"], bw, bo)
    assert rel(tr, g["transient"]) < 1e-5
    gv = oracle.volume_confocal_transposed(g["transient_grad"], g["volume"].shape, g["mp"],
                                           g["origin"], g["size"], bw, bo)
    assert rel(gv, g["grad_volume"]) < 1e-5
    gm = oracle.volume_confocal_grad_mp(g["volume"], g["mp"], g["transient_grad"], g["origin"],
                                        g["size"], bw, bo)
    assert rel(gm, g["grad_mp"]) < 1e-5


def test_volume_exhaustive_golden():
    g = load("volume_exhaustive")
    T, bw, bo = int(g["bin"][0]), float(g["bin"][1]), float(g["bin"][2])
    tr = oracle.volume_exhaustive_forward(g["volume"][0], g["scan_points"][0],
                                          g["laser_points"][0], T, g["start"], g["end"], bw, bo)
    assert rel(tr, g["transient"][0]) < 1e-5


def test_backprojection_golden():
    g = load("backprojection")
    shape = tuple(int(x) for x in g["shape"])
    v = oracle.bp_confocal_velten(g["transient_confocal"][0], g["scan_points"][0],
                                  g["scan_origin"][0], shape, g["start"], g["end"], 0.02, 0.0)
    assert rel(v, g["volume_confocal"][0]) < 1e-5
    v = oracle.bp_exhaustive_velten(g["transient_exhaustive"][0], g["scan_points"][0],
                                    g["laser_points"][0], None, None, shape, g["start"], g["end"],
                                    0.01, 0.0)
    assert rel(v, g["volume_exhaustive"][0]) < 1e-5
    v = oracle.bp_exhaustive_arellano(g["transient_exhaustive"][0], g["scan_points"][0].T,
                                      g["laser_points"][0].T, None, None, shape, g["start"],
                                      g["end"], 0.01, 0.0)
    assert rel(v, g["volume_arellano"][0]) < 1e-5


def test_rbf_golden():
    g = load("rbf2volume")
    shape = tuple(int(x) for x in g["shape"])
    vol = oracle.rbf2volume_forward(g["rbf"][0], shape, g["start"], g["end"])
    assert rel(vol, g["volume"][0]) < 1e-5
    rg = oracle.rbf2volume_grad(g["rbf"][0], g["volume"][0], g["volume_grad"][0], g["start"],
                                g["end"])
    assert rel(rg, g["rbf_grad"][0]) < 1e-5


def test_visibility_bvh_equals_brute_force():
    from totri_gb300 import scenes
    for seed in (0, 3):
        s = scenes.confocal_small(seed=seed)
        v, f, sp = s["verts"][0].numpy(), s["faces"][0].numpy(), s["scan_points"][0].numpy()
        assert np.array_equal(oracle.mesh_visibility(v, f, sp),
                              oracle.mesh_visibility(v, f, sp, bvh=True))


def test_visibility_occluder_blocks():
    # a large quad between the wall and a small triangle hides it from every wall point
    verts = np.array([[-0.05, -0.05, 1.0], [0.05, -0.05, 1.0], [0.0, 0.05, 1.0],
                      [-2, -2, 0.5], [2, -2, 0.5], [2, 2, 0.5], [-2, 2, 0.5]], np.float32)
    faces = np.array([[0, 1, 2], [3, 4, 5], [3, 5, 6]])
    pts = np.array([[0.0, 0.0, 0.0], [0.3, 0.1, 0.0]], np.float32)
    vis = oracle.mesh_visibility(verts, faces, pts)
    assert vis[:, 0].sum() == 0 and vis[:, 1:].sum() == 4
    faces_pad = np.array([[0, 1, 2], [3, -1, 5], [3, 5, 6]])  # list ends at face 1
    vis = oracle.mesh_visibility(verts, faces_pad, pts)
    assert vis[:, 0].sum() == 2 and vis[:, 1:].sum() == 0
    assert oracle.mesh_count_faces(faces_pad, 7) == 1


def test_rbf_gradient_matches_fp64_central_differences():
    """RBF gradient formula vs central differences of the FP64 forward (h = 1e-4)."""
    rng = np.random.default_rng(9)
    N = 5
    rbf = np.concatenate([rng.uniform(-0.3, 0.3, (N, 3)) + np.array([0, 0, 1.0]),
                          rng.uniform(0.1, 0.2, (N, 1)), rng.random((N, 1))], 1)
    rbf = rbf.astype(np.float32).astype(np.float64)
    shape, st, en = (6, 5, 4), (-0.5, -0.5, 0.5), (0.5, 0.5, 1.5)
    w = rng.standard_normal((2,) + shape)
    vol = oracle.rbf2volume_forward(rbf, shape, st, en)
    g = oracle.rbf2volume_grad(rbf, vol, w, st, en)
    for i in range(N):
        for c in range(5):
            rp, rm = rbf.copy(), rbf.copy()
            rp[i, c] = np.float32(rbf[i, c] + 1e-4)
            rm[i, c] = np.float32(rbf[i, c] - 1e-4)
            h = float(rp[i, c]) - float(rm[i, c])
            fd = ((w * oracle.rbf2volume_forward(rp, shape, st, en)).sum() -
                  (w * oracle.rbf2volume_forward(rm, shape, st, en)).sum()) / h
            assert abs(fd - g[i, c]) <= 1e-3 * max(1.0, abs(g[i, c])), (i, c, fd, g[i, c])


@pytest.mark.parametrize("kind", ["confocal", "exhaustive"])
def test_mesh_gradient_matches_fp64_central_differences(kind):
    """The restated gradient formula against central differences of the FP64
    forward with the visibility masks held fixed (h = 1e-5; vertices whose
    perturbation moves a bin boundary or the vertex order are skipped by
    comparing only where both one-sided slopes agree)."""
    from totri_gb300 import scenes
    s = scenes.confocal_small(seed=2)
    v, f, c = s["verts"][0].numpy(), s["faces"][0].numpy(), s["colors"][0].numpy()
    sp = scenes.wall_grid(6)[0].numpy()
    lp = scenes.wall_grid(2)[0].numpy()
    nb, bw = 300, 0.02
    vis_s = oracle.mesh_visibility(v, f, sp)
    vis_l = oracle.mesh_visibility(v, f, lp)
    w = np.random.default_rng(5).standard_normal(
        (nb, sp.shape[0]) if kind == "confocal" else (nb, sp.shape[0], lp.shape[0]))

    def loss(vv):
        if kind == "confocal":
            t = oracle.mesh_confocal_forward(vv, f, c, sp, None, vis_s, nb, bw, 0.0)
        else:
            t = oracle.mesh_exhaustive_forward(vv, f, c, sp, lp, None, None, vis_s, vis_l, nb, bw,
                                               0.0)
        return float((w * t).sum())

    if kind == "confocal":
        g, _ = oracle.mesh_confocal_grad(v, f, c, sp, None, vis_s, nb, bw, 0.0, w)
    else:
        g, _ = oracle.mesh_exhaustive_grad(v, f, c, sp, lp, None, None, vis_s, vis_l, nb, bw, 0.0,
                                           w)
    rng = np.random.default_rng(6)
    checked = 0
    for vi in rng.choice(v.shape[0], 24, replace=False):
        for a in range(3):
            vp, vm = v.copy(), v.copy()
            vp[vi, a] = np.float32(v[vi, a] + 1e-5)
            vm[vi, a] = np.float32(v[vi, a] - 1e-5)
            hp, hm = float(vp[vi, a]) - float(v[vi, a]), float(v[vi, a]) - float(vm[vi, a])
            l0, lp_, lm = loss(v), loss(vp), loss(vm)
            sp_, sm_ = (lp_ - l0) / hp, (l0 - lm) / hm
            scale = max(abs(sp_), abs(sm_), 1e-3)
            if abs(sp_ - sm_) > 0.005 * scale:  # kink: a discrete decision moved
                continue
            fd = (lp_ - lm) / (hp + hm)
            assert abs(fd - g[vi, a]) <= 1e-3 * scale + 1e-6, (vi, a, fd, g[vi, a])
            checked += 1
    assert checked >= 30
