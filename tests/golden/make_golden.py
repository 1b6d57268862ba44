"""Generates the golden vectors in tests/golden/ from the reference's own code.

The reference's kernel sources are compiled for the CPU by oracle/ref_harness.py
(which needs the reference tree) and run on small seeded inputs; inputs and
reference outputs are stored as compressed .npz files. The mesh programs trace
visibility through OptiX, whose intersection code is closed, so their
visibility masks are an input here (taken from the oracle's FP32 ray test and
stored alongside).

Run: python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from oracle import ref_harness as RH  # noqa: E402
from totri_gb300 import scenes  # noqa: E402


def wall(n, g=None, random=False, count=None):
    if random:
        return np.stack([g.uniform(-1, 1, count), g.uniform(-1, 1, count), np.zeros(count)],
                        1).astype(np.float32)
    return scenes.wall_grid(n)[0].numpy()


def save(name, **arrays):
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **arrays)


def mesh_goldens():
    s = scenes.confocal_small(seed=0)
    v = s["verts"][0].numpy()
    f = s["faces"][0].numpy()
    c = s["colors"][0].numpy()
    sp = wall(16)
    nb, bw, bo = 512, 0.01, 0.0
    vis = oracle.mesh_visibility(v, f, sp)
    tr = RH.mesh_confocal_forward(v, f, c, sp, None, vis, nb, bw, bo)
    # gradient on an 8x8 sub-grid; float16-exact incoming gradient (stored as float16)
    sub = np.arange(0, 256, 2)[:64]
    tg = np.random.default_rng(10).standard_normal((nb, sub.size)).astype(np.float16)
    vg, mg = RH.mesh_confocal_grad(v, f, c, sp[sub], None, vis[sub], nb, bw, bo,
                                   tg.astype(np.float32))
    so = np.tile(np.array([[0.3, -0.2, -1.0]], np.float32), (sp.shape[0], 1))
    tr_o = RH.mesh_confocal_forward(v, f, c, sp, so, vis, 1024, bw, bo)
    save("mesh_confocal", verts=v, faces=f, colors=c, scan_points=sp, vis=vis,
         bin=np.array([nb, bw, bo]), transient=tr, grad_points=sub, transient_grad=tg,
         verts_grad=vg, colors_grad=mg, scan_origin=so, transient_origin=tr_o)

    s1 = scenes.confocal_small(seed=1)
    v1 = s1["verts"][0].numpy()
    c1 = s1["colors"][0].numpy()
    sp1, lp1 = wall(6), wall(2)
    nb1, bw1 = 256, 0.02
    vis_s = oracle.mesh_visibility(v1, f, sp1)
    vis_l = oracle.mesh_visibility(v1, f, lp1)
    tr1 = RH.mesh_exhaustive_forward(v1, f, c1, sp1, lp1, None, None, vis_s, vis_l, nb1, bw1,
                                     0.0)
    tg1 = np.random.default_rng(11).standard_normal(tr1.shape).astype(np.float16)
    vg1, mg1 = RH.mesh_exhaustive_grad(v1, f, c1, sp1, lp1, None, None, vis_s, vis_l, nb1, bw1,
                                       0.0, tg1.astype(np.float32))
    save("mesh_exhaustive", verts=v1, faces=f, colors=c1, scan_points=sp1, laser_points=lp1,
         vis_s=vis_s, vis_l=vis_l, bin=np.array([nb1, bw1, 0.0]), transient=tr1,
         transient_grad=tg1, verts_grad=vg1, colors_grad=mg1)


def volume_goldens():
    g = np.random.default_rng(20)
    X = Y = Z = 12
    N, T = 40, 96
    vol = ((g.random((X, Y, Z)) < 0.1) * g.random((X, Y, Z))).astype(np.float32)
    mp = wall(0, g, True, N).T.copy()
    org, size, bw, bo = np.array([-0.5, -0.5, 0.5]), np.array([1.0, 1.0, 1.0]), 0.03, 0.0
    tr = RH.volume_confocal_forward(vol, mp, T, org, size, bw, bo)
    tg = g.standard_normal((N, T)).astype(np.float32)
    gv = RH.volume_confocal_grad_volume(tg, (X, Y, Z), mp, org, size, bw, bo)
    gm = RH.volume_confocal_grad_mp(vol, mp, tg, org, size, bw, bo)
    save("volume_confocal", volume=vol, mp=mp, origin=org, size=size,
         bin=np.array([T, bw, bo]), transient=tr, transient_grad=tg, grad_volume=gv,
         grad_mp=gm)

    D, H, W, S, L, T2 = 6, 5, 7, 9, 4, 64
    v4 = ((g.random((1, D, H, W)) < 0.3) * g.random((1, D, H, W))).astype(np.float32)
    sp = wall(0, g, True, S).T[None].copy()
    lp = wall(0, g, True, L).T[None].copy()
    st, en, bw2 = np.array([-0.5, -0.5, 0.5]), np.array([0.5, 0.5, 1.5]), 0.05
    tr2 = RH.volume_exhaustive_forward(v4, sp, lp, T2, st, en, bw2, 0.0)
    save("volume_exhaustive", volume=v4, scan_points=sp, laser_points=lp, start=st, end=en,
         bin=np.array([T2, bw2, 0.0]), transient=tr2)


def backprojection_goldens():
    g = np.random.default_rng(30)
    S, T, L = 50, 128, 6
    D, H, W = 8, 9, 10
    st, en = np.array([-0.5, -0.5, 0.5]), np.array([0.5, 0.5, 1.5])
    trc = g.random((1, T, S)).astype(np.float32)
    sp = wall(0, g, True, S)[None]
    so = np.tile(np.array([[0.2, 0.1, -1.0]], np.float32), (S, 1))[None]
    vc = RH.bp_confocal_velten(trc, sp, so, (D, H, W), st, en, 0.02, 0.0)
    tre = g.random((1, T, S, L)).astype(np.float32)
    lp = wall(0, g, True, L)[None]
    ve = RH.bp_exhaustive_velten(tre, sp, lp, (D, H, W), st, en, 0.01, 0.0)
    spa = np.ascontiguousarray(sp.transpose(0, 2, 1))
    lpa = np.ascontiguousarray(lp.transpose(0, 2, 1))
    va = RH.bp_exhaustive_arellano(tre, spa, lpa, (D, H, W), st, en, 0.01, 0.0)
    save("backprojection", transient_confocal=trc, scan_points=sp, scan_origin=so,
         transient_exhaustive=tre, laser_points=lp, start=st, end=en, shape=np.array([D, H, W]),
         volume_confocal=vc, volume_exhaustive=ve, volume_arellano=va)


def rbf_goldens():
    g = np.random.default_rng(40)
    N = 7
    rbf = np.concatenate([g.uniform(-0.5, 0.5, (N, 3)) + np.array([0, 0, 1.0]),
                          g.uniform(0.05, 0.2, (N, 1)), g.random((N, 2))], 1)[None]
    rbf = rbf.astype(np.float32)
    shape = (6, 5, 4)
    st, en = np.array([-0.5, -0.5, 0.5]), np.array([0.5, 0.5, 1.5])
    vol = RH.rbf2volume_forward(rbf, shape, st, en)
    vg = g.standard_normal(vol.shape).astype(np.float32)
    rg = RH.rbf2volume_grad(rbf, vol, vg, st, en)
    save("rbf2volume", rbf=rbf, shape=np.array(shape), start=st, end=en, volume=vol,
         volume_grad=vg, rbf_grad=rg)


if __name__ == "__main__":
    RH.build()
    mesh_goldens()
    volume_goldens()
    backprojection_goldens()
    rbf_goldens()
    for f in sorted(os.listdir(HERE)):
        if f.endswith(".npz"):
            print(f, os.path.getsize(os.path.join(HERE, f)))
