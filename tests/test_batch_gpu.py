"""Visibility traversal modes, the batched graph-captured renderer and the
tile autotuner on the GPU.

Bars: visibility bits equal across the warp-packet walk, the per-lane walk and
brute force (and the oracle); batched results equal the per-mesh C-ABI calls
up to the FP32 reordering of shared-memory atomics (rel-L2 1e-6 forward,
1e-5 gradients).
"""
import json

import numpy as np
import pytest
import torch

import oracle
from totri_gb300 import autotune, scenes
from totri_gb300.batch import BatchedMeshRenderer
from totri_gb300.data.util import merge_meshes
from totri_gb300.totri_cpp import render as R
from totri_gb300.types import BinDef

from mesh_util import rel_l2, unpack_mask

pytestmark = pytest.mark.gpu


def _occluded_scene():
    """Two jittered spheres, the second half hidden behind the first, plus a
    small third one inside the line of sight: heavy occlusion for the walk."""
    a = scenes.jittered_sphere(3, 11, radius=0.25, center=(0.0, 0.0, 0.8))
    b = scenes.jittered_sphere(3, 12, radius=0.3, center=(0.15, 0.1, 1.3))
    c = scenes.jittered_sphere(2, 13, radius=0.08, center=(-0.2, 0.0, 0.45))
    verts, faces = merge_meshes([a[0][0], b[0][0], c[0][0]], [a[1][0], b[1][0], c[1][0]])
    return verts[None].contiguous(), faces[None].contiguous(), scenes.wall_grid(24)


def _masks(verts, faces, sp, mode=0, brute=False):
    autotune.set_tile("mesh.visibility.mode", mode)
    try:
        m = R.mesh_visibility(verts, faces, sp, brute_force=brute)[0].cpu().numpy()
    finally:
        autotune.set_tile("mesh.visibility.mode", 0)
    return unpack_mask(m, faces.shape[1])


def test_visibility_modes_agree_under_occlusion(cuda_lib):
    verts, faces, sp = _occluded_scene()
    d = [t.cuda() for t in (verts, faces, sp)]
    ref = oracle.mesh_visibility(verts[0].numpy(), faces[0].numpy(), sp[0].numpy())
    for mode in (0, 1, 2, 3, 4, 5, 6, 7):  # 0: the built-in choice
        assert np.array_equal(_masks(*d, mode=mode), ref), mode
    assert np.array_equal(_masks(*d, brute=True), ref)
    assert 0.05 < ref.mean() < 0.5


def test_visibility_modes_agree_full_size(cuda_lib):
    s = scenes.confocal_differentiable()
    d = [s[k].cuda() for k in ("verts", "faces", "scan_points")]
    ray = _masks(*d, mode=1)
    for mode in (0, 2, 3, 5, 6, 7):
        assert np.array_equal(_masks(*d, mode=mode), ray), mode


def _meshes():
    out = []
    for lvl, seed, c in ((2, 21, (0.0, 0.0, 1.0)), (3, 22, (0.1, -0.1, 1.2)),
                         (3, 23, (-0.1, 0.05, 0.9))):
        v, f, m = scenes.displaced_sphere(lvl, seed, center=c)
        out.append((v[0], f[0], m[0]))
    return out


@pytest.mark.parametrize("graph", [True, False])
def test_batched_confocal_matches_per_mesh_calls(cuda_lib, tmp_path, monkeypatch, graph):
    monkeypatch.setenv("TOTRI_TUNE_CACHE", str(tmp_path / "tune.json"))
    meshes = _meshes()
    sp = scenes.wall_grid(24)[0].cuda()
    bd = BinDef(0.01, 0.0, 400)
    br = BatchedMeshRenderer([tuple(t.cuda() for t in m) for m in meshes], sp, bd,
                             graph=graph, tune=True)
    g = torch.Generator(device="cuda").manual_seed(0)
    tg = torch.randn(br.transient.shape, device="cuda", generator=g)
    row = {i: r for r, i in enumerate(br.wave_order())}
    for rep in range(2):  # replays reuse the captured buffers
        br.step(tg)
        tr = br.transient
        grads = br.mesh_grads()
        for i, (v, f, m) in enumerate(meshes):
            v, f, m = v[None].cuda(), f[None].cuda(), m[None].cuda()
            empty = torch.empty((1, 0, 3), device="cuda")
            out = torch.empty((1, bd.num, sp.shape[0]), device="cuda")
            R.mesh_confocal_forward(v, f, m, sp[None], empty, out, bd.width, bd.offset, 0)
            assert rel_l2(tr[row[i]].cpu().numpy(), out[0].cpu().numpy()) < 1e-6
            vg, mg = torch.empty_like(v), torch.empty_like(m)
            R.mesh_confocal_grad_verts(v, f, m, sp[None], empty, tg[row[i]:row[i] + 1].contiguous(),
                                       vg, mg, bd.width, bd.offset, 0)
            assert rel_l2(grads[i][0].cpu().numpy(), vg[0].cpu().numpy()) < 1e-5
            assert rel_l2(grads[i][1].cpu().numpy(), mg[0].cpu().numpy()) < 1e-5
    ref = tr.clone()
    fwd = br.forward()
    assert rel_l2(fwd.cpu().numpy(), ref.cpu().numpy()) < 1e-6


def test_batched_exhaustive_matches_per_mesh_calls(cuda_lib, tmp_path, monkeypatch):
    monkeypatch.setenv("TOTRI_TUNE_CACHE", str(tmp_path / "tune.json"))
    meshes = _meshes()[:2]
    sp = scenes.wall_grid(6)[0].cuda()
    lp = (scenes.wall_grid(3)[0] * 0.8).cuda()
    bd = BinDef(0.02, 0.0, 300)
    br = BatchedMeshRenderer([tuple(t.cuda() for t in m) for m in meshes], sp, bd,
                             laser_points=lp)
    tg = torch.randn(br.transient.shape, device="cuda")
    br.step(tg)
    tr = br.transient
    row = {i: r for r, i in enumerate(br.wave_order())}
    grads = br.mesh_grads()
    for i, (v, f, m) in enumerate(meshes):
        v, f, m = v[None].cuda(), f[None].cuda(), m[None].cuda()
        so = torch.empty((1, 0, 3), device="cuda")
        lo = torch.empty((1, 0, 3), device="cuda")
        out = torch.empty((1, bd.num, sp.shape[0], lp.shape[0]), device="cuda")
        R.mesh_exhaustive_forward(v, f, m, sp[None], lp[None], so, lo, out, bd.width,
                                  bd.offset, 0)
        assert rel_l2(tr[row[i]].cpu().numpy(), out[0].cpu().numpy()) < 1e-6
        vg, mg = torch.empty_like(v), torch.empty_like(m)
        R.mesh_exhaustive_grad_verts(v, f, m, sp[None], lp[None], so, lo,
                                     tg[row[i]:row[i] + 1].contiguous(), vg, mg, bd.width,
                                     bd.offset, 0)
        assert rel_l2(grads[i][0].cpu().numpy(), vg[0].cpu().numpy()) < 1e-5
        assert rel_l2(grads[i][1].cpu().numpy(), mg[0].cpu().numpy()) < 1e-5


def test_energy_head_in_waves_matches_per_mesh_calls(cuda_lib, tmp_path, monkeypatch):
    """A budget of two transients per wave splits three meshes into two waves
    captured in one graph; loss 0.5 ||tr||^2 and its gradient per mesh match
    plain calls with transient_grad = transient."""
    monkeypatch.setenv("TOTRI_TUNE_CACHE", str(tmp_path / "tune.json"))
    meshes = _meshes()
    sp = scenes.wall_grid(16)[0].cuda()
    bd = BinDef(0.01, 0.0, 300)
    budget = 2 * 4 * bd.num * sp.shape[0] + 1
    br = BatchedMeshRenderer([tuple(t.cuda() for t in m) for m in meshes], sp, bd,
                             grad="energy", hbm_budget=budget)
    assert len(br.waves) == 2
    for _ in range(2):
        loss = br.step().clone()
        grads = br.mesh_grads()
        for i, (v, f, m) in enumerate(meshes):
            v, f, m = v[None].cuda(), f[None].cuda(), m[None].cuda()
            empty = torch.empty((1, 0, 3), device="cuda")
            out = torch.empty((1, bd.num, sp.shape[0]), device="cuda")
            R.mesh_confocal_forward(v, f, m, sp[None], empty, out, bd.width, bd.offset, 0)
            ref = 0.5 * float((out.double() ** 2).sum())
            assert abs(float(loss[i]) - ref) <= 1e-5 * ref
            vg, mg = torch.empty_like(v), torch.empty_like(m)
            R.mesh_confocal_grad_verts(v, f, m, sp[None], empty, out, vg, mg, bd.width,
                                       bd.offset, 0)
            assert rel_l2(grads[i][0].cpu().numpy(), vg[0].cpu().numpy()) < 1e-5
            assert rel_l2(grads[i][1].cpu().numpy(), mg[0].cpu().numpy()) < 1e-5


def _fill_normal(n, seed):
    import ctypes
    from totri_gb300 import _lib
    out = torch.empty(n, device="cuda")
    _lib.check(_lib.load().totri_fill_normal(ctypes.c_void_p(out.data_ptr()), n, seed,
                                             _lib.stream_of(out.device)))
    return out


def test_fill_normal_is_counter_based_and_standard(cuda_lib):
    """Element i depends on (seed, i) only: a prefix of a longer fill is the
    shorter fill, seeds differ, and the values are standard normal."""
    a = _fill_normal(1 << 20, 7)
    assert torch.equal(_fill_normal(1000, 7), a[:1000])
    assert not torch.equal(_fill_normal(1000, 8), a[:1000])
    x = a.double()
    assert abs(float(x.mean())) < 5e-3 and abs(float(x.std()) - 1.0) < 5e-3
    assert float((x.abs() > 3.0).double().mean()) == pytest.approx(0.0027, abs=5e-4)
    assert torch.isfinite(a).all()


def test_normal_head_in_waves_matches_per_mesh_calls(cuda_lib, tmp_path, monkeypatch):
    """The seeded N(0, 1) head: three meshes in two waves; each mesh's
    transient gradient is the field drawn from seed + its index, so plain calls
    with the same fill give the same loss <tr, g> and gradients."""
    monkeypatch.setenv("TOTRI_TUNE_CACHE", str(tmp_path / "tune.json"))
    meshes = _meshes()
    sp = scenes.wall_grid(16)[0].cuda()
    bd = BinDef(0.01, 0.0, 300)
    budget = 2 * 2 * 4 * bd.num * sp.shape[0] + 1  # two meshes (transient + gradient)
    br = BatchedMeshRenderer([tuple(t.cuda() for t in m) for m in meshes], sp, bd,
                             grad="normal", hbm_budget=budget, normal_seed=40)
    assert len(br.waves) == 2
    loss = br.step().clone()
    grads = br.mesh_grads()
    for i, (v, f, m) in enumerate(meshes):
        v, f, m = v[None].cuda(), f[None].cuda(), m[None].cuda()
        empty = torch.empty((1, 0, 3), device="cuda")
        out = torch.empty((1, bd.num, sp.shape[0]), device="cuda")
        R.mesh_confocal_forward(v, f, m, sp[None], empty, out, bd.width, bd.offset, 0)
        tg = _fill_normal(out.numel(), 40 + i).reshape(out.shape)
        ref = float((out.double() * tg.double()).sum())
        assert abs(float(loss[i]) - ref) <= 1e-5 * float((out.double() * tg.double()).abs().sum())
        vg, mg = torch.empty_like(v), torch.empty_like(m)
        R.mesh_confocal_grad_verts(v, f, m, sp[None], empty, tg, vg, mg, bd.width, bd.offset, 0)
        assert rel_l2(grads[i][0].cpu().numpy(), vg[0].cpu().numpy()) < 1e-5
        assert rel_l2(grads[i][1].cpu().numpy(), mg[0].cpu().numpy()) < 1e-5


def test_autotune_sweeps_then_reads_cache(cuda_lib, tmp_path, monkeypatch):
    path = tmp_path / "tune.json"
    monkeypatch.setenv("TOTRI_TUNE_CACHE", str(path))
    s = scenes.confocal_small()
    d = {k: s[k].cuda() for k in ("verts", "faces", "colors", "scan_points")}
    bd = s["bin_def"]
    out = torch.empty((1, bd.num, d["scan_points"].shape[1]), device="cuda")
    empty = torch.empty((1, 0, 3), device="cuda")

    def run():
        R.mesh_confocal_forward(d["verts"], d["faces"], d["colors"], d["scan_points"], empty,
                                out, bd.width, bd.offset, 0)

    key = "mesh.confocal.splat.ts"
    try:
        best, times = autotune.tune(key, run, "small")
        assert best in autotune.CANDIDATES[key]
        assert len(times) >= 2 and best == min(times, key=times.get)
        assert autotune.get_tile(key) == best
        cached = json.loads(path.read_text())
        assert list(cached.values())[0]["best"] == best
        autotune.set_tile(key, 0)
        again, _ = autotune.tune(key, run, "small")
        assert again == best and autotune.get_tile(key) == best
        ref = out.clone()
        autotune.set_tile(key, 0)
        run()
        assert rel_l2(out.cpu().numpy(), ref.cpu().numpy()) < 1e-6
    finally:
        autotune.set_tile(key, 0)
