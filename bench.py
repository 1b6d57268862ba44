#!/usr/bin/env python
"""Benchmark of the differentiable confocal mesh render (forward + backward).

Workload (the headline differentiable configuration): level-5 icosphere
(20,480 faces) with 0.05 m low-frequency radial displacement, 64x64 confocal
scan on [-1,1]^2, 1,024 bins of 0.005 m, visibility on, MSE loss against a
target transient rendered from a second seeded mesh; gradients with respect to
vertex positions and albedo. One step = forward render + loss + backward
through ``totri_gb300.render.MeshRenderConfocal``. Unit of work: one
(scan point, face) pair; 83,886,080 pairs per step.

Prints one JSON line. ``--impl reference`` times the CPU restatement of the
reference algorithm (oracle/) on the host cores instead (the reference's
mesh path needs the OptiX SDK and cannot be built).
"""
import argparse
import ctypes
import json
import math
import os
import subprocess
import sys
import tempfile
import time

import numpy as np
import torch

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

METRIC = "mesh fwd+bwd scanpt·tri pairs/s"
UNIT = "pairs/s"
WORKLOAD = ("confocal mesh fwd+bwd: level-5 icosphere 20480 faces, radial SH displacement "
            "0.05 m, 64x64 scan, 1024 bins x 0.005 m, visibility on, MSE vs target mesh")
# FLOP model per (scan point, face) pair: add/mul = 1, FMA = 2, div/sqrt/exp = 1.
FLOP_SPLAT = 116.0       # forward geometry, alpha, bins
FLOP_GRAD = 190.0        # backward recomputation + alpha log-derivative
FLOP_PER_SEG_FWD = 10.0  # per bin segment of the tent (forward)
FLOP_PER_SEG_BWD = 60.0  # per bin segment (backward)


def bench_config(faces, scan_points, bins, world):
    """The `config` of both arms' JSON lines (the same dict for the same run)."""
    return {"workload": WORKLOAD, "faces": faces, "scan_points": scan_points, "bins": bins,
            "pairs_per_step": faces * scan_points,
            "parallelism": "replicas" if world > 1 else "single",
            "l2": "GPU arm: flushed between timed steps (256 MiB memset); CPU arm: each step "
                  "is the whole workload"}


def flop_visibility(num_faces):
    """Per-ray BVH visibility model: 2 box tests x 20 per level + 4 triangle tests x 36."""
    return 40.0 * math.ceil(math.log2(max(num_faces, 2))) + 144.0


# The secondary, batched and serving measurements are single-GPU figures: they
# run on one-process runs only, so a multi-rank run holds its GPUs just for the
# headline step.


def parse_args():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=20)
    p.add_argument("--warmup", type=int, default=5)
    p.add_argument("--impl", choices=["gb300", "reference"], default="gb300")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-secondary", action="store_true")
    p.add_argument("--no-batched", action="store_true")
    p.add_argument("--no-serve", action="store_true")
    p.add_argument("--e2e-steps", type=int, default=None)
    return p.parse_args()


# ---------------------------------------------------------------------------
# Distributed helpers (one process per GPU; replicas, no data-path collective).

def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1 and not torch.distributed.is_initialized():
        backend = "nccl" if torch.cuda.is_available() else "gloo"
        torch.distributed.init_process_group(backend)
    return world, rank, local


def barrier(world):
    if world > 1:
        torch.distributed.barrier()


def max_over_ranks(x, world, device):
    if world == 1:
        return x
    t = torch.tensor([x], dtype=torch.float64, device=device)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


# ---------------------------------------------------------------------------
# Clock sampling during the timed region.

class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.out = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.FIELDS,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=self.out, stderr=subprocess.DEVNULL)
        except (OSError, ValueError):
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.out.close()
        rows = []
        with open(self.path) as f:
            for line in f:
                parts = [x.strip() for x in line.split(",")]
                if len(parts) >= 9:
                    rows.append(parts)
        os.unlink(self.path)
        if not rows:
            return None
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({n for r in rows for n, v in zip(names, r[5:9]) if v == "Active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


# ---------------------------------------------------------------------------
# Workload.

def make_workload(device):
    from totri_gb300 import scenes
    from totri_gb300.render import MeshRenderConfocal
    s = scenes.confocal_differentiable()
    bd = s["bin_def"]
    w = {k: (v.to(device) if torch.is_tensor(v) else v) for k, v in s.items()}
    with torch.no_grad():
        target = MeshRenderConfocal.apply(w["target_verts"], w["faces"], w["scan_points"], bd,
                                          w["target_colors"])
    w["target"] = target.contiguous()
    w["host"] = s
    return w


def step(w, verts, colors, faces, scan_points, target):
    from totri_gb300.render import MeshRenderConfocal
    verts = verts.detach().requires_grad_(True)
    colors = colors.detach().requires_grad_(True)
    tr = MeshRenderConfocal.apply(verts, faces, scan_points, w["bin_def"], colors)
    loss = torch.mean((tr - target) ** 2)
    loss.backward()
    return loss, verts.grad, colors.grad


def mean_segments(w, device, stride=8):
    """b-bar: mean bin count of the tent per (scan point, face) pair, 0 for pairs
    that are occluded or out of range (computed on a 1/stride scan subset)."""
    from totri_gb300.totri_cpp import render as R
    verts, faces, sp = w["verts"], w["faces"], w["scan_points"][:, ::stride].contiguous()
    bd = w["bin_def"]
    F = faces.shape[1]
    mask = R.mesh_visibility(verts, faces, sp)[0]
    bits = ((mask.unsqueeze(-1) >> torch.arange(32, device=device, dtype=torch.int32)) & 1)
    vis = bits.reshape(mask.shape[0], -1)[:, :F].bool()
    tri = verts[0][faces[0].long()]                         # [F, 3, 3]
    d = torch.linalg.norm(tri[None] - sp[0][:, None, None, :], dim=-1)  # [S', F, 3]
    c = (2.0 * d - bd.offset) / bd.width
    lo = c.min(dim=-1).values.floor()
    hi = c.max(dim=-1).values.floor().clamp(max=bd.num - 1)
    seg = (hi - lo.clamp(min=0) + 1).clamp(min=0)
    seg = torch.where(vis & (lo < bd.num), seg, torch.zeros_like(seg))
    return float(seg.mean())


def _timed(fn, flush, reps, warmup=3):
    """Mean device milliseconds of fn() over reps calls (L2 flushed between calls)."""
    stream = torch.cuda.current_stream()
    for _ in range(warmup):
        fn()
    total = 0.0
    for _ in range(reps):
        flush.zero_()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        fn()
        e1.record(stream)
        e1.synchronize()
        total += e0.elapsed_time(e1)
    return total / reps


def pose_fit_rate(device, iterations=50):
    """(iterations, device-timed ms) of one rigid pose fit on the plain
    confocal workload (320 faces, 32x32 scan, 512 bins), target offset by
    (3, -2, 4) cm."""
    from totri_gb300 import scenes
    from totri_gb300.fitting import PoseFitting
    from totri_gb300.render import MeshRenderConfocal
    s = scenes.confocal_small(seed=2)
    v, f, sp = (s[k][0].to(device) for k in ("verts", "faces", "scan_points"))
    bd = s["bin_def"]
    with torch.no_grad():
        target = MeshRenderConfocal.apply(
            (v + torch.tensor((0.03, -0.02, 0.04), device=device))[None], f[None], sp[None],
            bd)[0]
    PoseFitting(bd).fit(target, sp, [v], [f], num_iter=3, stop_loss=None)
    stream = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    PoseFitting(bd).fit(target, sp, [v], [f], num_iter=iterations, stop_loss=None)
    e1.record(stream)
    e1.synchronize()
    return iterations, e0.elapsed_time(e1)


def secondary_metrics(device, flush, reps=5):
    """The other throughputs named by the headline metric, on the 128^3 workloads:
    Velten backprojection (128^3 voxels x 128x128 scan points x 1024 bins),
    volume render + exact adjoint, RBF splat + gradient (4096 Gaussians),
    marching cubes + gradient on that RBF volume, a pose fit, f-k
    migration and a shaded 512x512 preview of a 20,480-face mesh."""
    from totri_gb300 import scenes
    from totri_gb300.totri_cpp import reconstruct as K
    from totri_gb300.totri_cpp import render as R
    from totri_gb300.totri_cpp import util as U
    s = scenes.volume_scene()
    vd, bd = s["volume_def"], s["bin_def"]
    sp = s["scan_points"].to(device)
    S = sp.shape[1]
    nvox = int(np.prod(vd.resolution))
    tr = torch.rand((1, bd.num, S), device=device)
    vol_out = torch.empty((1,) + tuple(vd.resolution), device=device)
    empty = torch.empty_like(sp[:, :0])
    ms_bp = _timed(lambda: K.backprojection_confocal_velten_forward(
        tr, sp, empty, vol_out, vd.start, vd.end, bd.width, bd.offset), flush, reps)
    vol = s["volume"].to(device)
    mp = sp[0].T.contiguous()
    size = tuple(e - a for a, e in zip(vd.start, vd.end))
    trv = torch.empty((S, bd.num), device=device)
    adj = torch.empty_like(vol)
    ms_vf = _timed(lambda: R.volume_confocal_forward(vol, mp, trv, vd.start, size, bd.width,
                                                     bd.offset), flush, reps)
    ms_va = _timed(lambda: R.volume_confocal_adjoint(adj, mp, trv, vd.start, size, bd.width,
                                                     bd.offset), flush, 2)
    rbf = scenes.rbf_set(4096, seed=5).to(device)
    rvol = torch.empty((1, 2) + tuple(vd.resolution), device=device)
    ms_rf = _timed(lambda: U.rbf2volume_gaussian_forward(rbf, rvol, vd.start, vd.end), flush,
                   reps)
    rgrad = torch.zeros_like(rbf)
    vg = torch.randn_like(rvol)
    ms_rg = _timed(lambda: U.rbf2volume_gaussian_grad(rbf, rvol, vg, rgrad, vd.start, vd.end),
                   flush, reps)
    from totri_gb300.util.marching_cubes import marching_cubes, marching_cubes_grad
    U.rbf2volume_gaussian_forward(rbf, rvol, vd.start, vd.end)
    mc_out = {}

    def mc_forward():
        mc_out["r"] = marching_cubes(rvol, 0.5, vd.start, vd.end)
    ms_mc = _timed(mc_forward, flush, reps)
    verts, edges, tri = mc_out["r"]
    mgrad = torch.randn_like(verts)
    ms_mcg = _timed(lambda: marching_cubes_grad(rvol, 0.5, vd.start, vd.end, edges, mgrad),
                    flush, reps)
    cells = int(np.prod([r - 1 for r in vd.resolution]))
    pairs = nvox * S
    fit_iter, ms_fit = pose_fit_rate(device)
    from totri_gb300.reconstruct import FkMigration
    fk_in = torch.rand((1, 512, 64, 64), device=device) ** 4
    fk = FkMigration(512 * 0.005, 2.0, 2.0)
    ms_fk = _timed(lambda: fk(fk_in), flush, reps)
    from totri_gb300.util import UnitCubeMeshRender
    pv, pf, _ = scenes.displaced_sphere(5, 1)
    pv, pf = pv[0].to(device), pf[0].to(device)
    preview = UnitCubeMeshRender(resolution=512)
    ms_pv = _timed(lambda: preview.apply(pv, pf), flush, reps)
    return {
        "preview images/s": {"value": 1e3 / ms_pv, "ms": ms_pv,
                             "workload": "UnitCubeMeshRender 512x512 of a 20,480-face mesh "
                                         "(vertex normals, projection, raster, Phong shading; "
                                         "allocation of the image included)"},
        "fk migration voxels/s": {"value": 512 * 64 * 64 / (ms_fk / 1e3), "ms": ms_fk,
                                  "workload": "512 bins x 64 x 64 scan points (2 x 512 x 64 x "
                                              "64 complex FFTs, cuFFT through torch.fft)"},
        "pose fit iterations/s": {"value": fit_iter / (ms_fit / 1e3), "ms": ms_fit,
                                  "workload": "PoseFitting (translation + quaternion, Adam) "
                                              "of a 320-face mesh to a 32x32 x 512-bin "
                                              "transient, %d iterations, no early stop"
                                              % fit_iter},
        "marching cubes cells/s": {"value": cells / (ms_mc / 1e3), "ms": ms_mc,
                                   "triangles": int(tri[0]),
                                   "workload": "RBF volume of 4096 Gaussians, 128^3, iso 0.5, "
                                               "1 attribute; count + emit with the host "
                                               "read of the triangle count"},
        "marching cubes grad vertices/s": {"value": verts.shape[1] / (ms_mcg / 1e3),
                                           "ms": ms_mcg},
        "backproj voxel·scanpt/s": {"value": pairs / (ms_bp / 1e3), "ms": ms_bp,
                                    "workload": "Velten confocal, 128^3 voxels x 16384 scan "
                                                "points x 1024 bins"},
        "volume render voxel·scanpt/s": {"value": pairs / (ms_vf / 1e3), "ms": ms_vf,
                                         "workload": "confocal forward, 128^3 (2% occupied) x "
                                                     "16384 points x 1024 bins"},
        "volume adjoint voxel·scanpt/s": {"value": pairs / (ms_va / 1e3), "ms": ms_va},
        "rbf2volume voxel·gaussian/s": {"value": nvox * 4096 / (ms_rf / 1e3), "ms": ms_rf,
                                        "workload": "4096 Gaussians, 128^3, 1 attribute"},
        "rbf2volume grad voxel·gaussian/s": {"value": nvox * 4096 / (ms_rg / 1e3),
                                             "ms": ms_rg},
    }


def batched_metrics(device, count=32, steps=2, seed=1234):
    """Batched exhaustive mesh forward + backward: 32 meshes with triangle
    counts log-uniform in [1k, 50k] (lat/long spheres and random boxes),
    64x64 detector x 16x16 laser points, 2048 bins of 0.005 m; d loss /
    d transient of mesh i a seeded N(0, 1) field (totri_fill_normal, seed
    `seed` + i), loss = <transient, d loss / d transient>. One graph replay
    per step (waves within an 80 GB budget for the transients and their
    gradients, tiles from the autotuner) against the same work as 32
    sequential plain calls (forward, the same N(0, 1) field, gradient). A
    second line runs the energy head (loss 0.5 ||transient||^2, gradient =
    transient: one buffer per mesh, larger waves). The plain pass also gives
    the fraction of its wall time the GPU spends in the library's kernels,
    which bounds what any batching of these calls can gain. Unit: (face,
    detector point, laser point) triples per second."""
    from totri_gb300 import _lib, scenes
    from totri_gb300.batch import BatchedMeshRenderer, chunked_dot
    from totri_gb300.totri_cpp import render as R
    s = scenes.batched_exhaustive(count=count)
    meshes = [tuple(t.to(device) for t in m) for m in s["meshes"]]
    sp, lp, bd = s["scan_points"].to(device), s["laser_points"].to(device), s["bin_def"]
    S, L = sp.shape[0], lp.shape[0]
    triples = sum(m[1].shape[0] for m in meshes) * S * L
    stream = torch.cuda.current_stream()

    def timed(fn, n):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(stream)
        for _ in range(n):
            fn()
        e1.record(stream)
        e1.synchronize()
        return e0.elapsed_time(e1) / n

    def batched(head):
        t0 = time.time()
        br = BatchedMeshRenderer(meshes, sp, bd, laser_points=lp, grad=head, hbm_budget=80e9,
                                 normal_seed=seed)
        setup_s = time.time() - t0
        br.step()
        ms = timed(br.step, steps)
        out = {"ms": ms, "value": triples / (ms / 1e3), "waves": [len(w.members) for w in br.waves],
               "tiles": {str(k): v for k, v in br.tiles.items()}, "setup_s": setup_s}
        # per-kernel times of the same step launched eagerly (graph replays are
        # not visible to the library's launch profiler)
        _lib.profile_reset()
        _lib.profile_enable(True)
        with torch.cuda.stream(br.stream):
            br._step_calls()
        br.stream.synchronize()
        _lib.profile_enable(False)
        out["kernels_eager"] = {k: {"launches": v[0], "ms": v[2]}
                                for k, v in _lib.profile_read().items()}
        del br
        torch.cuda.empty_cache()
        return out

    normal = batched("normal")
    energy = batched("energy")
    so = torch.empty((1, 0, 3), device=device)
    lib = _lib.load()

    def plain():
        for i, (v, f, m) in enumerate(meshes):
            v, f, m = v[None], f[None], m[None]
            out = torch.empty((1, bd.num, S, L), device=device)
            R.mesh_exhaustive_forward(v, f, m, sp[None], lp[None], so, so, out, bd.width,
                                      bd.offset, 0)
            tg = torch.empty_like(out)
            _lib.check(lib.totri_fill_normal(ctypes.c_void_p(tg.data_ptr()), tg.numel(),
                                             seed + i, _lib.stream_of(device)))
            chunked_dot(out, tg)  # the loss, as the batched normal head forms it
            del out
            vg, mg = torch.empty_like(v), torch.empty_like(m)
            R.mesh_exhaustive_grad_verts(v, f, m, sp[None], lp[None], so, so, tg, vg, mg,
                                         bd.width, bd.offset, 0)

    plain()
    _lib.profile_reset()
    _lib.profile_enable(True)
    ms_plain = timed(plain, 1)
    _lib.profile_enable(False)
    kernels = {k: {"launches": v[0], "ms": v[2]} for k, v in _lib.profile_read().items()}
    busy = sum(v["ms"] for v in kernels.values()) / ms_plain
    torch.cuda.empty_cache()
    return {
        "kernels_plain_pass": kernels,
        "kernels_batched_eager": normal.pop("kernels_eager"),
        "value": normal["value"], "unit": "triples/s", "ms": normal["ms"],
        "plain_calls": {"value": triples / (ms_plain / 1e3), "ms": ms_plain,
                        "gpu_busy_fraction": busy},
        "speedup_vs_plain": ms_plain / normal["ms"],
        "speedup_bound_from_idle_gpu": 1.0 / busy if busy > 0 else None,
        "workload": "32 meshes, %d triangles in total (log-uniform 1k-50k), 64x64 detector x "
                    "16x16 laser points, 2048 bins x 0.005 m, fwd+bwd, seeded N(0,1) "
                    "d loss/d transient" % sum(m[1].shape[0] for m in meshes),
        "waves": normal["waves"], "tiles": normal["tiles"], "setup_s": normal["setup_s"],
        "energy_head": {k: v for k, v in energy.items() if k != "kernels_eager"},
    }


def serve_metrics(device, num_requests=100, seed=0, slots=4):
    """Serving mix (60% mesh renders/gradients, 40% Velten backprojections;
    grids 32^2-256^2, 512-4096 bins, meshes 320-50k faces, volumes 64^3-192^3)
    through ``totri_gb300.serve.Server`` under an 80 GB budget, against the
    same requests as back-to-back plain per-call API calls. Each arm returns
    results to pinned host memory. The server first answers one untimed pass of
    the request list (its steady state: resident BVHs, cached masks); then
    (a) all requests submitted at once give the throughput, (b) Poisson
    arrivals at 70% of that throughput give p50/p99 latency."""
    from totri_gb300 import scenes
    from totri_gb300.serve import Request, Server
    from totri_gb300.totri_cpp import reconstruct as K
    from totri_gb300.totri_cpp import render as R
    mix = scenes.serving_mix(num_requests, seed=seed)
    bins = scenes.SERVE_BINS
    dev_meshes = {k: tuple(t.to(device) for t in m) for k, m in mix["meshes"].items()}
    dev_grids = {k: g.to(device) for k, g in mix["grids"].items()}
    empty = torch.empty((1, 0, 3), device=device)
    tv, tf, tc = (t.to(device)[None] for t in mix["target"])
    meas = {}
    for g, sp in dev_grids.items():
        for b, bd in enumerate(bins):
            out = torch.empty((1, bd.num, sp.shape[0]), device=device)
            R.mesh_confocal_forward(tv, tf, tc, sp[None], empty, out, bd.width, bd.offset, 0)
            meas["%s_b%d" % (g, b)] = out[0]
    reqs = mix["requests"]

    def plain(r):
        sp = dev_grids[r["grid"]][None]
        bd = bins[r["bins"]]
        if r["kind"] == "backproject":
            vd = r["volume"]
            vol = torch.empty((1,) + tuple(vd.resolution), device=device)
            K.backprojection_confocal_velten_forward(meas[r["target"]][None], sp, empty, vol,
                                                     vd.start, vd.end, bd.width, bd.offset)
            return vol[0].cpu()
        v, f, c = (t[None] for t in dev_meshes[r["mesh"]])
        tr = torch.empty((1, bd.num, sp.shape[1]), device=device)
        R.mesh_confocal_forward(v, f, c, sp, empty, tr, bd.width, bd.offset, 0)
        if r["kind"] == "render":
            return tr[0].cpu()
        diff = tr - meas[r["target"]]
        loss = (diff * diff).mean()
        vg, cg = torch.empty_like(v), torch.empty_like(c)
        R.mesh_confocal_grad_verts(v, f, c, sp, empty, diff.mul_(2.0 / diff.numel()), vg, cg,
                                   bd.width, bd.offset, 0)
        return loss.cpu(), vg[0].cpu(), cg[0].cpu()

    plain(reqs[0])
    torch.cuda.synchronize(device)
    call_ms = []  # each plain call ends in a host copy, so its wall time is its own
    t0 = time.perf_counter()
    for r in reqs:
        t1 = time.perf_counter()
        plain(r)
        call_ms.append(1e3 * (time.perf_counter() - t1))
    plain_s = time.perf_counter() - t0
    torch.cuda.empty_cache()

    def req(r):
        return Request(r["kind"], r["grid"], mesh=r.get("mesh"), bins=bins[r["bins"]],
                       target=r.get("target"), volume=r.get("volume"))

    srv = Server(device, hbm_budget=80e9, slots=slots)
    for k, (v, f, c) in dev_meshes.items():
        srv.register_mesh(k, v, f, c)
    for k, sp in dev_grids.items():
        srv.register_grid(k, sp)
    for k, t in meas.items():
        srv.register_measurement(k, t, k.split("_")[0], bins[int(k.split("_b")[1])])
    resident = srv.budget.resident
    with srv:
        for fut in [srv.submit(req(r)) for r in reqs]:  # steady state: BVHs, masks
            fut.result()
        srv.completed.clear()
        t0 = time.perf_counter()
        for fut in [srv.submit(req(r)) for r in reqs]:
            fut.result()
        burst_s = time.perf_counter() - t0
        srv.completed.clear()
        rate = 0.7 * len(reqs) / burst_s
        gaps = np.random.default_rng(seed + 1).exponential(1.0 / rate, len(reqs))
        futs = []
        t0 = time.perf_counter()
        due = t0
        for r, gap in zip(reqs, gaps):
            due += gap
            while time.perf_counter() < due:
                time.sleep(min(1e-3, max(0.0, due - time.perf_counter())))
            futs.append(srv.submit(req(r)))
        for fut in futs:
            fut.result()
        poisson_s = time.perf_counter() - t0
        p50, p99 = srv.latency_ms()
        breakdown = srv.latency_breakdown()
    kinds = {k: sum(1 for r in reqs if r["kind"] == k) for k in ("render", "grad", "backproject")}
    out = {
        "value": len(reqs) / burst_s, "unit": "requests/s",
        # Each request alone, back to back: the slowest ones (192^3 Velten
        # backprojections from 256^2 points) bound any p99 of the mix from below.
        "plain_calls": {"value": len(reqs) / plain_s, "s": plain_s,
                        "call_ms_p50": float(np.percentile(call_ms, 50)),
                        "call_ms_p99": float(np.percentile(call_ms, 99)),
                        "call_ms_max": max(call_ms)},
        "speedup_vs_plain": plain_s / burst_s,
        "poisson": {"rate_per_s": rate, "p50_ms": p50, "p99_ms": p99,
                    "throughput": len(reqs) / poisson_s,
                    # p50/p99 (ms) of queue wait and service time, all requests
                    # and per class (small: high-priority streams; large:
                    # estimated at >= 5 ms of GPU time)
                    "breakdown": {c: {k: (list(v) if isinstance(v, tuple) else v)
                                      for k, v in d.items()}
                                  for c, d in breakdown.items()}},
        "requests": len(reqs), "kinds": kinds, "slots": slots,
        "hbm_budget_gb": 80, "resident_gb": resident / 1e9,
        "peak_admitted_gb": srv.budget.peak / 1e9,
        "workload": "serving mix: 8 meshes (%s faces), grids 32^2-256^2, 512-4096 bins, "
                    "volumes 64^3-192^3; steady state (one untimed pass first)" %
                    ",".join(str(m[1].shape[0]) for m in mix["meshes"].values()),
    }
    del srv
    torch.cuda.empty_cache()
    return out


def load_traffic():
    path = os.path.join(ROOT, "profiles", "traffic.json")
    if not os.path.exists(path):
        return {}
    with open(path) as f:
        return json.load(f)


def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            return json.load(f)
    return {}


# ---------------------------------------------------------------------------
# CPU baseline (the oracle restatement on the host cores).

def cpu_baseline(w_host, scan_subset):
    import oracle
    v = w_host["verts"][0].numpy()
    f = w_host["faces"][0].numpy()
    c = w_host["colors"][0].numpy()
    sp = w_host["scan_points"][0].numpy()[scan_subset]
    bd = w_host["bin_def"]
    oracle.lib()
    t0 = time.perf_counter()
    vis = oracle.mesh_visibility(v, f, sp, bvh=True)
    tr = oracle.mesh_confocal_forward(v, f, c, sp, None, vis, bd.num, bd.width, bd.offset,
                                      fp64=False)
    g = 2.0 * tr / tr.size
    oracle.mesh_confocal_grad(v, f, c, sp, None, vis, bd.num, bd.width, bd.offset, g,
                              fp64=False)
    dt = time.perf_counter() - t0
    pairs = sp.shape[0] * f.shape[0]
    return pairs / dt, dt, pairs


def cpu_cores():
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def reference_gpu_secondary(device, reps=2):
    """The reference's own volume, backprojection and RBF kernels (its sources
    compiled for sm_103a, launched with its launchers' geometry) timed on the
    workloads of the secondary lines, on the same GPU."""
    from oracle import ref_gpu
    from totri_gb300 import scenes
    flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device=device)
    s = scenes.volume_scene()
    vd, bd = s["volume_def"], s["bin_def"]
    sp = s["scan_points"].to(device).contiguous()
    S = sp.shape[1]
    nvox = int(np.prod(vd.resolution))
    tr = torch.rand((1, bd.num, S), device=device)
    vol_out = torch.empty((1,) + tuple(vd.resolution), device=device)
    empty = torch.zeros((1, 0, 3), device=device)
    ms_bp = _timed(lambda: ref_gpu.backprojection_confocal_velten(
        tr, sp, empty, vol_out, vd.start, vd.end, bd.width, bd.offset), flush, reps, warmup=1)
    vol = s["volume"].to(device).contiguous()
    mp = sp[0].T.contiguous()
    size = tuple(e - a for a, e in zip(vd.start, vd.end))
    trv = torch.empty((S, bd.num), device=device)
    ms_vf = _timed(lambda: ref_gpu.volume_confocal_forward(vol, mp, trv, vd.start, size,
                                                           bd.width, bd.offset),
                   flush, reps, warmup=1)
    adj = torch.empty_like(vol)
    ms_va = _timed(lambda: ref_gpu.volume_confocal_grad_volume(adj, mp, trv, vd.start, size,
                                                               bd.width, bd.offset),
                   flush, reps, warmup=1)
    rbf = scenes.rbf_set(4096, seed=5).to(device).contiguous()
    rvol = torch.empty((1, 2) + tuple(vd.resolution), device=device)
    ms_rf = _timed(lambda: ref_gpu.rbf2volume_forward(rbf, rvol, vd.start, vd.end), flush,
                   reps, warmup=1)
    rgrad = torch.empty_like(rbf)
    vg = torch.randn_like(rvol)
    ms_rg = _timed(lambda: ref_gpu.rbf2volume_grad(rbf, rvol, vg, rgrad, vd.start, vd.end),
                   flush, reps, warmup=1)
    pairs = nvox * S
    return {
        "backproj voxel·scanpt/s": {"value": pairs / (ms_bp / 1e3), "ms": ms_bp},
        "volume render voxel·scanpt/s": {"value": pairs / (ms_vf / 1e3), "ms": ms_vf},
        "volume adjoint voxel·scanpt/s": {
            "value": pairs / (ms_va / 1e3), "ms": ms_va,
            "note": "the reference's transposed operator (its volume backward)"},
        "rbf2volume voxel·gaussian/s": {"value": nvox * 4096 / (ms_rf / 1e3), "ms": ms_rf},
        "rbf2volume grad voxel·gaussian/s": {"value": nvox * 4096 / (ms_rg / 1e3),
                                             "ms": ms_rg},
    }


def run_reference(args, world, rank):
    if rank != 0:
        return
    from totri_gb300 import scenes
    s = scenes.confocal_differentiable()
    S = s["scan_points"].shape[1]
    n_sub = S  # each step is the whole workload (~4 s on 16 cores)
    subset = np.arange(S, dtype=np.int64)
    for _ in range(args.warmup):
        cpu_baseline(s, subset[::64])
    rates, times = [], []
    for _ in range(args.steps):
        r, dt, pairs = cpu_baseline(s, subset)
        rates.append(r)
        times.append(dt)
    value = float(np.median(rates))
    total_pairs = S * s["faces"].shape[1]
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT,
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1000.0 * total_pairs / value, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": bench_config(int(s["faces"].shape[1]), S, s["bin_def"].num, args.gpus),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cpu_cores(), "kind": "port",
                         "sample": "%d of %d scan points x all faces per step (BVH visibility, "
                                   "forward, gradient; FP32; OpenMP)" % (n_sub, S)},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "the reference mesh path needs the OptiX SDK (absent); this arm runs the "
                "CPU restatement of its algorithm",
        "secondary": None,
    }
    from oracle import ref_gpu
    if not args.no_secondary and ref_gpu.available():
        line["secondary"] = reference_gpu_secondary(torch.device("cuda", 0))
        line["secondary_note"] = ("the reference's own volume, backprojection and RBF CUDA "
                                  "kernels, built from its sources for sm_103a, on the "
                                  "workloads of this bench's secondary lines, same GPU")
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------

def main():
    args = parse_args()
    if args.impl == "reference":
        # rank 0 alone times the CPU restatement; other ranks exit without work
        run_reference(args, int(os.environ.get("WORLD_SIZE", "1")),
                      int(os.environ.get("RANK", "0")))
        return
    world, rank, local = dist_setup()
    from totri_gb300 import _lib
    device = torch.device("cuda", local)
    torch.cuda.set_device(device)
    _lib.load()
    w = make_workload(device)
    S, F = w["scan_points"].shape[1], w["faces"].shape[1]
    pairs = S * F
    flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device=device)
    stream = torch.cuda.current_stream(device)

    for _ in range(max(args.warmup, 3)):
        step(w, w["verts"], w["colors"], w["faces"], w["scan_points"], w["target"])
    torch.cuda.synchronize(device)

    # Device-timed region: inputs resident, L2 flushed between steps.
    clocks = ClockSampler(device.index)
    clocks.start()
    _lib.profile_reset()
    _lib.profile_enable(True)
    barrier(world)
    torch.cuda.synchronize(device)
    total_ms = 0.0
    for _ in range(args.steps):
        flush.zero_()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        step(w, w["verts"], w["colors"], w["faces"], w["scan_points"], w["target"])
        e1.record(stream)
        e1.synchronize()
        total_ms += e0.elapsed_time(e1)
    torch.cuda.synchronize(device)
    barrier(world)
    _lib.profile_enable(False)
    prof = _lib.profile_read()
    clk = clocks.stop()
    total_ms = max_over_ranks(total_ms, world, device)
    ms_per_step = total_ms / args.steps
    value = world * pairs * args.steps / (total_ms / 1000.0)
    launches = sum(v[0] for v in prof.values())

    # Roofline of the dominant kernel (FP32 SIMT: no tensor-core work exists here).
    bbar = mean_segments(w, device)
    flops = {
        "mesh visibility": flop_visibility(F),
        "mesh confocal splat": FLOP_SPLAT + FLOP_PER_SEG_FWD * bbar,
        "mesh confocal grad": FLOP_GRAD + FLOP_PER_SEG_BWD * bbar,
    }
    dom = max(prof.items(), key=lambda kv: kv[1][2])
    dom_name, (dom_launches, dom_timed, dom_ms) = dom
    peaks = measured_peaks()
    sm_count = torch.cuda.get_device_properties(device).multi_processor_count
    max_mhz = peaks.get("sm_max_mhz", 2070.0)
    fp32_peak = sm_count * 128 * 2 * max_mhz * 1e6 / 1e12
    roof = None
    if dom_name in flops and dom_timed > 0:
        per_launch_ms = dom_ms / dom_timed
        achieved = pairs * flops[dom_name] / (per_launch_ms / 1000.0) / 1e12
        traffic = load_traffic().get(dom_name)
        roof = {"bound": "fp32", "kernel": dom_name, "achieved": achieved, "peak": fp32_peak,
                "unit": "TFLOP/s", "frac": achieved / fp32_peak,
                "traffic": traffic.get("bytes_per_launch") if traffic else None,
                "peak_source": "nominal FP32 SIMT: %d SMs x 128 lanes x 2 FLOP x %.0f MHz "
                               "(MEASURED_PEAKS.json holds no FP32 figure)" % (sm_count, max_mhz),
                "flop_per_pair": flops[dom_name], "pairs_per_launch": pairs,
                "ms_per_launch": per_launch_ms, "b_bar": bbar}
        # The kernel is bound by instruction issue, not by FP32 arithmetic or
        # HBM: the issue view of the same kernel from its ncu capture (issue
        # slots in use, threads per warp instruction, thread instructions per
        # ray), as recorded beside its DRAM traffic.
        if traffic and "issue_active_pct" in traffic:
            roof["issue"] = {k: traffic[k] for k in (
                "issue_active_pct", "warps_active_pct", "threads_per_inst",
                "warp_inst_per_launch", "ms_under_ncu") if k in traffic}
            roof["issue"]["thread_inst_per_pair"] = (
                traffic["warp_inst_per_launch"] * traffic["threads_per_inst"] / pairs)
            roof["issue"]["source"] = traffic.get("source")
    kernels = {k: {"launches": v[0], "ms_per_step": v[2] / args.steps} for k, v in prof.items()}

    # End to end through the public API with host buffers.
    h = w["host"]
    pin = {k: h[k].pin_memory() for k in ("verts", "faces", "colors", "scan_points")}
    pin["target"] = w["target"].cpu().pin_memory()
    h2d = sum(t.numel() * t.element_size() for t in pin.values())
    out_loss = torch.empty((), dtype=torch.float32).pin_memory()
    out_vg = torch.empty_like(pin["verts"]).pin_memory()
    out_cg = torch.empty_like(pin["colors"]).pin_memory()
    d2h = 4 + out_vg.numel() * 4 + out_cg.numel() * 4
    e2e_steps = args.e2e_steps or args.steps
    for it in range(2 + e2e_steps):
        if it == 2:
            torch.cuda.synchronize(device)
            barrier(world)
            t0 = time.perf_counter()
        d = {k: v.to(device, non_blocking=True) for k, v in pin.items()}
        loss, vg, cg = step(w, d["verts"], d["colors"], d["faces"], d["scan_points"],
                            d["target"])
        out_loss.copy_(loss.detach(), non_blocking=True)
        out_vg.copy_(vg, non_blocking=True)
        out_cg.copy_(cg, non_blocking=True)
        torch.cuda.synchronize(device)
    e2e_s = max_over_ranks(time.perf_counter() - t0, world, device)
    e2e_value = world * pairs * e2e_steps / e2e_s

    secondary = None
    if rank == 0 and world == 1 and not args.no_secondary:
        secondary = secondary_metrics(device, flush)
    batched = None
    if rank == 0 and world == 1 and not args.no_batched:
        batched = batched_metrics(device)
    served = None
    if rank == 0 and world == 1 and not args.no_serve:
        served = serve_metrics(device)

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        everything = np.arange(S, dtype=np.int64)
        cpu_baseline(h, everything[::64])
        runs = [cpu_baseline(h, everything) for _ in range(3)]
        rate = float(np.median([r[0] for r in runs]))
        cpu = {"value": rate, "unit": UNIT, "cores": cpu_cores(), "kind": "port",
               "sample": "the whole step (4096 scan points x 20480 faces, %d pairs) 3 times, "
                         "%.1f s total, median rate: CPU-BVH visibility + forward + gradient, "
                         "FP32, OpenMP" % (runs[0][2], sum(r[1] for r in runs))}

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_per_step,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic",
            "config": bench_config(F, S, w["bin_def"].num, world),
            "roofline": roof, "cpu_baseline": cpu,
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h},
            "clocks": clk, "gpu_launches": launches, "kernels": kernels,
            "secondary": secondary,
            "batched": batched,
            "serve": served,
        }
        print(json.dumps(line), flush=True)
    barrier(world)


if __name__ == "__main__":
    main()
