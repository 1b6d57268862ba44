"""Named kernel workloads for timing and profiling, one process per call:

    python -m totri_gb300.cases <case> [--small] [--reps N] [--set key=value ...]

Each case builds its inputs on cuda:0, runs its operator calls once untimed,
then `reps` times between CUDA events on the current stream, and prints one
JSON line with the mean milliseconds per call of each timed operator. Under
ncu, capture with -k <kernel regex> -s <launches to skip> -c 1..3. `--small`
shrinks the inputs (for multi-pass captures: a few hundred MB on the device);
`--set` overrides a tuning key (totri_gb300.autotune.set_tile) for the run.

Cases (full size / --small):
  visibility        the differentiable mesh workload's visibility: 20,480 faces
                    x 64x64 scan points (mesh_visibility, BVH build included)
  confocal-step     its render + loss + gradient step (one fwd+bwd of the bench)
  exhaustive        one 20k-face mesh, 32x32 detector x 16x16 laser points, 2,048
                    bins: forward, then gradient for an N(0, 1) cotangent
                    (--small: 16x16 x 8x8; --scan-res / --laser-res set the
                    grid sides)
  volume            128^3 voxels (2% occupied) x 128x128 points x 1,024 bins:
                    forward and exact adjoint (--small: 32x32 columns of 128
                    cells x 64x64 points)
  velten            Velten confocal backprojection of a 1,024-bin 128x128 scan
                    into 128^3 voxels (--small: 64^3 from 64x64; --volume-res,
                    --scan-res and --bins set the sides and the bin count over
                    the same 5.12 m)
  rbf               4,096 Gaussians into 128^3 voxels: forward and gradient
                    (--small: 1,024 Gaussians, 64^3)
"""
import argparse
import json

import torch

from . import autotune, scenes
from .types import BinDef


def _timed(calls, reps):
    """{name: mean ms per call} over `reps` rounds after one untimed round."""
    for fn in calls.values():
        fn()
    torch.cuda.synchronize()
    out = {}
    for name, fn in calls.items():
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(reps):
            fn()
        e1.record()
        torch.cuda.synchronize()
        out[name] = e0.elapsed_time(e1) / reps
    return out


def _mesh_differentiable(small):
    from .render import MeshRenderConfocal
    from .totri_cpp import render as R
    s = scenes.confocal_differentiable()
    d = {k: (v.cuda() if torch.is_tensor(v) else v) for k, v in s.items()}
    bd = d["bin_def"]
    with torch.no_grad():
        target = MeshRenderConfocal.apply(d["target_verts"], d["faces"], d["scan_points"], bd,
                                          d["target_colors"])
    return d, bd, target, R, MeshRenderConfocal


def case_visibility(small):
    d, _, _, R, _ = _mesh_differentiable(small)
    return {"mesh_visibility": lambda: R.mesh_visibility(d["verts"], d["faces"],
                                                         d["scan_points"])}, \
        {"faces": int(d["faces"].shape[1]), "scan_points": int(d["scan_points"].shape[1])}


def case_confocal_step(small):
    d, bd, target, _, Render = _mesh_differentiable(small)

    def step():
        v = d["verts"].detach().requires_grad_(True)
        c = d["colors"].detach().requires_grad_(True)
        tr = Render.apply(v, d["faces"], d["scan_points"], bd, c)
        torch.mean((tr - target) ** 2).backward()
    return {"fwd+bwd": step}, {"faces": int(d["faces"].shape[1]),
                               "scan_points": int(d["scan_points"].shape[1]), "bins": bd.num}


def case_exhaustive(small, scan_res=None, laser_res=None):
    from .totri_cpp import render as R
    v, f, a = (t.cuda() for t in scenes.uv_sphere(20000, 7))
    gs, gl = (16, 8) if small else (32, 16)
    gs, gl = scan_res or gs, laser_res or gl
    sp, lp = scenes.wall_grid(gs).cuda(), scenes.wall_grid(gl).cuda()
    bd = BinDef(0.005, 0.0, 2048)
    empty = torch.empty_like(sp[:, :0])
    tr = torch.empty((1, bd.num, sp.shape[1], lp.shape[1]), device="cuda")
    tg = torch.randn(tr.shape, device="cuda",
                     generator=torch.Generator(device="cuda").manual_seed(5))
    vg, mg = torch.empty_like(v), torch.empty_like(a)
    return {"forward": lambda: R.mesh_exhaustive_forward(v, f, a, sp, lp, empty, empty, tr,
                                                         bd.width, bd.offset, 0),
            "grad": lambda: R.mesh_exhaustive_grad_verts(v, f, a, sp, lp, empty, empty, tg, vg,
                                                         mg, bd.width, bd.offset, 0)}, \
        {"faces": int(f.shape[1]), "scan_points": int(sp.shape[1]),
         "laser_points": int(lp.shape[1]), "bins": bd.num}


def case_volume(small):
    from .totri_cpp import render as R
    s = scenes.volume_scene(scan_res=64 if small else 128)
    vd, bd = s["volume_def"], s["bin_def"]
    vol = s["volume"]
    start, end = list(vd.start), list(vd.end)
    if small:  # the central 32 x 32 columns, all 128 cells
        vol = vol[48:80, 48:80].contiguous()
        for i in range(2):
            w = (vd.end[i] - vd.start[i]) / 128
            start[i], end[i] = vd.start[i] + 48 * w, vd.start[i] + 80 * w
    size = tuple(e - a for a, e in zip(start, end))
    vol = vol.cuda()
    mp = s["scan_points"][0].T.contiguous().cuda()
    tr = torch.empty((mp.shape[1], bd.num), device="cuda")
    y = torch.rand(tr.shape, device="cuda", generator=torch.Generator(device="cuda").manual_seed(3))
    adj = torch.empty_like(vol)
    return {"forward": lambda: R.volume_confocal_forward(vol, mp, tr, start, size, bd.width,
                                                         bd.offset),
            "adjoint": lambda: R.volume_confocal_adjoint(adj, mp, y, start, size, bd.width,
                                                         bd.offset)}, \
        {"voxels": list(vol.shape), "points": int(mp.shape[1]), "bins": bd.num}


def case_velten(small, volume_res=None, scan_res=None, bins=None):
    from .totri_cpp import reconstruct as K
    res = volume_res or (64 if small else 128)
    s = scenes.volume_scene(res=res, scan_res=scan_res or res)
    vd, bd = s["volume_def"], s["bin_def"]
    if bins:  # the same 5.12 m span in finer bins, as the serving mix's bin sets
        bd = BinDef(5.12 / bins, 0.0, bins)
    sp = s["scan_points"].cuda()
    tr = torch.rand((1, bd.num, sp.shape[1]), device="cuda",
                    generator=torch.Generator(device="cuda").manual_seed(4))
    out = torch.empty((1, res, res, res), device="cuda")
    empty = torch.empty((1, 0, 3), device="cuda")
    return {"velten": lambda: K.backprojection_confocal_velten_forward(
        tr, sp, empty, out, vd.start, vd.end, bd.width, bd.offset)}, \
        {"voxels": res ** 3, "scan_points": int(sp.shape[1]), "bins": bd.num}


def case_rbf(small):
    from .totri_cpp import util as U
    n, res = (1024, 64) if small else (4096, 128)
    s = scenes.volume_scene(res=res)
    vd = s["volume_def"]
    rbf = scenes.rbf_set(n, 5).cuda()
    vol = torch.empty((1, 2, res, res, res), device="cuda")
    vg = torch.rand_like(vol)
    rg = torch.empty_like(rbf)
    return {"forward": lambda: U.rbf2volume_gaussian_forward(rbf, vol, vd.start, vd.end),
            "grad": lambda: U.rbf2volume_gaussian_grad(rbf, vol, vg, rg, vd.start, vd.end)}, \
        {"gaussians": n, "voxels": res ** 3}


CASES = {"visibility": case_visibility, "confocal-step": case_confocal_step,
         "exhaustive": case_exhaustive, "volume": case_volume, "velten": case_velten,
         "rbf": case_rbf}


def main(argv=None):
    p = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    p.add_argument("case", choices=sorted(CASES))
    p.add_argument("--small", action="store_true")
    p.add_argument("--reps", type=int, default=3)
    p.add_argument("--set", action="append", default=[], metavar="KEY=VALUE")
    p.add_argument("--scan-res", type=int, default=None,
                   help="exhaustive: detector grid side (default 32, --small 16); "
                   "velten: scan grid side (default the volume side)")
    p.add_argument("--laser-res", type=int, default=None,
                   help="exhaustive: laser grid side (default 16, --small 8)")
    p.add_argument("--volume-res", type=int, default=None,
                   help="velten: voxels per side (default 128, --small 64)")
    p.add_argument("--bins", type=int, default=None,
                   help="velten: bins over 5.12 m (default 1,024 of 0.005 m)")
    a = p.parse_args(argv)
    keys = {}
    for kv in a.set:
        k, v = kv.split("=")
        keys[k] = int(v)
        autotune.set_tile(k, int(v))
    extra = {}
    if a.case == "exhaustive":
        extra = dict(scan_res=a.scan_res, laser_res=a.laser_res)
    elif a.case == "velten":
        extra = dict(volume_res=a.volume_res, scan_res=a.scan_res, bins=a.bins)
    calls, config = CASES[a.case](a.small, **extra)
    ms = _timed(calls, a.reps)
    print(json.dumps({"case": a.case, "small": a.small, "reps": a.reps, "tune": keys,
                      "ms": ms, "config": config}))


if __name__ == "__main__":
    main()
