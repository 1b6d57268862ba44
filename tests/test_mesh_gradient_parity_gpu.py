"""Gradient parity at the benchmarked sizes.

* The differentiable confocal workload (20,480 faces, 64x64 scan points,
  1,024 bins of 5 mm, MSE loss against a transient rendered from a second
  seeded mesh): the GPU's vertex and albedo gradients against the FP64 oracle
  evaluated on the same visibility masks, rel-L2 <= GRAD_TOL; and against FP64
  central differences of the loss (h = 1e-4 m) on a seeded vertex subset,
  skipping vertices whose +-h step flips any visibility bit.
* A batched-workload-sized exhaustive mesh (a 20,448-face displaced sphere,
  2,048 bins of 5 mm, an 8x8 subset of the 64x64 detector grid x a 4x4 subset
  of the 16x16 laser grid): forward and gradient against the FP64 oracle at
  every laser tile the autotuner can pick.

The bin coordinates are some hundreds of bins, so FP32 arithmetic (the
reference's kernels, or the oracle's FP32 mode) leaves the vertex gradient
~2e-4 from FP64 on this scene; the gradient kernels take the tent corners
relative to their first bin from double-float path lengths, which brings them
within GRAD_TOL. The central differences carry a truncation error that
falls as h^2 (on the CPU, FP64 differences against the FP64 analytic
gradient on 12 visible vertices: 2.1e-2 rel-L2 at h = 1e-4, 5.3e-4 at 1e-5,
5.3e-6 at 1e-6; tents of faces seen nearly edge-on span a small fraction of a
bin, so their higher derivatives are large). The test therefore takes the
specified step h = 1e-4 with a bound of 0.1 and the step 1e-6, where the
differences have converged, with a bound of 1e-4 (FD_TOL).
"""
import numpy as np
import pytest
import torch

import oracle
from totri_gb300 import autotune, scenes
from totri_gb300.totri_cpp import render as R
from totri_gb300.types import BinDef

from mesh_util import rel_l2, unpack_mask

pytestmark = pytest.mark.gpu

FWD_TOL = 1e-5
GRAD_TOL = 1e-5
FD_TOL = {1e-4: 0.1, 1e-6: 1e-4}  # central-difference step -> rel-L2 bound


@pytest.fixture(scope="module")
def differentiable(cuda_lib):
    """The workload on the device, its GPU masks (checked against the oracle on
    sampled pairs), the GPU transient and the MSE loss's transient gradient."""
    s = scenes.confocal_differentiable()
    bd = s["bin_def"]
    d = {k: (v.cuda() if torch.is_tensor(v) else v) for k, v in s.items()}
    F = d["faces"].shape[1]
    S = d["scan_points"].shape[1]
    empty = torch.empty_like(d["scan_points"][:, :0])
    masks = R.mesh_visibility(d["verts"], d["faces"], d["scan_points"])
    vis = unpack_mask(masks[0].cpu().numpy(), F)
    g = np.random.default_rng(21)
    pp, pf = g.integers(0, S, 2000), g.integers(0, F, 2000)
    n = {k: s[k][0].numpy() for k in ("verts", "faces", "colors", "scan_points")}
    ref = oracle.mesh_visibility_pairs(n["verts"], n["faces"], n["scan_points"], pp, pf)
    assert np.array_equal(vis[pp, pf], ref)

    def render(verts, colors):
        out = torch.empty((1, bd.num, S), device="cuda")
        R.mesh_confocal_forward(verts, d["faces"], colors, d["scan_points"], empty, out,
                                bd.width, bd.offset, 0)
        return out

    tr = render(d["verts"], d["colors"])
    target = render(d["target_verts"], d["target_colors"])
    tg = (2.0 / tr.numel()) * (tr - target)
    return dict(s=s, d=d, n=n, bd=bd, masks=masks, vis=vis, tr=tr, target=target, tg=tg,
                empty=empty)


def _gpu_grad(w):
    d, bd = w["d"], w["bd"]
    vg = torch.full_like(d["verts"], 5.0)
    mg = torch.full_like(d["colors"], 5.0)
    R.mesh_confocal_grad_verts(d["verts"], d["faces"], d["colors"], d["scan_points"], w["empty"],
                               w["tg"], vg, mg, bd.width, bd.offset, 0)
    return vg[0].double().cpu().numpy(), mg[0].double().cpu().numpy()


def test_differentiable_forward_matches_fp64_oracle(differentiable):
    w = differentiable
    n, bd = w["n"], w["bd"]
    ref = oracle.mesh_confocal_forward(n["verts"], n["faces"], n["colors"], n["scan_points"],
                                       None, w["vis"], bd.num, bd.width, bd.offset)
    assert rel_l2(w["tr"][0].double().cpu().numpy(), ref) < FWD_TOL


def test_differentiable_gradients_match_fp64_oracle(differentiable):
    """Vertex and albedo gradients of the MSE loss at full size against the FP64
    oracle on the same masks and the same transient gradient."""
    w = differentiable
    n, bd = w["n"], w["bd"]
    tg = w["tg"][0].double().cpu().numpy()
    rv, rm = oracle.mesh_confocal_grad(n["verts"], n["faces"], n["colors"], n["scan_points"],
                                       None, w["vis"], bd.num, bd.width, bd.offset, tg)
    gv, gm = _gpu_grad(w)
    ev, em = rel_l2(gv, rv), rel_l2(gm, rm)
    print("vertex gradient rel-L2 %.3e, albedo gradient rel-L2 %.3e" % (ev, em))
    assert ev < GRAD_TOL
    assert em < GRAD_TOL
    # the FP32 oracle (the reference's arithmetic) is further away than the GPU
    fv, _ = oracle.mesh_confocal_grad(n["verts"], n["faces"], n["colors"], n["scan_points"],
                                      None, w["vis"], bd.num, bd.width, bd.offset, tg,
                                      fp64=False)
    print("FP32 oracle vertex gradient rel-L2 %.3e" % rel_l2(fv, rv))


def test_differentiable_gradient_matches_central_differences(differentiable):
    """FP64 central differences of the loss (h = 1e-4 m and 1e-6 m along each
    axis) for a seeded subset of vertices against the GPU gradient. The gradient, like the
    reference's (mesh_confocal_grad_verts_optix.cu), treats visibility as a
    constant, so the differences are taken with the unperturbed masks held
    fixed. Only the faces around a vertex change with it, so the loss at v +- h
    is formed from the FP64 oracle's full transient with those faces'
    contributions replaced. A vertex whose step flips a visibility bit of one
    of its own faces (GPU masks of the perturbed mesh) is skipped: its
    contributions would jump. Bits of other faces flip for nearly every vertex
    at this step (rays that graze the moved faces); those jumps of the true loss
    are outside any gradient and are only counted."""
    w = differentiable
    n, bd, d = w["n"], w["bd"], w["d"]
    v, f, c, p = n["verts"], n["faces"], n["colors"], n["scan_points"]
    vis = w["vis"]
    base_t = oracle.mesh_confocal_forward(v, f, c, p, None, vis, bd.num, bd.width, bd.offset)
    resid = base_t - w["target"][0].double().cpu().numpy()
    N = base_t.size
    gv, _ = _gpu_grad(w)
    rng = np.random.default_rng(11)
    fd_all, g_all, skipped, used, elsewhere = {}, {}, 0, 0, 0
    # vertices no scan point sees (zero gradient) test nothing and are passed over
    for vi in rng.permutation(v.shape[0])[:400]:
        if used == 12:
            break
        if not np.any(gv[vi]):
            continue
        inc = np.nonzero((f == vi).any(1))[0]
        fi, vs = f[inc], np.ascontiguousarray(vis[:, inc])

        def t_inc(vv):
            return oracle.mesh_confocal_forward(vv, fi, c, p, None, vs, bd.num, bd.width,
                                                bd.offset)

        t0 = t_inc(v)
        rest = resid - t0
        steps = []
        for h in FD_TOL:
            for a in range(3):
                vp, vm = v.copy(), v.copy()
                vp[vi, a] = np.float32(v[vi, a] + h)
                vm[vi, a] = np.float32(v[vi, a] - h)
                steps.append((h, a, vp, vm))
        words = torch.from_numpy(inc // 32).cuda()
        shifts = torch.from_numpy(inc % 32).int().cuda()
        own = lambda m: (m[0][:, words] >> shifts) & 1  # noqa: E731
        base = own(w["masks"])
        flipped = False
        for _, _, vp, vm in steps:  # the larger steps first
            for vv in (vp, vm):
                m = R.mesh_visibility(torch.from_numpy(vv)[None].cuda(), d["faces"],
                                      d["scan_points"])
                flipped = not torch.equal(own(m), base)
                elsewhere += int(not torch.equal(m, w["masks"]))
                if flipped:
                    break
            if flipped:
                break
        if flipped:
            skipped += 1
            continue
        used += 1
        for h, a, vp, vm in steps:
            hp = float(vp[vi, a]) - float(v[vi, a])
            hm = float(v[vi, a]) - float(vm[vi, a])
            tp, tm = t_inc(vp), t_inc(vm)
            # loss(+) - loss(-) term by term, without forming the two losses
            dl = np.sum((tp - tm) * (2.0 * rest + tp + tm)) / N
            fd_all.setdefault(h, []).append(dl / (hp + hm))
            g_all.setdefault(h, []).append(gv[vi, a])
    errs = {h: rel_l2(np.array(g_all[h]), np.array(fd_all[h])) for h in fd_all}
    print("central differences: %d vertices, %d skipped, %d of the steps flip bits of other "
          "faces, rel-L2 %s" % (used, skipped, elsewhere,
                                ", ".join("%.3e at h=%g" % (e, h) for h, e in errs.items())))
    assert used >= 8
    for h, tol in FD_TOL.items():
        assert errs[h] < tol, (h, errs[h])


@pytest.fixture(scope="module")
def exhaustive_large(cuda_lib):
    v, f, a = scenes.uv_sphere(20448, 1005, radius=0.3, center=(0.05, -0.03, 1.0))
    grid_s = scenes.wall_grid(64)[0].reshape(64, 64, 3)
    grid_l = scenes.wall_grid(16)[0].reshape(16, 16, 3)
    sp = grid_s[4::8, 4::8].reshape(1, -1, 3).contiguous()   # 8x8 of the 64x64 detectors
    lp = grid_l[2::4, 2::4].reshape(1, -1, 3).contiguous()   # 4x4 of the 16x16 lasers
    bd = BinDef(0.005, 0.0, 2048)
    n = dict(verts=v[0].numpy(), faces=f[0].numpy(), colors=a[0].numpy(), sp=sp[0].numpy(),
             lp=lp[0].numpy())
    assert n["faces"].shape[0] >= 20000
    d = dict(verts=v.cuda(), faces=f.cuda(), colors=a.cuda(), sp=sp.cuda(), lp=lp.cuda())
    F = n["faces"].shape[0]
    vs = unpack_mask(R.mesh_visibility(d["verts"], d["faces"], d["sp"])[0].cpu().numpy(), F)
    vl = unpack_mask(R.mesh_visibility(d["verts"], d["faces"], d["lp"])[0].cpu().numpy(), F)
    assert np.array_equal(vs, oracle.mesh_visibility(n["verts"], n["faces"], n["sp"], bvh=True))
    assert np.array_equal(vl, oracle.mesh_visibility(n["verts"], n["faces"], n["lp"], bvh=True))
    ref = oracle.mesh_exhaustive_forward(n["verts"], n["faces"], n["colors"], n["sp"], n["lp"],
                                         None, None, vs, vl, bd.num, bd.width, bd.offset)
    tg = np.random.default_rng(33).standard_normal(ref.shape).astype(np.float32)
    rv, rm = oracle.mesh_exhaustive_grad(n["verts"], n["faces"], n["colors"], n["sp"], n["lp"],
                                         None, None, vs, vl, bd.num, bd.width, bd.offset,
                                         tg.astype(np.float64))
    return dict(n=n, d=d, bd=bd, ref=ref, tg=torch.from_numpy(tg)[None].cuda(), rv=rv, rm=rm)


_SPLAT_VARIANTS = [{}, {"mesh.exhaustive.splat.occupancy": 1},
                   {"mesh.exhaustive.splat.cluster": 1},
                   {"mesh.exhaustive.splat.occupancy": 1, "mesh.exhaustive.splat.cluster": 1}]


@pytest.mark.parametrize("keys", _SPLAT_VARIANTS, ids=lambda k: ",".join(
    "%s=%d" % (a.split(".")[-1], b) for a, b in k.items()) or "default")
@pytest.mark.parametrize("lt", autotune.CANDIDATES["mesh.exhaustive.splat.lt"])
def test_exhaustive_large_forward_at_every_laser_tile(exhaustive_large, lt, keys):
    """Every laser tile, with the register-capped splat (the default) or the
    uncapped one ("mesh.exhaustive.splat.occupancy" = 1), and for tiles
    narrower than 8 lasers with the cluster flush (the default) or each tile
    flushing alone ("mesh.exhaustive.splat.cluster" = 1)."""
    w = exhaustive_large
    d, bd = w["d"], w["bd"]
    empty = torch.empty_like(d["sp"][:, :0])
    out = torch.full((1, bd.num, d["sp"].shape[1], d["lp"].shape[1]), 3.0, device="cuda")
    autotune.set_tile("mesh.exhaustive.splat.lt", lt)
    for k, v in keys.items():
        autotune.set_tile(k, v)
    try:
        call = lambda: R.mesh_exhaustive_forward(  # noqa: E731
            d["verts"], d["faces"], d["colors"], d["sp"], d["lp"], empty, empty, out, bd.width,
            bd.offset, 0)
        if bd.num * lt * 4 > 200 * 1024:
            # the [bins][tile] histogram would not fit in shared memory: the
            # library refuses the tile, so the autotuner never picks it here
            with pytest.raises((ValueError, RuntimeError)):
                call()
            return
        call()
    finally:
        autotune.set_tile("mesh.exhaustive.splat.lt", 0)
        for k in keys:
            autotune.set_tile(k, 0)
    assert rel_l2(out[0].double().cpu().numpy(), w["ref"]) < FWD_TOL


_GRAD_VARIANTS = [{}, {"mesh.exhaustive.grad.mode": 1}, {"mesh.exhaustive.grad.mode": 2},
                  {"mesh.exhaustive.grad.occupancy": 4}, {"mesh.exhaustive.grad.layout": 2},
                  {"mesh.exhaustive.grad.layout": 2, "mesh.exhaustive.grad.sslice": 7,
                   "mesh.exhaustive.grad.lchunk": 5},
                  {"mesh.exhaustive.grad.chunk": 7},
                  {"mesh.exhaustive.grad.chunk": 32, "mesh.exhaustive.grad.lchunk": 5},
                  {"mesh.exhaustive.grad.faces": 1},
                  {"mesh.exhaustive.grad.faces": 5}, {"mesh.exhaustive.grad.faces": 32},
                  {"mesh.exhaustive.grad.lchunk": 5}, {"mesh.exhaustive.grad.lchunk": 8},
                  {"mesh.exhaustive.grad.sslice": 7},
                  {"mesh.exhaustive.grad.sslice": 32, "mesh.exhaustive.grad.lchunk": 5}]


@pytest.mark.parametrize("keys", _GRAD_VARIANTS, ids=lambda k: ",".join(
    "%s=%d" % (a.split(".")[-1], b) for a, b in k.items()) or "default")
def test_exhaustive_large_gradient_matches_fp64_oracle(exhaustive_large, keys):
    """The three gradient kernels (separable point records, the default;
    per-lane mask tests; compacted triples) and the point-record kernel's
    register cap, its transient_grad read in place or through bins-last
    copies of 7 or 32 scan points at a time, faces-per-CTA and laser-chunk shapes (including counts that
    do not divide the face or laser count) against the FP64 oracle."""
    w = exhaustive_large
    d, bd = w["d"], w["bd"]
    empty = torch.empty_like(d["sp"][:, :0])
    vg = torch.full_like(d["verts"], 2.0)
    mg = torch.full_like(d["colors"], 2.0)
    for k, v in keys.items():
        autotune.set_tile(k, v)
    try:
        R.mesh_exhaustive_grad_verts(d["verts"], d["faces"], d["colors"], d["sp"], d["lp"], empty,
                                     empty, w["tg"], vg, mg, bd.width, bd.offset, 0)
    finally:
        for k in keys:
            autotune.set_tile(k, 0)
    ev = rel_l2(vg[0].double().cpu().numpy(), w["rv"])
    em = rel_l2(mg[0].double().cpu().numpy(), w["rm"])
    print("exhaustive gradient rel-L2: vertices %.3e, albedo %.3e" % (ev, em))
    assert ev < GRAD_TOL
    assert em < GRAD_TOL
