"""Pose fitting on the GPU: the loop recovers a known rigid offset; the same
loop driven by the FP64 CPU oracle's render and gradient follows the same
parameter trajectory; and a fit submitted to the request server gives the
same pose alone and in a mix of other requests."""
import numpy as np
import pytest
import torch

import oracle
from totri_gb300 import scenes
from totri_gb300.fitting import PoseFitting, Rotation, Translation, apply_transform
from totri_gb300.render import MeshRenderConfocal
from totri_gb300.types import BinDef

pytestmark = pytest.mark.gpu

OFFSET = (0.03, -0.02, 0.04)


def _scene():
    s = scenes.confocal_small(seed=2)
    v, f = s["verts"][0].cuda(), s["faces"][0].cuda()
    sp = s["scan_points"][0].cuda()
    bd = BinDef(0.01, 0.0, 512)
    with torch.no_grad():
        target = MeshRenderConfocal.apply((v + torch.tensor(OFFSET, device="cuda"))[None],
                                          f[None], sp[None], bd)[0]
    return v, f, sp, bd, target


def test_pose_fitting_recovers_a_translation(cuda_lib):
    v, f, sp, bd, target = _scene()
    fit = PoseFitting(bd)
    (t,), (q,) = fit.fit(target, sp, [v], [f], num_iter=300)
    err = (t.translation.detach()[0].cpu() - torch.tensor(OFFSET)).norm()
    assert float(fit.losses[-1]) < 0.05 * float(fit.losses[0])
    assert float(err) < 5e-3


class _OracleRender(torch.autograd.Function):
    """MeshRenderConfocal on the CPU oracle (FP64, brute-force visibility)."""

    @staticmethod
    def forward(ctx, verts, faces, scan_points, bin_def, colors=None, scan_origin=None):
        v, f, sp = (t[0].detach().cpu().numpy() for t in (verts, faces, scan_points))
        vis = oracle.mesh_visibility(v, f, sp)
        ctx.args = (v, f, sp, vis, bin_def)
        tr = oracle.mesh_confocal_forward(v, f, None, sp, None, vis, bin_def.num,
                                          bin_def.width, bin_def.offset)
        return torch.tensor(tr, dtype=torch.float32, device=verts.device)[None]

    @staticmethod
    def backward(ctx, g):
        v, f, sp, vis, bd = ctx.args
        vg, _ = oracle.mesh_confocal_grad(v, f, None, sp, None, vis, bd.num, bd.width,
                                          bd.offset, g[0].detach().cpu().numpy())
        return torch.tensor(vg, dtype=torch.float32, device=g.device)[None], None, None, None, \
            None, None


def test_pose_trajectory_matches_the_oracle_driven_loop(cuda_lib, monkeypatch):
    from totri_gb300.fitting import pose as pose_module
    v, f, sp, bd, target = _scene()
    runs = []
    for render in (MeshRenderConfocal, _OracleRender):
        monkeypatch.setattr(pose_module, "MeshRenderConfocal", render)
        fit = PoseFitting(bd)
        (t,), (q,) = fit.fit(target, sp, [v], [f], num_iter=8, stop_loss=None)
        with torch.no_grad():
            posed = apply_transform([v], [t], [q])[0]
        runs.append((posed.cpu().numpy(), torch.stack(fit.losses).cpu().numpy()))
    (p0, l0), (p1, l1) = runs
    # compared through the posed vertices: the quaternion's scale has a zero
    # gradient that Adam turns into rounding-sized steps of either sign
    assert np.abs(p0 - p1).max() < 1e-4
    assert np.abs(l0 - l1).max() <= 1e-3 * np.abs(l1).max()


def test_fit_request_alone_and_in_the_mix(cuda_lib):
    from totri_gb300.serve import Request, Server
    s = scenes.confocal_small(seed=2)
    v, f = s["verts"][0], s["faces"][0]
    sp = s["scan_points"][0]
    bd = BinDef(0.01, 0.0, 512)
    with torch.no_grad():
        target = MeshRenderConfocal.apply(
            (v.cuda() + torch.tensor(OFFSET, device="cuda"))[None], f.cuda()[None],
            sp.cuda()[None], bd)[0]
    other = scenes.displaced_sphere(3, 9)
    srv = Server(hbm_budget=8e9, slots=3)
    srv.register_mesh("m", v, f)
    srv.register_mesh("o", other[0][0], other[1][0])
    srv.register_grid("g", sp)
    srv.register_measurement("t", target, "g", bd)
    fit = Request("fit_pose", "g", mesh="m", bins=bd, target="t", iterations=40)
    with srv:
        alone = srv.submit(fit).result()
        futs = [srv.submit(Request("render", "g", mesh="o", bins=bd)) for _ in range(3)]
        mixed = srv.submit(Request("fit_pose", "g", mesh="m", bins=bd, target="t",
                                   iterations=40))
        futs += [srv.submit(Request("grad", "g", mesh="o", bins=bd, target="t"))
                 for _ in range(3)]
        mixed = mixed.result()
        for fu in futs:
            fu.result()
    assert torch.allclose(alone[0], mixed[0], atol=1e-4)  # translation (m)
    qa, qb = alone[1] / alone[1].norm(), mixed[1] / mixed[1].norm()
    assert torch.allclose(qa, qb, atol=1e-4)
    # losses along the way: FP32 gradients summed by atomics in either order
    assert float((alone[2] - mixed[2]).abs().max()) <= 1e-3 * float(alone[2].max())
    assert float(alone[2][-1]) < float(alone[2][0])


def _bump_target(res=16, laser=False):
    from totri_gb300.fitting import DepthMap
    from totri_gb300.types import VolumeDef
    vd = VolumeDef((-0.4, -0.4, 0.6), (0.4, 0.4, 1.4), (1, res, res))
    truth = DepthMap(VolumeDef(vd.start, vd.end, vd.resolution))
    y, x = torch.meshgrid(torch.linspace(-1, 1, res), torch.linspace(-1, 1, res), indexing="ij")
    with torch.no_grad():
        truth.depth[:] = (0.5 + 0.3 * torch.exp(-(x * x + y * y) / 0.3)).cuda()
        truth.clamp_params(None)
    sp = scenes.wall_grid(24)[0].cuda()
    lp = scenes.wall_grid(4)[0].cuda() if laser else None
    bd = BinDef(0.01, 0.0, 400)
    with torch.no_grad():
        if laser:
            from totri_gb300.render import MeshRenderExhaustive
            target = MeshRenderExhaustive.apply(truth.verts()[None], truth.faces[None], sp[None],
                                                lp[None], bd, truth.color.view(1, -1, 1))[0]
        else:
            target = MeshRenderConfocal.apply(truth.verts()[None], truth.faces[None], sp[None],
                                              bd, truth.color.view(1, -1, 1))[0]
    return vd, truth, sp, lp, bd, target


def test_depth_map_fitting_reduces_loss_and_depth_error(cuda_lib):
    from totri_gb300.fitting import DepthMap, DepthMapFitting
    from totri_gb300.types import VolumeDef
    vd, truth, sp, _, bd, target = _bump_target()
    dm = DepthMap(VolumeDef(vd.start, vd.end, vd.resolution))
    err0 = float((dm.depth - truth.depth).abs().mean())
    fit = DepthMapFitting(bd)
    fit.fit(dm, target, sp, num_iter=150, lambda_depth=0.02, lambda_color=0.01)
    assert float(fit.losses[-1]) < 0.2 * float(fit.losses[0])
    assert float((dm.depth - truth.depth).abs().mean()) < 0.75 * err0


def test_depth_map_fitting_exhaustive_subsets_and_subdivision(cuda_lib):
    """The exhaustive render, scan-point subsets and a grid refinement in one
    short run: the loss stays finite and the grid doubles."""
    from totri_gb300.fitting import DepthMap, DepthMapFitting
    from totri_gb300.types import VolumeDef
    vd, _, sp, lp, bd, target = _bump_target(res=8, laser=True)
    dm = DepthMap(VolumeDef(vd.start, vd.end, vd.resolution))
    fit = DepthMapFitting(bd)
    fit.fit(dm, target, sp, laser_points=lp, scan_point_limit=200, num_iter=6,
            subdivide_at=[3])
    assert dm.depth.shape == (16, 16) and dm.faces.shape[0] == 2 * 15 * 15
    assert all(torch.isfinite(l) for l in fit.losses)


def _rbf_problem():
    from totri_gb300.fitting import GaussianRbfBase
    from totri_gb300.types import VolumeDef
    vd = VolumeDef((-0.5, -0.5, 0.5), (0.5, 0.5, 1.5), (24, 24, 24))
    truth = GaussianRbfBase(VolumeDef(vd.start, vd.end, vd.resolution))
    for x, y, z in ((-0.1, 0.05, 0.95), (0.12, -0.08, 1.05), (0.0, 0.15, 1.1)):
        truth.append(x, y, z)
    sp = scenes.wall_grid(16)[0].cuda()
    bd = BinDef(0.01, 0.0, 320)
    return vd, truth, sp, bd


def test_rbf_optimize_reduces_loss(cuda_lib):
    """The inner loop (Adam through RBF splat -> marching cubes -> render)
    moves perturbed blobs towards the ones that made the measurement."""
    from totri_gb300.fitting import RbfFitting, TransientBackgroundEmpty
    vd, truth, sp, bd = _rbf_problem()
    fit = RbfFitting(bd, sp)
    with torch.no_grad():
        target = fit.base_to_transient(truth, TransientBackgroundEmpty(),
                                       torch.ones(1, device="cuda"))[1]
    target = target / target.mean()
    base = truth.clone()
    with torch.no_grad():
        base.params[:, :3] += torch.tensor([[0.04, -0.03, 0.03]], device="cuda")
    bg = TransientBackgroundEmpty()
    _, before = fit.loss_all(base, bg, target)
    losses, after, iters = fit.optimize(base, bg, target, num_iter=150)
    assert iters > 10
    assert float(after) < 0.5 * float(before)


def test_rbf_fit_moves_add_blobs(cuda_lib):
    """Three driver moves from no blobs at all: the volume and surface moves
    add blobs and the loss falls below that of the empty base."""
    from totri_gb300.fitting import GaussianRbfBase, RbfFitting, TransientBackgroundEmpty
    from totri_gb300.types import VolumeDef
    vd, truth, sp, bd = _rbf_problem()
    fit = RbfFitting(bd, sp)
    with torch.no_grad():
        target = fit.base_to_transient(truth, TransientBackgroundEmpty(),
                                       torch.ones(1, device="cuda"))[1]
    torch.manual_seed(0)
    base = GaussianRbfBase(VolumeDef(vd.start, vd.end, vd.resolution))
    norm = target / target.mean()
    _, empty_loss = fit.loss_all(base, TransientBackgroundEmpty(), norm)
    out = fit.fit(base, target, num_iter=2)
    _, final = fit.loss_all(out, TransientBackgroundEmpty(), norm)
    assert out.num_rbf() > 0
    assert float(final) < float(empty_loss)


class _CheckedRender:
    """MeshRenderConfocal (the GPU path, whose results the loop uses) with each
    forward it computes compared on the spot with the FP64 oracle at the same
    inputs, and each gradient recorded beside the oracle's gradient for the
    same upstream cotangent (compared after the loop)."""

    def __init__(self):
        self.forward_errors, self.entries = [], []

    def apply(self, verts, faces, scan_points, bin_def, colors=None, scan_origin=None):
        if verts.requires_grad:  # not for the loop's untracked intensity render
            verts.retain_grad()
            colors.retain_grad()
        y = MeshRenderConfocal.apply(verts, faces, scan_points, bin_def, colors, scan_origin)
        v = verts[0].detach().cpu().numpy()
        f = faces[0].cpu().numpy()
        sp = scan_points[0].cpu().numpy()
        c = colors[0].detach().cpu().numpy()
        bd = bin_def
        vis = oracle.mesh_visibility(v, f, sp)
        ref = oracle.mesh_confocal_forward(v, f, c, sp, None, vis, bd.num, bd.width, bd.offset)
        self.forward_errors.append(rel_l2(y[0].detach().cpu().numpy(), ref))
        entry = {"verts": verts, "colors": colors}

        def hook(g):
            entry["ref"] = oracle.mesh_confocal_grad(v, f, c, sp, None, vis, bd.num, bd.width,
                                                     bd.offset, g[0].cpu().numpy())
        if y.requires_grad:
            y.register_hook(hook)
        self.entries.append(entry)
        return y


def rel_l2(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def test_depth_map_loop_matches_the_oracle_at_every_step(cuda_lib, monkeypatch):
    """Eight steps of the depth-map fit: at every parameter state the loop
    visits, the GPU render equals the FP64 oracle's (1e-5) and so do the
    vertex and albedo gradients for that step's cotangent (1e-5). Two
    independently driven runs are not compared: Adam's first steps have the
    size of the learning rate for any gradient sign, so rounding-level
    gradient differences on near-zero entries would show as whole steps."""
    from totri_gb300.fitting import DepthMap, DepthMapFitting
    from totri_gb300.fitting import depth_map as dm_module
    from totri_gb300.types import VolumeDef
    vd, truth, _, _, bd, target = _bump_target(res=10)
    sp = scenes.wall_grid(12)[0].cuda()
    with torch.no_grad():
        target = MeshRenderConfocal.apply(truth.verts()[None], truth.faces[None], sp[None], bd,
                                          truth.color.view(1, -1, 1))[0]
    checked = _CheckedRender()
    monkeypatch.setattr(dm_module, "MeshRenderConfocal", checked)
    dm = DepthMap(VolumeDef(vd.start, vd.end, vd.resolution))
    fit = DepthMapFitting(bd)
    fit.fit(dm, target, sp, num_iter=8, lambda_depth=0.02, lambda_color=0.01)
    # one untracked render for the intensity, then one per step
    assert len(checked.forward_errors) == 9
    assert max(checked.forward_errors) < 1e-5, checked.forward_errors
    graded = [e for e in checked.entries if "ref" in e]
    assert len(graded) == 8
    for e in graded:
        rv, rm = e["ref"]
        assert rel_l2(e["verts"].grad[0].cpu().numpy(), rv) < 1e-5
        assert rel_l2(e["colors"].grad[0].cpu().numpy(), rm) < 1e-5
    assert float(fit.losses[-1]) < float(fit.losses[0])


def _robust_same(a, b, lr_bound):
    """Two runs of an Adam loop whose gradients differ by summation order
    (30 steps of a 12 x 12 depth map differ by a median 6.5e-5): half the
    entries within a tenth of one learning-rate step, the rest by at most the
    steps taken."""
    d = (a - b).abs().flatten()
    assert float(d.median()) <= 1e-3
    assert float(d.max()) <= lr_bound


def test_fit_depth_map_request_alone_and_in_the_mix(cuda_lib):
    from totri_gb300.fitting import DepthMap, DepthMapFitting
    from totri_gb300.serve import Request, Server
    from totri_gb300.types import VolumeDef
    vd, truth, sp, _, bd, target = _bump_target(res=12)
    other = scenes.displaced_sphere(3, 9)
    srv = Server(hbm_budget=8e9, slots=3)
    srv.register_mesh("o", other[0][0], other[1][0])
    srv.register_grid("g", sp.cpu())
    srv.register_measurement("t", target.cpu(), "g", bd)
    req = lambda: Request("fit_depth_map", "g", bins=bd, target="t", volume=vd,  # noqa: E731
                          iterations=30)
    with srv:
        alone = srv.submit(req()).result()
        futs = [srv.submit(Request("render", "g", mesh="o", bins=bd)) for _ in range(3)]
        mixed = srv.submit(req())
        futs += [srv.submit(Request("grad", "g", mesh="o", bins=bd, target="t"))
                 for _ in range(3)]
        mixed = mixed.result()
        for fu in futs:
            fu.result()
    dm = DepthMap(VolumeDef(vd.start, vd.end, vd.resolution))
    direct = DepthMapFitting(bd)
    direct.fit(dm, target, sp, num_iter=30)
    losses = torch.stack(direct.losses).cpu()
    for run in (alone, mixed):
        assert run[0].shape == (12, 12) and run[2].shape == (30,)
        _robust_same(run[0], dm.depth.cpu(), 2 * 1e-2 * 30)
        _robust_same(run[1], dm.color.cpu(), 2 * 1e-2 * 30)
        assert float((run[2] - losses).abs().max()) <= 1e-3 * float(losses.max())
    assert float(alone[2][-1]) < float(alone[2][0])


def test_fit_rbf_request_runs_beside_other_requests(cuda_lib):
    """A blob fit served on its worker thread: it adds blobs and lowers the
    loss below the empty set's, and the renders submitted beside it equal the
    same renders served alone."""
    from totri_gb300.fitting import GaussianRbfBase, RbfFitting, TransientBackgroundEmpty
    from totri_gb300.serve import Request, Server
    from totri_gb300.types import VolumeDef
    vd, truth, sp, bd = _rbf_problem()
    fit = RbfFitting(bd, sp)
    with torch.no_grad():
        target = fit.base_to_transient(truth, TransientBackgroundEmpty(),
                                       torch.ones(1, device="cuda"))[1]
    norm = target / target.mean()
    empty_loss = float(fit.loss_all(GaussianRbfBase(VolumeDef(vd.start, vd.end, vd.resolution)),
                                    TransientBackgroundEmpty(), norm)[0]["data"])
    other = scenes.displaced_sphere(3, 9)
    srv = Server(hbm_budget=8e9, slots=2, large_slots=1)
    srv.register_mesh("o", other[0][0], other[1][0])
    srv.register_grid("g", sp.cpu())
    srv.register_measurement("t", target.cpu(), "g", bd)
    with srv:
        ref = srv.submit(Request("render", "g", mesh="o", bins=bd)).result()
        blob = srv.submit(Request("fit_rbf", "g", bins=bd, target="t", volume=vd, iterations=2,
                                  seed=5))
        renders = [srv.submit(Request("render", "g", mesh="o", bins=bd)) for _ in range(4)]
        params, loss = blob.result()
        renders = [fu.result() for fu in renders]
    assert any(r.kind == "fit_rbf" and r.large for r in srv.completed)
    assert params.shape[0] > 0 and params.shape[1] == 4
    assert float(loss) < empty_loss
    for r in renders:
        assert torch.allclose(r, ref, rtol=1e-5, atol=1e-6 * float(ref.abs().max()))
