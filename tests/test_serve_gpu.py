"""Request server on the GPU: every result is the same alone and in the mix.

Tolerances: renders and backprojections within rel-L2 1e-6 of the same
request run alone and of the plain per-call API (shared-memory atomics add in
a run-dependent order); gradients within 1e-5; losses within 1e-6 relative.
"""
import numpy as np
import pytest
import torch

from totri_gb300 import scenes
from totri_gb300.serve import Request, Server
from totri_gb300.totri_cpp import reconstruct as K
from totri_gb300.totri_cpp import render as R
from totri_gb300.types import BinDef, VolumeDef

from mesh_util import rel_l2

pytestmark = pytest.mark.gpu

BINS = BinDef(0.01, 0.0, 300)
BINS2 = BinDef(0.005, 0.0, 700)
VOL = VolumeDef((-0.5, -0.5, 0.5), (0.5, 0.5, 1.5), 32)
VOL2 = VolumeDef((-0.4, -0.4, 0.6), (0.4, 0.4, 1.4), (40, 24, 32))


def _scene():
    meshes = {
        "ico": scenes.jittered_sphere(2, 31),
        "bumpy": scenes.displaced_sphere(3, 32, center=(0.1, 0.0, 1.1)),
        "box": scenes.random_box(2000, 33),
    }
    grids = {"g16": scenes.wall_grid(16)[0], "g24": scenes.wall_grid(24)[0]}
    return meshes, grids


def _plain_render(m, sp, bd):
    v, f, c = (t.cuda() for t in m)
    out = torch.empty((1, bd.num, sp.shape[0]), device="cuda")
    R.mesh_confocal_forward(v, f, c, sp[None].cuda(), torch.empty((1, 0, 3), device="cuda"),
                            out, bd.width, bd.offset, 0)
    return out


def _server(meshes, grids, **kw):
    srv = Server(**kw)
    for name, (v, f, c) in meshes.items():
        srv.register_mesh(name, v[0], f[0], c[0])
    for name, sp in grids.items():
        srv.register_grid(name, sp)
    target = scenes.displaced_sphere(3, 35, center=(0.0, 0.05, 1.05))  # not a request mesh
    for g, sp in grids.items():
        for bd, tag in ((BINS, "a"), (BINS2, "b")):
            meas = _plain_render(target, sp, bd)[0]
            srv.register_measurement("%s_%s" % (g, tag), meas, g, bd)
    return srv


def _requests():
    reqs = []
    for mesh in ("ico", "bumpy", "box"):
        for g in ("g16", "g24"):
            reqs.append(Request("render", g, mesh=mesh, bins=BINS))
            reqs.append(Request("grad", g, mesh=mesh, bins=BINS2, target=g + "_b"))
    reqs.append(Request("render", "g24", mesh="ico", bins=BINS2))
    reqs.append(Request("backproject", "g16", target="g16_a", volume=VOL))
    reqs.append(Request("backproject", "g24", target="g24_b", volume=VOL2))
    reqs.append(Request("grad", "g16", mesh="box", bins=BINS, target="g16_a"))
    return reqs


def _clone(r):
    return Request(r.kind, r.grid, mesh=r.mesh, bins=r.bins, target=r.target, volume=r.volume)


def _compare(kind, a, b):
    if kind == "grad":
        assert abs(float(a[0]) - float(b[0])) <= 1e-6 * abs(float(b[0]))
        assert rel_l2(a[1].numpy(), b[1].numpy()) < 1e-5
        assert rel_l2(a[2].numpy(), b[2].numpy()) < 1e-5
    else:
        assert rel_l2(a.numpy(), b.numpy()) < 1e-6


def test_results_same_alone_and_in_the_mix(cuda_lib):
    meshes, grids = _scene()
    reqs = _requests()
    alone = []
    with _server(meshes, grids, slots=1) as srv:
        for r in reqs:
            alone.append(srv.submit(_clone(r)).result(timeout=120))
    # a low threshold sends part of the mix to the normal-priority streams
    with _server(meshes, grids, slots=4, large_slots=2, large_ms=0.02) as srv:
        futs = [srv.submit(_clone(r)) for r in reqs * 3]  # each request three times
        mixed = [f.result(timeout=300) for f in futs]
        p50, p99 = srv.latency_ms()
        assert p50 is not None and p99 >= p50
        assert srv.budget.peak <= srv.budget.total
        br = srv.latency_breakdown()
        assert br["small"]["requests"] > 0 and br["large"]["requests"] > 0
        assert br["all"]["requests"] == len(futs)
        for cls in ("small", "large"):
            wait, service = br[cls]["wait"], br[cls]["service"]
            assert wait[0] >= 0 and service[0] > 0 and service[1] >= service[0]
    for i, r in enumerate(reqs * 3):
        _compare(r.kind, mixed[i], alone[i % len(reqs)])


def test_cancelled_requests_release_their_memory(cuda_lib):
    """A request cancelled while queued never runs; one cancelled in flight
    runs to its end on the GPU, its result is dropped, its device memory
    returns to the budget and its visibility mask is unpinned; the server then
    serves the next request. The scheduler's steps are driven by hand here, so
    the request is certainly in flight when it is cancelled."""
    meshes, grids = _scene()
    srv = _server(meshes, grids)
    queued = srv.submit(Request("render", "g16", mesh="ico", bins=BINS))
    assert queued.cancel()
    flight = srv.submit(Request("grad", "g24", mesh="bumpy", bins=BINS2, target="g24_b"))
    with srv.cv:
        assert srv._admit_one()  # drops the cancelled request
        assert len(srv.queue) == 1 and not srv.inflight
        assert srv._admit_one()
        assert len(srv.inflight) == 1 and srv.budget.inflight > 0
        assert srv.masks.pins
        assert flight.cancel()
        torch.cuda.synchronize()
        assert srv._reap()
    assert srv.cancelled == 1 and not srv.completed
    assert srv.budget.inflight == 0 and not srv.masks.pins
    assert queued.cancelled() and flight.cancelled()
    with srv:
        ok = srv.submit(Request("render", "g16", mesh="ico", bins=BINS))
        assert ok.result(timeout=60).shape == (BINS.num, 256)
    assert srv.budget.inflight == 0


def test_results_match_plain_calls(cuda_lib):
    meshes, grids = _scene()
    reqs = _requests()
    with _server(meshes, grids, slots=4) as srv:
        res = [f.result(timeout=300) for f in [srv.submit(_clone(r)) for r in reqs]]
        meas = {k: v for k, v in srv.measurements.items()}
    for r, got in zip(reqs, res):
        sp = grids[r.grid]
        if r.kind == "render":
            ref = _plain_render(meshes[r.mesh], sp, r.bins)[0].cpu()
            _compare("render", got, ref)
        elif r.kind == "grad":
            v, f, c = (t.cuda() for t in meshes[r.mesh])
            tr = _plain_render(meshes[r.mesh], sp, r.bins)
            target = meas[r.target][0]
            diff = tr - target
            loss = (diff * diff).mean()
            vg, cg = torch.empty_like(v), torch.empty_like(c)
            R.mesh_confocal_grad_verts(v, f, c, sp[None].cuda(),
                                       torch.empty((1, 0, 3), device="cuda"),
                                       (diff * (2.0 / diff.numel())).contiguous(), vg, cg,
                                       r.bins.width, r.bins.offset, 0)
            _compare("grad", got, (loss.cpu(), vg[0].cpu(), cg[0].cpu()))
        else:
            tr, _, bd = meas[r.target]
            vol = torch.empty((1,) + tuple(r.volume.resolution), device="cuda")
            K.backprojection_confocal_velten_forward(tr, sp[None].cuda(),
                                                     torch.empty((1, 0, 3), device="cuda"), vol,
                                                     r.volume.start, r.volume.end, bd.width,
                                                     bd.offset)
            _compare("backproject", got, vol[0].cpu())


def test_admission_under_a_small_budget(cuda_lib):
    """A budget that holds one transient at a time still serves every request
    (requests wait for memory; masks are evicted when not in use), and a
    request larger than the whole budget fails alone."""
    meshes, grids = _scene()
    probe = _server(meshes, grids)
    resident = probe.budget.resident
    one = 4 * BINS2.num * 24 * 24 * 2 + (1 << 20)
    with _server(meshes, grids, slots=4, hbm_budget=resident + one) as srv:
        reqs = _requests()
        futs = [srv.submit(_clone(r)) for r in reqs if r.kind != "backproject"]
        for f in futs:
            f.result(timeout=300)
        assert srv.budget.peak <= srv.budget.total
        big = srv.submit(Request("render", "g24", mesh="ico", bins=BinDef(0.01, 0.0, 100000)))
        with pytest.raises(MemoryError):
            big.result(timeout=60)
        ok = srv.submit(Request("render", "g16", mesh="ico", bins=BINS))
        assert ok.result(timeout=60).shape == (BINS.num, 256)
    assert np.isfinite(srv.latency_ms()[1])
