"""Differentiable marching cubes on the GPU against the numpy oracle: vertices
and edge records bit for bit (FP32 with one rounding per operation on both
sides), gradients within FP32 atomics-order rounding, batch and edge cases,
and the RBF -> volume -> mesh -> transient chain end to end."""
import numpy as np
import pytest
import torch

import oracle
from totri_gb300 import scenes
from totri_gb300.types import BinDef, VolumeDef
from totri_gb300.util import MarchingCubesFunction, Rbf2VolumeGaussian
from totri_gb300.util.marching_cubes import marching_cubes, marching_cubes_grad

pytestmark = pytest.mark.gpu


def _rbf_volume(res, seed, n=64, attrs=1):
    g = np.random.default_rng(seed)
    rbf = np.concatenate([g.uniform(-0.35, 0.35, (n, 2)), g.uniform(0.65, 1.35, (n, 1)),
                          g.uniform(0.05, 0.12, (n, 1)), g.uniform(0, 1, (n, attrs))], 1)
    vd = VolumeDef((-0.5, -0.5, 0.5), (0.5, 0.5, 1.5), res)
    vol = Rbf2VolumeGaussian.apply(torch.tensor(rbf, dtype=torch.float32, device="cuda")[None], vd)
    return vol, vd


def _check_item(verts, edges, tri, ref_v, ref_e):
    n = 3 * int(tri)
    assert n == ref_v.shape[0]
    assert np.array_equal(edges[:n], ref_e)
    assert np.array_equal(verts[:n], ref_v)
    assert np.all(verts[n:] == 0) and np.all(edges[n:] == -1)


@pytest.mark.parametrize("res,iso", [((40, 40, 40), 0.5), ((33, 47, 29), 1.2)])
def test_matches_oracle_bit_for_bit(cuda_lib, res, iso):
    vol, vd = _rbf_volume(res, 0)
    verts, edges, tri = marching_cubes(vol, iso, vd.start, vd.end)
    ref_v, ref_e = oracle.marching_cubes(vol[0].cpu().numpy(), iso, vd.start, vd.end)
    assert ref_v.shape[0] > 300
    _check_item(verts[0].cpu().numpy(), edges[0].cpu().numpy(), tri[0], ref_v, ref_e)


def test_batch_and_edge_cases(cuda_lib):
    """Items with no crossing (all outside, all inside), grid values equal to
    iso (t = 0 vertices), the minimal 2x2x2 grid and a field item of its own
    size in one batch: counts, vertices and padding per item."""
    vol, vd = _rbf_volume((24, 24, 24), 1, attrs=2)
    v = vol[0]
    items = [torch.full_like(v, -1.0), torch.full_like(v, 3.0), v.clone(), v.clone()]
    items[3][0] = torch.round(items[3][0] * 4) / 4  # many grid values exactly at iso 0.5
    batch = torch.stack(items)
    verts, edges, tri = marching_cubes(batch, 0.5, vd.start, vd.end)
    assert tri[0] == 0 and tri[1] == 0
    for b in range(4):
        ref_v, ref_e = oracle.marching_cubes(batch[b].cpu().numpy(), 0.5, vd.start, vd.end)
        _check_item(verts[b].cpu().numpy(), edges[b].cpu().numpy(), tri[b], ref_v, ref_e)
    tiny = torch.tensor([[[[0.0, 1.0], [0.0, 0.0]], [[0.0, 0.0], [0.0, 0.0]]]],
                        device="cuda")[None]
    v2, e2, t2 = marching_cubes(tiny, 0.5, (0, 0, 0), (1, 1, 1))
    ref_v, ref_e = oracle.marching_cubes(tiny[0].cpu().numpy(), 0.5, (0, 0, 0), (1, 1, 1))
    assert int(t2[0]) == 1
    _check_item(v2[0].cpu().numpy(), e2[0].cpu().numpy(), t2[0], ref_v, ref_e)
    flat = torch.zeros((1, 1, 1, 5, 5), device="cuda")  # one slice: no cells
    v3, _, t3 = marching_cubes(flat, 0.5, (0, 0, 0), (1, 1, 1))
    assert int(t3[0]) == 0 and v3.shape[1] == 0


def test_gradient_matches_oracle(cuda_lib):
    vol, vd = _rbf_volume((32, 32, 32), 2, attrs=2)
    verts, edges, tri = marching_cubes(vol, 0.5, vd.start, vd.end)
    g = torch.randn(verts.shape, device="cuda", generator=torch.Generator("cuda").manual_seed(4))
    got = marching_cubes_grad(vol, 0.5, vd.start, vd.end, edges, g)[0].double().cpu().numpy()
    n = 3 * int(tri[0])
    ref = oracle.marching_cubes_grad(vol[0].cpu().numpy(), 0.5, vd.start, vd.end,
                                     edges[0, :n].cpu().numpy(), g[0, :n].cpu().numpy())
    err = np.linalg.norm(got - ref) / np.linalg.norm(ref)
    assert err < 1e-5


def test_rbf_to_transient_chain(cuda_lib):
    """RBF parameters -> volume -> marching cubes -> confocal render -> loss:
    the backward reaches the RBF parameters through every stage, and the
    marching-cubes stage of it equals the oracle's for the same cotangent."""
    from totri_gb300.render import MeshRenderConfocal
    g = np.random.default_rng(7)
    n = 24
    rbf = np.concatenate([g.uniform(-0.25, 0.25, (n, 2)), g.uniform(0.8, 1.2, (n, 1)),
                          g.uniform(0.06, 0.1, (n, 1))], 1)
    rbf = torch.tensor(rbf, dtype=torch.float32, device="cuda")[None].requires_grad_(True)
    vd = VolumeDef((-0.5, -0.5, 0.5), (0.5, 0.5, 1.5), (48, 48, 48))
    vol = Rbf2VolumeGaussian.apply(rbf, vd)
    vol.retain_grad()
    verts = MarchingCubesFunction.apply(vol, 0.5, vd.start, vd.end)
    verts.retain_grad()
    sp = scenes.wall_grid(16)[0][None].cuda()
    tr = MeshRenderConfocal.apply(verts[:, :, :3].contiguous(), None, sp,
                                  BinDef(0.01, 0.0, 512))
    loss = (tr * tr).sum()
    loss.backward()
    assert verts.shape[1] > 300 and float(loss.detach()) > 0
    assert torch.isfinite(rbf.grad).all() and float(rbf.grad.abs().sum()) > 0
    _, edges, tri = marching_cubes(vol.detach(), 0.5, vd.start, vd.end)
    k = 3 * int(tri[0])
    ref = oracle.marching_cubes_grad(vol[0].detach().cpu().numpy(), 0.5, vd.start, vd.end,
                                     edges[0, :k].cpu().numpy(), verts.grad[0, :k].cpu().numpy())
    got = vol.grad[0].double().cpu().numpy()
    assert np.linalg.norm(got - ref) / np.linalg.norm(ref) < 1e-5
