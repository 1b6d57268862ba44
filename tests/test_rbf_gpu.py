"""RBF-to-volume on the GPU against the FP64 oracle and the reference's golden
vectors, and the gradient against FP64 central differences of the oracle.

Tolerances (rel-L2): forward 1e-5 vs the FP64 oracle, 1e-4 vs the reference's
FP32 outputs; gradient 1e-4 vs the oracle.
"""
import os

import numpy as np
import pytest
import torch

import oracle
from totri_gb300 import scenes
from totri_gb300.types import VolumeDef
from totri_gb300.util import Rbf2VolumeGaussian

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def test_golden_vectors(cuda_lib):
    g = dict(np.load(os.path.join(GOLDEN, "rbf2volume.npz")))
    vd = VolumeDef(tuple(g["start"].tolist()), tuple(g["end"].tolist()),
                   tuple(int(x) for x in g["shape"]))
    rbf = torch.as_tensor(g["rbf"]).cuda().requires_grad_(True)
    vol = Rbf2VolumeGaussian.apply(rbf, vd)
    assert rel(vol.detach().cpu().numpy(), g["volume"]) < 1e-4
    vol.backward(torch.as_tensor(g["volume_grad"]).cuda())
    assert rel(rbf.grad.cpu().numpy(), g["rbf_grad"]) < 1e-4


@pytest.mark.parametrize("attrs", [0, 1, 3])
def test_against_oracle(cuda_lib, attrs):
    rng = np.random.default_rng(attrs)
    N = 300
    rbf = np.concatenate([rng.uniform(-0.5, 0.5, (N, 3)) + np.array([0, 0, 1.0]),
                          rng.uniform(0.02, 0.08, (N, 1)), rng.random((N, attrs))], 1)
    rbf = rbf.astype(np.float32)
    vd = VolumeDef((-0.5, -0.5, 0.5), (0.5, 0.5, 1.5), (20, 17, 13))
    r = torch.as_tensor(rbf[None]).cuda().requires_grad_(True)
    vol = Rbf2VolumeGaussian.apply(r, vd)
    ref = oracle.rbf2volume_forward(rbf, vd.resolution, vd.start, vd.end)
    assert rel(vol[0].detach().cpu().numpy(), ref) < 1e-5
    vg = torch.randn_like(vol)
    vol.backward(vg)
    rg = oracle.rbf2volume_grad(rbf, ref, vg[0].cpu().numpy(), vd.start, vd.end)
    assert rel(r.grad[0].cpu().numpy(), rg) < 1e-4


def test_full_gaussian_count(cuda_lib):
    """4,096 Gaussians (the RBF workload's count) on a 32^3 grid against the oracle."""
    rbf = scenes.rbf_set(4096, seed=5)
    vd = VolumeDef((-0.5, -0.5, 0.5), (0.5, 0.5, 1.5), 32)
    r = rbf.cuda().requires_grad_(True)
    vol = Rbf2VolumeGaussian.apply(r, vd)
    ref = oracle.rbf2volume_forward(rbf[0].numpy(), vd.resolution, vd.start, vd.end)
    assert rel(vol[0].detach().cpu().numpy(), ref) < 1e-5
    vg = torch.randn_like(vol)
    vol.backward(vg)
    rg = oracle.rbf2volume_grad(rbf[0].numpy(), ref, vg[0].cpu().numpy(), vd.start, vd.end)
    assert rel(r.grad[0].cpu().numpy(), rg) < 1e-4


def _with_cull(off, fn):
    from totri_gb300 import autotune
    autotune.set_tile("rbf.cull", 1 if off else 0)
    try:
        return fn()
    finally:
        autotune.set_tile("rbf.cull", 0)


@pytest.mark.parametrize("attrs", [0, 1, 3])
def test_underflow_cull_is_bit_identical(cuda_lib, attrs):
    """Gaussians whose ex2 value underflows to zero over a whole voxel brick
    are skipped; the forward stays bit for bit the same (zero terms, same
    order), also with non-finite and degenerate Gaussians in the set and a
    grid that does not divide into bricks, and with one voxel per thread
    instead of two ("rbf.forward.vz" = 1); the gradient (summed with atomics,
    so only equal up to their order) agrees to FP32 rounding."""
    from totri_gb300.totri_cpp import util as U
    rng = np.random.default_rng(40 + attrs)
    N = 700
    rbf = np.concatenate([rng.uniform(-0.5, 0.5, (N, 3)) + np.array([0, 0, 1.0]),
                          rng.uniform(0.01, 0.05, (N, 1)), rng.random((N, attrs))], 1)
    rbf = rbf.astype(np.float32)
    rbf[5, 0] = np.inf          # a non-finite centre is never culled
    rbf[9, 3] = 0.0             # sigma 0: infinite exponent constant
    if attrs:
        rbf[11, 4] = np.nan     # a non-finite attribute is never culled
    r = torch.as_tensor(rbf[None]).cuda()
    shape = (37, 21, 19)
    start, end = (-0.5, -0.5, 0.5), (0.5, 0.5, 1.5)

    def fwd():
        v = torch.full((1, 1 + attrs) + shape, 7.0, device="cuda")
        U.rbf2volume_gaussian_forward(r, v, start, end)
        return v

    on, off = fwd(), _with_cull(True, fwd)
    assert torch.equal(torch.nan_to_num(on, nan=1234.5), torch.nan_to_num(off, nan=1234.5))
    assert torch.equal(torch.isnan(on), torch.isnan(off))
    # one voxel per thread instead of two (paired FP32): the same bits
    from totri_gb300 import autotune
    autotune.set_tile("rbf.forward.vz", 1)
    try:
        one = fwd()
    finally:
        autotune.set_tile("rbf.forward.vz", 0)
    assert torch.equal(torch.nan_to_num(on, nan=1234.5), torch.nan_to_num(one, nan=1234.5))
    assert torch.equal(torch.isnan(on), torch.isnan(one))

    ok = np.isfinite(rbf).all(1) & (rbf[:, 3] > 0)  # the gradient on finite Gaussians
    r = torch.as_tensor(rbf[ok][None]).cuda()
    vol = fwd()
    vg = torch.randn_like(vol)

    def grad():
        g = torch.zeros_like(r)
        U.rbf2volume_gaussian_grad(r, vol, vg, g, start, end)
        return g

    g_on, g_off = grad(), _with_cull(True, grad)
    assert rel(g_on.cpu().numpy(), g_off.cpu().numpy()) < 1e-6
    # one Gaussian per warp iteration instead of two (paired FP32)
    autotune.set_tile("rbf.grad.pair", 2)
    try:
        g_one = grad()
    finally:
        autotune.set_tile("rbf.grad.pair", 0)
    assert rel(g_on.cpu().numpy(), g_one.cpu().numpy()) < 1e-6
