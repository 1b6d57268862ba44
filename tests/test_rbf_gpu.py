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
