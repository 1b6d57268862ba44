"""The volume, backprojection and RBF operators against the reference's own
kernels run on the same GPU (oracle/ref_gpu.py: the reference's kernel sources
compiled for sm_103a and launched with its launchers' geometry) on the same
seeded inputs. Tolerance: rel-L2 1e-4 (FP32 on both sides), except where the
reference's GPU build takes a discrete decision from a value rounded by a
CUDA math function: its squares come from powf(x, 2) and its lengths from
norm3df (each within 2 ulp of the correctly rounded value; the same image
built without fused multiply-adds gives the same differences), while this
repo computes the FP32 chain that the oracle and the reference's CPU-built
golden vectors pin. A few bin or cell decisions in a million then fall on the
other side of an edge, each moving one output by one sample (measured on
these inputs: Velten 10-24 of 32,768 voxels, the transposed volume operator
4-7 of 32,768, the measurement-point gradient 0-2 of 768; the volume forward
matches to 2.6e-7). Those checks bound the rel-L2 by 1e-3 and require 99.9%
(99% for the 768 gradient entries) of the outputs to agree to 1e-5. Skipped
where the reference's kernel image has not been built (it is built only where
the reference tree is present)."""
import numpy as np
import pytest
import torch

from oracle import ref_gpu
from totri_gb300.totri_cpp import reconstruct as K
from totri_gb300.totri_cpp import render as R
from totri_gb300.totri_cpp import util as U

pytestmark = [pytest.mark.gpu,
              pytest.mark.skipif(not ref_gpu.available(),
                                 reason="reference kernel image not built")]


def rel(a, b):
    a = a.double()
    b = b.double()
    return float(torch.linalg.norm(a - b) / torch.clamp(torch.linalg.norm(b), min=1e-300))


def near_bins(ours, ref, frac=0.999):
    """Agreement up to a few samples on the other side of a bin or cell edge:
    rel-L2 below 1e-3 and all but (1 - frac) of the entries within 1e-5."""
    err = rel(ours, ref)
    close = torch.isclose(ours, ref, rtol=1e-5, atol=1e-5 * float(ref.abs().max()))
    return err < 1e-3 and float(close.double().mean()) > frac


@pytest.fixture(autouse=True)
def _seed():
    torch.manual_seed(0)


def wall(n, g):
    x, y = np.meshgrid(np.linspace(-1, 1, n), np.linspace(-1, 1, n))
    p = np.stack([x.ravel(), y.ravel(), np.zeros(n * n)], 1)
    p[:, :2] += g.uniform(-0.01, 0.01, (n * n, 2))
    return torch.tensor(p, dtype=torch.float32, device="cuda")


def test_volume_confocal(cuda_lib):
    g = np.random.default_rng(0)
    X, T, bw, bo = 32, 512, 0.005, 0.0
    vol = torch.tensor((g.random((X, X, X)) < 0.05) * g.random((X, X, X)), dtype=torch.float32,
                       device="cuda")
    mp = wall(16, g).T.contiguous()
    org, size = (-0.5, -0.5, 0.5), (1.0, 1.0, 1.0)
    N = mp.shape[1]
    ours, ref = torch.empty((N, T), device="cuda"), torch.empty((N, T), device="cuda")
    R.volume_confocal_forward(vol, mp, ours, org, size, bw, bo)
    ref_gpu.volume_confocal_forward(vol, mp, ref, org, size, bw, bo)
    assert rel(ours, ref) < 1e-4
    y = torch.randn((N, T), device="cuda")
    ours_v, ref_v = torch.empty_like(vol), torch.empty_like(vol)
    R.volume_confocal_grad_volume(ours_v, mp, y, org, size, bw, bo)
    ref_gpu.volume_confocal_grad_volume(ref_v, mp, y, org, size, bw, bo)
    assert near_bins(ours_v, ref_v), rel(ours_v, ref_v)
    ours_m, ref_m = torch.empty_like(mp), torch.empty_like(mp)
    R.volume_confocal_grad_measurement_points(ours_m, vol, mp, y, org, size, bw, bo)
    ref_gpu.volume_confocal_grad_mp(ref_m, vol, mp, y, org, size, bw, bo)
    assert near_bins(ours_m, ref_m, 0.99), rel(ours_m, ref_m)


def test_volume_exhaustive(cuda_lib):
    g = np.random.default_rng(1)
    D, S, L, T = 16, 64, 8, 256
    vol = torch.tensor((g.random((1, D, D, D)) < 0.1) * g.random((1, D, D, D)),
                       dtype=torch.float32, device="cuda")
    sp = wall(8, g).T[None].contiguous()
    lp = wall(3, g)[:L].T[None].contiguous()
    so = torch.tensor([[[0.2], [0.1], [-1.0]]], device="cuda").expand(1, 3, S).contiguous()
    lo = torch.zeros((1, 3, 0), device="cuda")
    st, en = (-0.5, -0.5, 0.5), (0.5, 0.5, 1.5)
    ours = torch.empty((1, T, S, L), device="cuda")
    ref = torch.empty_like(ours)
    R.volume_render_exhaustive_forward(vol, sp, lp, so, lo, ours, st, en, 0.02, 0.0)
    ref_gpu.volume_exhaustive_forward(vol, sp, lp, so, lo, ref, st, en, 0.02, 0.0)
    assert rel(ours, ref) < 1e-4


@pytest.mark.parametrize("origin", [False, True])
def test_velten_confocal(cuda_lib, origin):
    g = np.random.default_rng(2)
    T, D = 512, 32
    sp = wall(16, g)[None].contiguous()
    S = sp.shape[1]
    so = (torch.tensor([[[0.1, -0.2, -1.2]]], device="cuda").expand(1, S, 3).contiguous()
          if origin else torch.zeros((1, 0, 3), device="cuda"))
    tr = torch.rand((1, T, S), device="cuda")
    st, en = (-0.5, -0.5, 0.5), (0.5, 0.5, 1.5)
    ours = torch.empty((1, D, D, D), device="cuda")
    ref = torch.empty_like(ours)
    bw, bo = 0.01, 0.2 if origin else 0.0
    K.backprojection_confocal_velten_forward(tr, sp, so, ours, st, en, bw, bo)
    ref_gpu.backprojection_confocal_velten(tr, sp, so, ref, st, en, bw, bo)
    assert near_bins(ours, ref), rel(ours, ref)


def test_velten_exhaustive_and_arellano(cuda_lib):
    g = np.random.default_rng(3)
    T, D, L = 256, 16, 6
    sp = wall(8, g)[None].contiguous()
    lp = wall(3, g)[:L][None].contiguous()
    S = sp.shape[1]
    so, lo = torch.zeros((1, 0, 3), device="cuda"), torch.zeros((1, 0, 3), device="cuda")
    tr = torch.rand((1, T, S, L), device="cuda")
    st, en = (-0.5, -0.5, 0.5), (0.5, 0.5, 1.5)
    ours = torch.empty((1, D, D, D), device="cuda")
    ref = torch.empty_like(ours)
    K.backprojection_exhaustive_velten_forward(tr, sp, lp, so, lo, ours, st, en, 0.02, 0.0)
    ref_gpu.backprojection_exhaustive_velten(tr, sp, lp, so, lo, ref, st, en, 0.02, 0.0)
    assert near_bins(ours, ref), rel(ours, ref)
    spt, lpt = sp.transpose(1, 2).contiguous(), lp.transpose(1, 2).contiguous()
    sot, lot = torch.zeros((1, 3, 0), device="cuda"), torch.zeros((1, 3, 0), device="cuda")
    ours.zero_()
    K.backprojection_exhaustive_arellano_forward(tr, spt, lpt, sot, lot, ours, st, en, 0.02,
                                                 0.0)
    ref_gpu.backprojection_exhaustive_arellano(tr, spt, lpt, sot, lot, ref, st, en, 0.02, 0.0)
    assert rel(ours, ref) < 1e-4


def test_rbf2volume(cuda_lib):
    g = np.random.default_rng(4)
    N, R3 = 256, 24
    c = g.uniform(-0.5, 0.5, (N, 3))
    c[:, 2] += 1.0
    rbf = np.concatenate([c, g.uniform(0.02, 0.08, (N, 1)), g.uniform(0, 1, (N, 1))], 1)
    rbf = torch.tensor(rbf[None], dtype=torch.float32, device="cuda")
    st, en = (-0.5, -0.5, 0.5), (0.5, 0.5, 1.5)
    ours = torch.empty((1, 2, R3, R3, R3), device="cuda")
    ref = torch.empty_like(ours)
    U.rbf2volume_gaussian_forward(rbf, ours, st, en)
    ref_gpu.rbf2volume_forward(rbf, ref, st, en)
    assert rel(ours, ref) < 1e-4
    vg = torch.randn_like(ref)
    og, rg = torch.zeros_like(rbf), torch.empty_like(rbf)
    U.rbf2volume_gaussian_grad(rbf, ref, vg, og, st, en)
    ref_gpu.rbf2volume_grad(rbf, ref, vg, rg, st, en)
    assert rel(og, rg) < 1e-4
