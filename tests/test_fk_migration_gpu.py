"""f-k migration on the GPU against the reference's own outputs (golden) and
the FP64 oracle: the full pipeline (odd and even sizes, shifts folded into the
resampling) and the Stolt resampling alone."""
import os

import numpy as np
import pytest
import torch

import oracle
from totri_gb300.reconstruct import FkMigration, StoltInterpolation
from totri_gb300.reconstruct.fk_migration import stolt

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "fk_migration.npz")


def _rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


def test_fk_migration_matches_reference(cuda_lib):
    g = np.load(GOLDEN)
    for i in range(2):
        tr = torch.tensor(g["transient_%d" % i], device="cuda")
        v = FkMigration(*g["dims_%d" % i])(tr).cpu().numpy()
        assert v.shape == g["volume_%d" % i].shape
        assert _rel(v, g["volume_%d" % i]) < 1e-4


def test_stolt_matches_reference_and_folded_shifts(cuda_lib):
    g = np.load(GOLDEN)
    f = torch.view_as_complex(torch.tensor(g["stolt_in"], device="cuda").contiguous())
    s = StoltInterpolation(*g["stolt_dims"])(f)
    ref = g["stolt_out"][..., 0] + 1j * g["stolt_out"][..., 1]
    assert _rel(s.cpu().numpy(), ref) < 1e-5
    # reading an un-centred spectrum and writing an un-centred result equals
    # fftshift -> resample -> ifftshift
    x = f.reshape(-1, *f.shape[2:])
    dims = (1, 2, 3)
    raw = torch.fft.ifftshift(x, dim=dims)
    folded = stolt(raw, *g["stolt_dims"], input_centred=False, output_centred=False)
    explicit = torch.fft.ifftshift(stolt(x, *g["stolt_dims"]), dim=dims)
    assert torch.allclose(folded, explicit, atol=1e-6)


def test_batched_and_larger_against_oracle(cuda_lib):
    g = np.random.default_rng(3)
    tr = (g.random((2, 64, 24, 20)) ** 3).astype(np.float32)
    dims = (0.64, 2.0, 1.8)
    v = FkMigration(*dims)(torch.tensor(tr, device="cuda")).cpu().numpy()
    ref = oracle.fk_migration(tr, *dims)
    assert _rel(v, ref) < 1e-4
