"""f-k migration oracle on the CPU, pinned against the reference's own
implementation run on seeded inputs (tests/golden/fk_migration.npz)."""
import os

import numpy as np

import oracle

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "fk_migration.npz")


def _rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


def test_oracle_matches_reference_golden():
    g = np.load(GOLDEN)
    for i in range(2):
        v = oracle.fk_migration(g["transient_%d" % i], *g["dims_%d" % i])
        assert _rel(v, g["volume_%d" % i]) < 1e-5
    si = g["stolt_in"]
    s = oracle.stolt(si[..., 0] + 1j * si[..., 1], *g["stolt_dims"])
    ref = g["stolt_out"][..., 0] + 1j * g["stolt_out"][..., 1]
    assert _rel(s, ref) < 1e-5
