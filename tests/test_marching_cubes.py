"""Marching cubes on the CPU: the oracle's case table against the library's
(both derived, neither copied), the surface properties the derivation
promises, and the oracle gradient against central finite differences."""
import ctypes
from collections import Counter

import numpy as np
import pytest

import oracle
from oracle import isosurface as om


def _closed_noise(n, seed, channels=1):
    g = np.random.default_rng(seed)
    vol = g.standard_normal((channels, n, n, n)).astype(np.float32)
    vol[0, [0, -1]] = -1.0
    vol[0, :, [0, -1]] = -1.0
    vol[0, :, :, [0, -1]] = -1.0
    return vol


def _global_edges(shape, edges):
    C, D, H, W = shape
    pa, _ = om._endpoints(shape, edges)
    return ((pa[2] * H + pa[1]) * W + pa[0]) * 3 + (edges % 12) // 4


def test_library_table_equals_oracle_table(cuda_free_lib):
    ntri = (ctypes.c_uint8 * 256)()
    edges = (ctypes.c_int8 * (256 * 15))()
    assert cuda_free_lib.totri_marching_cubes_table(ntri, edges) == 0
    n2, e2 = oracle.marching_cubes_table()
    assert np.array_equal(np.frombuffer(ntri, np.uint8), n2)
    assert np.array_equal(np.frombuffer(edges, np.int8).reshape(256, 15), e2)


def test_case_table_uses_exactly_the_crossing_edges():
    ntri, table = oracle.marching_cubes_table()
    assert ntri[0] == 0 and ntri[255] == 0 and ntri.max() == 5
    for m in range(256):
        inside = [(m >> i) & 1 for i in range(8)]
        crossing = {e for e in range(12)
                    if inside[om.EDGES[e][0]] != inside[om.EDGES[e][1]]}
        used = table[m, :3 * ntri[m]].reshape(-1, 3)
        assert set(used.reshape(-1).tolist()) == crossing, m
        assert all(len(set(t)) == 3 for t in used.tolist()), m
        assert np.all(table[m, 3 * ntri[m]:] == -1)
        # loops of L points give L - 2 triangles
        assert ntri[m] == len(crossing) - 2 * len(_loops(m)), m


def _loops(m):
    ntri, table = oracle.marching_cubes_table()
    tris = table[m, :3 * ntri[m]].reshape(-1, 3).tolist()
    parent = {}

    def find(a):
        while parent.setdefault(a, a) != a:
            a = parent[a]
        return a
    for t in tris:
        for a in t[1:]:
            parent[find(a)] = find(t[0])
    return {find(a) for t in tris for a in t}


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_surface_is_closed_manifold_and_outward(seed):
    """Noise exercises every case, ambiguous faces included: each directed
    mesh edge (by grid edge) appears once and its reverse once, and the
    enclosed volume is positive (normals point out of the inside region)."""
    vol = _closed_noise(20, seed)
    verts, edges = oracle.marching_cubes(vol, 0.0, (-1, -1, -1), (1, 1, 1))
    keys = _global_edges(vol.shape, edges).reshape(-1, 3)
    c = Counter()
    for t in keys.tolist():
        for i in range(3):
            c[(t[i], t[(i + 1) % 3])] += 1
    assert all(k == 1 and c.get((b, a)) == 1 for (a, b), k in c.items())
    tri = verts[:, :3].reshape(-1, 3, 3).astype(np.float64)
    n = np.cross(tri[:, 1] - tri[:, 0], tri[:, 2] - tri[:, 0])
    assert np.einsum("ij,ij->i", tri[:, 0], n).sum() > 0


def test_sphere_area_and_volume():
    n = 48
    g = np.linspace(-1, 1, n)
    z, y, x = np.meshgrid(g, g, g, indexing="ij")
    r = np.sqrt(x * x + y * y + z * z)
    vol = np.stack([1.0 - r, x]).astype(np.float32)
    verts, _ = oracle.marching_cubes(vol, 0.4, (-1, -1, -1), (1, 1, 1))
    tri = verts[:, :3].reshape(-1, 3, 3).astype(np.float64)
    n_ = np.cross(tri[:, 1] - tri[:, 0], tri[:, 2] - tri[:, 0])
    area = 0.5 * np.linalg.norm(n_, axis=1).sum()
    volume = np.einsum("ij,ij->i", tri[:, 0], n_).sum() / 6
    assert abs(area / (4 * np.pi * 0.36) - 1) < 0.01
    assert abs(volume / (4 / 3 * np.pi * 0.216) - 1) < 0.01
    # the attribute channel is x, interpolated along the same edges
    assert np.abs(verts[:, 3] - verts[:, 0]).max() < 1e-6


def test_gradient_matches_finite_differences():
    g = np.random.default_rng(5)
    vol = _closed_noise(7, 3, channels=3).astype(np.float64)
    start, end = (-0.5, -0.4, 0.5), (0.5, 0.6, 1.3)
    iso = 0.1
    verts, edges = oracle.marching_cubes(vol, iso, start, end, dtype=np.float64)
    w = g.standard_normal(verts.shape)
    grad = oracle.marching_cubes_grad(vol, iso, start, end, edges, w)
    base_mask = om._cells(vol, iso, np.float64)
    h = 1e-6
    idx = np.argwhere(np.abs(grad) > 0)
    pick = idx[g.choice(len(idx), size=min(40, len(idx)), replace=False)]
    for c, z, y, x in pick:
        fd = []
        for s in (1, -1):
            v2 = vol.copy()
            v2[c, z, y, x] += s * h
            assert np.array_equal(om._cells(v2, iso, np.float64), base_mask)
            p, e2 = oracle.marching_cubes(v2, iso, start, end, dtype=np.float64)
            assert np.array_equal(e2, edges)
            fd.append((p * w).sum())
        num = (fd[0] - fd[1]) / (2 * h)
        assert abs(num - grad[c, z, y, x]) <= 1e-5 * max(1.0, abs(num)), (c, z, y, x)
