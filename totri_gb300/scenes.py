"""Seeded synthetic scenes for the benchmark workloads and the tests.

The reference ships no scenes or datasets usable here, so every workload is
generated from a seed (numpy PCG64): icospheres with jitter or low-frequency
radial displacement, random boxes, relay-wall scan grids, sparse volumes and
Gaussian RBF sets. Everything is produced on the CPU as float32 / int32
tensors and moved to the device by the caller.
"""
import math

import numpy as np
import torch

from .data.util import make_wall_grid
from .types import BinDef, VolumeDef


def rng(seed):
    return np.random.Generator(np.random.PCG64(seed))


def icosphere(level):
    """Unit icosphere: V = 10*4^level + 2 vertices, F = 20*4^level faces (outward CCW)."""
    t = (1.0 + math.sqrt(5.0)) / 2.0
    verts = [(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0), (0, -1, t), (0, 1, t),
             (0, -1, -t), (0, 1, -t), (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1)]
    verts = [np.array(v, np.float64) / np.linalg.norm(v) for v in verts]
    faces = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4),
             (11, 10, 2), (10, 7, 6), (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8),
             (3, 8, 9), (4, 9, 5), (2, 4, 11), (6, 2, 10), (8, 6, 7), (9, 8, 1)]
    for _ in range(level):
        cache = {}

        def mid(a, b):
            key = (min(a, b), max(a, b))
            if key not in cache:
                m = verts[a] + verts[b]
                verts.append(m / np.linalg.norm(m))
                cache[key] = len(verts) - 1
            return cache[key]

        nf = []
        for a, b, c in faces:
            ab, bc, ca = mid(a, b), mid(b, c), mid(c, a)
            nf += [(a, ab, ca), (b, bc, ab), (c, ca, bc), (ab, bc, ca)]
        faces = nf
    return np.array(verts, np.float64), np.array(faces, np.int64)


def _assoc_legendre(l, m, x):
    """P_l^m(x) (with the Condon-Shortley phase) by the standard recurrences."""
    pmm = np.ones_like(x)
    if m > 0:
        somx2 = np.sqrt(np.maximum(0.0, 1.0 - x * x))
        fact = 1.0
        for _ in range(m):
            pmm = -pmm * fact * somx2
            fact += 2.0
    if l == m:
        return pmm
    pmmp1 = x * (2 * m + 1) * pmm
    if l == m + 1:
        return pmmp1
    pll = pmmp1
    for ll in range(m + 2, l + 1):
        pll = ((2 * ll - 1) * x * pmmp1 - (ll + m - 1) * pmm) / (ll - m)
        pmm, pmmp1 = pmmp1, pll
    return pll


def real_sph_harm(l, m, theta, phi):
    """Orthonormal real spherical harmonic Y_lm at polar angle theta, azimuth phi."""
    am = abs(m)
    norm = math.sqrt((2 * l + 1) / (4 * math.pi) * math.factorial(l - am) /
                     math.factorial(l + am))
    p = _assoc_legendre(l, am, np.cos(theta))
    if m == 0:
        return norm * p
    if m > 0:
        return math.sqrt(2) * norm * p * np.cos(m * phi)
    return math.sqrt(2) * norm * p * np.sin(am * phi)


def radial_noise(dirs, seed, degree=4):
    """Sum of real spherical harmonics up to `degree` with N(0,1) coefficients,
    normalised to unit max magnitude, evaluated at unit directions [N, 3]."""
    g = rng(seed)
    theta = np.arccos(np.clip(dirs[:, 2], -1.0, 1.0))
    phi = np.arctan2(dirs[:, 1], dirs[:, 0])
    n = np.zeros(dirs.shape[0])
    for l in range(degree + 1):
        for m in range(-l, l + 1):
            n += g.standard_normal() * real_sph_harm(l, m, theta, phi)
    return n / max(np.abs(n).max(), 1e-12)


def wall_grid(res, extent=1.0):
    """[1, res*res, 3] float32 relay-wall grid on [-extent, extent]^2 at z = 0, x fastest."""
    return make_wall_grid(-extent, extent, res, -extent, extent, res,
                          device=torch.device('cpu'))[None].contiguous()


def _mesh_tensors(verts, faces, albedo):
    return (torch.from_numpy(verts.astype(np.float32))[None].contiguous(),
            torch.from_numpy(faces.astype(np.int32))[None].contiguous(),
            torch.from_numpy(albedo.astype(np.float32))[None, :, None].contiguous())


def jittered_sphere(level, seed, radius=0.3, center=(0.0, 0.0, 1.0), jitter=0.01):
    """Icosphere with per-vertex Gaussian jitter and albedo U[0.5, 1]."""
    g = rng(seed)
    v, f = icosphere(level)
    v = v * radius + np.array(center) + g.normal(0.0, jitter, size=v.shape)
    albedo = g.uniform(0.5, 1.0, size=v.shape[0])
    return _mesh_tensors(v, f, albedo)


def displaced_sphere(level, seed, radius=0.3, center=(0.0, 0.0, 1.0), amplitude=0.05):
    """Icosphere with radial displacement amplitude * (degree-4 SH noise) and
    albedo U[0.5, 1]."""
    v, f = icosphere(level)
    r = radius + amplitude * radial_noise(v, seed)
    albedo = rng(seed + 7919).uniform(0.5, 1.0, size=v.shape[0])
    return _mesh_tensors(v * r[:, None] + np.array(center), f, albedo)


def confocal_small(seed=0):
    """Plain confocal forward workload: level-2 icosphere (320 faces), radius 0.3 m
    at (0,0,1), jitter 0.01 m, albedo U[0.5,1]; 32x32 scan on [-1,1]^2;
    512 bins of 0.01 m."""
    verts, faces, colors = jittered_sphere(2, seed)
    return dict(verts=verts, faces=faces, colors=colors, scan_points=wall_grid(32),
                bin_def=BinDef(0.01, 0.0, 512))


def confocal_differentiable(seed=1, target_seed=2):
    """Differentiable confocal workload: level-5 icosphere (20,480 faces) with
    0.05 m low-frequency radial displacement; 64x64 scan; 1024 bins of 0.005 m;
    a target mesh from a second seed."""
    verts, faces, colors = displaced_sphere(5, seed)
    tverts, _, tcolors = displaced_sphere(5, target_seed)
    return dict(verts=verts, faces=faces, colors=colors, scan_points=wall_grid(64),
                bin_def=BinDef(0.005, 0.0, 1024), target_verts=tverts, target_colors=tcolors)


def sparse_volume(res, seed, fill=0.02):
    """[res]^3 float32 volume with Bernoulli(fill) placement and U[0,1] values."""
    g = rng(seed)
    occ = g.random((res, res, res)) < fill
    vals = g.uniform(0.0, 1.0, size=(res, res, res))
    return torch.from_numpy((occ * vals).astype(np.float32))


def volume_scene(res=128, scan_res=128, nbins=1024, seed=3):
    """Volume workload: res^3 voxels over [-0.5,0.5]^2 x [0.5,1.5] m, 2% occupied;
    scan_res^2 confocal scan on [-1,1]^2; nbins bins of 0.005 m."""
    return dict(volume=sparse_volume(res, seed), scan_points=wall_grid(scan_res),
                volume_def=VolumeDef((-0.5, -0.5, 0.5), (0.5, 0.5, 1.5), res),
                bin_def=BinDef(0.005, 0.0, nbins))


def rbf_set(n, seed, start=(-0.5, -0.5, 0.5), end=(0.5, 0.5, 1.5)):
    """[1, n, 5] Gaussians: centres uniform in the box, sigma U[0.01, 0.05], weight U[0,1]."""
    g = rng(seed)
    c = g.uniform(np.array(start), np.array(end), size=(n, 3))
    s = g.uniform(0.01, 0.05, size=(n, 1))
    w = g.uniform(0.0, 1.0, size=(n, 1))
    return torch.from_numpy(np.concatenate([c, s, w], axis=1).astype(np.float32))[None]
