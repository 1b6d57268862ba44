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


def uv_sphere(target_faces, seed, radius=0.3, center=(0.0, 0.0, 1.0), amplitude=0.05):
    """Latitude/longitude sphere with about `target_faces` triangles (n rings x
    2n segments: 4n(n-1) faces), radial displacement amplitude * (degree-4 SH
    noise) and albedo U[0.5, 1]."""
    n = max(3, int(round(0.5 + math.sqrt(target_faces / 4.0 + 0.25))))
    seg = 2 * n
    theta = np.pi * np.arange(1, n) / n
    phi = 2.0 * np.pi * np.arange(seg) / seg
    st, ct = np.sin(theta)[:, None], np.cos(theta)[:, None]
    ring = np.stack([st * np.cos(phi)[None], st * np.sin(phi)[None],
                     np.broadcast_to(ct, (n - 1, seg))], -1).reshape(-1, 3)
    dirs = np.concatenate([[[0.0, 0.0, 1.0]], ring, [[0.0, 0.0, -1.0]]])
    top, bot = 0, dirs.shape[0] - 1
    idx = lambda r, j: 1 + r * seg + (j % seg)  # noqa: E731
    faces = []
    for j in range(seg):
        faces.append((top, idx(0, j), idx(0, j + 1)))
        faces.append((bot, idx(n - 2, j + 1), idx(n - 2, j)))
    for r in range(n - 2):
        for j in range(seg):
            a, b, c, d = idx(r, j), idx(r, j + 1), idx(r + 1, j), idx(r + 1, j + 1)
            faces += [(a, c, b), (b, c, d)]
    rad = radius + amplitude * radial_noise(dirs, seed)
    albedo = rng(seed + 7919).uniform(0.5, 1.0, size=dirs.shape[0])
    return _mesh_tensors(dirs * rad[:, None] + np.array(center), np.array(faces), albedo)


def random_box(target_faces, seed, center=(0.0, 0.0, 1.0)):
    """Randomly sized and rotated box (edges U[0.2, 0.6] m) whose six sides are
    m x m grids of quads (12 m^2 triangles, m chosen for `target_faces`),
    albedo U[0.5, 1]."""
    g = rng(seed)
    m = max(1, int(round(math.sqrt(target_faces / 12.0))))
    half = g.uniform(0.1, 0.3, size=3)
    q, _ = np.linalg.qr(g.standard_normal((3, 3)))
    u = np.linspace(-1.0, 1.0, m + 1)
    uu, vv = np.meshgrid(u, u, indexing="ij")
    verts, faces = [], []
    for axis in range(3):
        for sign in (-1.0, 1.0):
            p = np.zeros((m + 1, m + 1, 3))
            p[..., axis] = sign
            p[..., (axis + 1) % 3] = uu
            p[..., (axis + 2) % 3] = vv
            base = sum(v.shape[0] for v in verts)
            verts.append(p.reshape(-1, 3))
            for i in range(m):
                for j in range(m):
                    a = base + i * (m + 1) + j
                    b, c, d = a + 1, a + m + 1, a + m + 2
                    faces += [(a, c, b), (b, c, d)] if sign > 0 else [(a, b, c), (b, d, c)]
    v = np.concatenate(verts) * half
    v = v @ q.T + np.array(center)
    albedo = g.uniform(0.5, 1.0, size=v.shape[0])
    return _mesh_tensors(v, np.array(faces), albedo)


def batched_exhaustive(count=32, seed=0, lo=1000, hi=50000):
    """Batched exhaustive workload: `count` meshes with triangle counts
    log-uniform in [lo, hi] (alternately displaced lat/long spheres and random
    boxes, centres jittered around (0, 0, 1)); 64x64 detector points and
    16x16 laser points on [-1,1]^2; 2048 bins of 0.005 m."""
    g = rng(seed)
    meshes = []
    for i in range(count):
        nf = int(round(math.exp(g.uniform(math.log(lo), math.log(hi)))))
        c = (float(g.uniform(-0.2, 0.2)), float(g.uniform(-0.2, 0.2)), float(g.uniform(0.8, 1.2)))
        if i % 2 == 0:
            v, f, a = uv_sphere(nf, seed * 1000 + i, radius=float(g.uniform(0.15, 0.35)), center=c)
        else:
            v, f, a = random_box(nf, seed * 1000 + i, center=c)
        meshes.append((v[0], f[0], a[0]))
    return dict(meshes=meshes, scan_points=wall_grid(64)[0], laser_points=wall_grid(16)[0],
                bin_def=BinDef(0.005, 0.0, 2048))


SERVE_BINS = (BinDef(0.01, 0.0, 512), BinDef(0.005, 0.0, 1024), BinDef(0.0025, 0.0, 2048),
              BinDef(0.00125, 0.0, 4096))
SERVE_GRIDS = (32, 64, 128, 256)
SERVE_VOLUMES = (64, 96, 128, 160, 192)


def serving_mix(num_requests, seed=0, num_meshes=8):
    """Serving workload: `num_meshes` meshes with 320 to 50k triangles (a
    jittered level-2 icosphere, a displaced level-3 icosphere, then lat/long
    spheres and random boxes with log-uniform counts), wall grids of 32^2 to
    256^2 scan points, bin sets of 512 to 4096 bins spanning 5.12 m, volumes
    of 64^3 to 192^3 over [-0.5,0.5]^2 x [0.5,1.5]; a request list of 60% mesh
    requests (half renders, half gradients) and 40% Velten backprojections
    with uniformly drawn grid, bins, mesh and volume. Measurements (gradient
    targets, backprojection inputs) are renders of a separate target mesh."""
    g = rng(seed)
    meshes = {"m0": jittered_sphere(2, seed + 1), "m1": displaced_sphere(3, seed + 2)}
    for i in range(2, num_meshes):
        nf = int(round(math.exp(g.uniform(math.log(320), math.log(50000)))))
        c = (float(g.uniform(-0.15, 0.15)), float(g.uniform(-0.15, 0.15)),
             float(g.uniform(0.9, 1.1)))
        meshes["m%d" % i] = (uv_sphere(nf, seed * 100 + i, center=c) if i % 2 == 0
                             else random_box(nf, seed * 100 + i, center=c))
    grids = {"g%d" % r: wall_grid(r)[0] for r in SERVE_GRIDS}
    target = displaced_sphere(3, seed + 99, center=(0.05, -0.05, 1.0))
    requests = []
    for _ in range(num_requests):
        u = g.uniform()
        grid = "g%d" % SERVE_GRIDS[g.integers(len(SERVE_GRIDS))]
        b = int(g.integers(len(SERVE_BINS)))
        meas = "%s_b%d" % (grid, b)
        if u < 0.3:
            requests.append(dict(kind="render", grid=grid, bins=b,
                                 mesh="m%d" % g.integers(num_meshes)))
        elif u < 0.6:
            requests.append(dict(kind="grad", grid=grid, bins=b, target=meas,
                                 mesh="m%d" % g.integers(num_meshes)))
        else:
            res = SERVE_VOLUMES[g.integers(len(SERVE_VOLUMES))]
            requests.append(dict(kind="backproject", grid=grid, bins=b, target=meas,
                                 volume=VolumeDef((-0.5, -0.5, 0.5), (0.5, 0.5, 1.5), res)))
    return dict(meshes={k: (v[0][0], v[1][0], v[2][0]) for k, v in meshes.items()},
                grids=grids, target=(target[0][0], target[1][0], target[2][0]),
                requests=requests)
