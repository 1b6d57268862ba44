"""CPU oracle for differentiable marching cubes (TEST INFRASTRUCTURE).

The reference calls ``tomcubes.MarchingCubesFunction.apply(volume[None], iso,
volume_def.start, volume_def.end)[0]`` (totri/fitting/rbf.py:88-98,
rbf_backup.py:154-160) on an RBF volume [1, 1+A, D, H, W] and renders the
result as a triangle soup with ``faces_of_verts(verts, None)`` (rbf.py:719),
taking vertex channels 3.. as colours (rbf.py:253, 258). The tomcubes source
is an un-vendored submodule (.gitmodules:4-6, ``extern/tomcubes`` is empty,
its pinned commit unknown), so parity is unpinned against it: this module
restates marching cubes (Lorensen and Cline, SIGGRAPH 1987) from the
mathematics, with a case table derived here rather than copied:

* a grid point is inside when its channel-0 value is above ``iso``;
* on each cube face, the contour segments cut off each maximal run of
  consecutive inside corners (on a face with two diagonal inside corners
  each corner is its own run, so the two are separated); the rule depends only
  on the face's four corners, so neighbouring cells agree and the surface is
  closed;
* segments are oriented with the inside corners on their left seen from
  outside the cube and chained into loops; each loop of L edge points is cut
  into L - 2 triangles whose diagonals never join two points of one cube face
  (such a diagonal would lie in the face and be shared with the neighbouring
  cell's triangles, leaving non-manifold edges): the first such triangulation
  in the order of a recursive split of the chord (q0, q[L-1]) at the lowest
  admissible apex. Triangles keep the reversed loop order, so their normals
  point from the inside to the outside;
* a vertex on the edge from grid point a (lower index) to b sits at
  p_a + t (p_b - p_a), t = (iso - v_a) / (v_b - v_a), in FP32 with one
  rounding per operation; attribute channels 1.. are interpolated with the
  same t. Grid coordinates are the inclusive linspace of the RBF splat
  (rbf2volume_cuda.cu:58-60).

Cells are visited in (z, y, x) order, x fastest; each cell emits its
triangles in table order. The gradient treats the case table (topology) as
constant and differentiates t with respect to v_a and v_b.
"""
import numpy as np

# corner i of a cell sits at (i & 1, (i >> 1) & 1, (i >> 2) & 1)
_CORNERS = [(i & 1, (i >> 1) & 1, (i >> 2) & 1) for i in range(8)]


def _edge_corners(e):
    """Edge e = 4 axis + r: the lower and upper corner indices."""
    axis, r = divmod(e, 4)
    other = [a for a in range(3) if a != axis]
    lo = [0, 0, 0]
    lo[other[0]] = r & 1
    lo[other[1]] = r >> 1
    hi = list(lo)
    hi[axis] = 1
    idx = lambda c: c[0] + 2 * c[1] + 4 * c[2]
    return idx(lo), idx(hi)


EDGES = [_edge_corners(e) for e in range(12)]
_EDGE_OF = {frozenset(EDGES[e]): e for e in range(12)}


def _faces():
    """Each face: its four corners in cyclic order and its outward normal."""
    out = []
    for axis in range(3):
        b, c = [a for a in range(3) if a != axis]
        for side in (0, 1):
            ring = []
            for (u, v) in ((0, 0), (1, 0), (1, 1), (0, 1)):
                p = [0, 0, 0]
                p[axis], p[b], p[c] = side, u, v
                ring.append(p[0] + 2 * p[1] + 4 * p[2])
            n = [0, 0, 0]
            n[axis] = 1 if side else -1
            out.append((ring, n))
    return out


FACES = _faces()
MAX_TRIANGLES = 5  # the derivation below never produces more (asserted in case_table)


def _mid(e):
    a, b = EDGES[e]
    return np.array([(_CORNERS[a][k] + _CORNERS[b][k]) * 0.5 for k in range(3)])


def _case(mask):
    inside = [(mask >> i) & 1 for i in range(8)]
    nxt = {}
    for ring, n in FACES:
        ins = [inside[c] for c in ring]
        if all(ins) or not any(ins):
            continue
        # runs of consecutive inside corners (cyclic); a diagonal pair of
        # inside corners gives two runs of one
        runs = []
        start = next(j for j in range(4) if ins[j] and not ins[j - 1])
        j = start
        for _ in range(4):
            if ins[j] and not ins[j - 1]:
                run = [j]
                k = (j + 1) % 4
                while ins[k]:
                    run.append(k)
                    k = (k + 1) % 4
                runs.append(run)
            j = (j + 1) % 4
        for run in runs:
            first, last = run[0], run[-1]
            e_in = _EDGE_OF[frozenset((ring[first - 1], ring[first]))]
            e_out = _EDGE_OF[frozenset((ring[last], ring[(last + 1) % 4]))]
            # orient so that the run's corners lie on the left seen from outside
            a, b = _mid(e_in), _mid(e_out)
            left = np.cross(np.array(n, float), b - a)
            c = np.array(_CORNERS[ring[first]], float)
            if np.dot(c - a, left) < 0:
                a_e, b_e = e_in, e_out
                e_in, e_out = b_e, a_e
            assert e_in not in nxt
            nxt[e_in] = e_out
    tris = []
    todo = sorted(nxt)
    used = set()
    for e0 in todo:
        if e0 in used:
            continue
        loop = [e0]
        used.add(e0)
        e = nxt[e0]
        while e != e0:
            loop.append(e)
            used.add(e)
            e = nxt[e]
        for (i, k, j) in _triangulate(loop):
            tris.append((loop[i], loop[j], loop[k]))
    return tris


def _faces_of_edge(e):
    a, b = EDGES[e]
    return {f for f, (ring, _) in enumerate(FACES) if a in ring and b in ring}


def _triangulate(loop):
    """Triangles (i, k, j), i < k < j, of the polygon loop[0..L-1] whose
    diagonals join no two points of one cube face."""
    L = len(loop)
    faces = [_faces_of_edge(e) for e in loop]

    def chord_ok(i, j):  # a side of the polygon, or a diagonal off the faces
        return j - i == 1 or (i == 0 and j == L - 1) or not (faces[i] & faces[j])

    def split(i, j):
        if j - i < 2:
            return []
        for k in range(i + 1, j):
            if chord_ok(i, k) and chord_ok(k, j):
                left, right = split(i, k), split(k, j)
                if left is not None and right is not None:
                    return left + [(i, k, j)] + right
        return None

    out = split(0, L - 1)
    assert out is not None, loop
    return out


def case_table():
    """(ntri [256] uint8, edges [256, 3 MAX_TRIANGLES] int8, -1 padded)."""
    ntri = np.zeros(256, np.uint8)
    edges = np.full((256, 3 * MAX_TRIANGLES), -1, np.int8)
    for m in range(256):
        tris = _case(m)
        assert len(tris) <= MAX_TRIANGLES
        ntri[m] = len(tris)
        for t, tri in enumerate(tris):
            edges[m, 3 * t:3 * t + 3] = tri
    return ntri, edges


_TABLE = None


def _table():
    global _TABLE
    if _TABLE is None:
        _TABLE = case_table()
    return _TABLE


def grid_coords(n, lo, hi, dtype):
    """Inclusive linspace of n points as the RBF splat computes it:
    lo + ((hi - lo) * i) / (n - 1), one rounding per operation."""
    lo, hi = dtype(lo), dtype(hi)
    i = np.arange(n).astype(dtype)
    if n == 1:
        return np.full(1, dtype(0.5) * (lo + hi), dtype)
    return (lo + ((hi - lo) * i) / dtype(n - 1)).astype(dtype)


def _cells(volume, iso, dtype):
    v = volume[0].astype(dtype)
    D, H, W = v.shape
    inside = v > dtype(iso)
    mask = np.zeros((max(D - 1, 0), max(H - 1, 0), max(W - 1, 0)), np.int64)
    for i, (cx, cy, cz) in enumerate(_CORNERS):
        mask |= inside[cz:cz + D - 1, cy:cy + H - 1, cx:cx + W - 1].astype(np.int64) << i
    return mask


def marching_cubes(volume, iso, start, end, dtype=np.float32):
    """volume [C, D, H, W] -> (verts [N, 3 + C - 1], edges [N] int64), N = 3 x
    triangles; edges[j] = 12 x (linear cell index, x fastest) + edge id."""
    ntri, table = _table()
    volume = np.asarray(volume)
    C, D, H, W = volume.shape
    mask = _cells(volume, iso, dtype)
    counts = ntri[mask].astype(np.int64)
    cell_ids = np.nonzero(counts.reshape(-1))[0]
    if cell_ids.size == 0:
        return np.zeros((0, 2 + C), dtype), np.zeros(0, np.int64)
    reps = counts.reshape(-1)[cell_ids] * 3
    cell_of = np.repeat(cell_ids, reps)
    slot = np.arange(cell_of.size) - np.repeat(np.cumsum(reps) - reps, reps)
    e = table[mask.reshape(-1)[cell_of], slot].astype(np.int64)
    edges = cell_of * 12 + e
    return _vertices(volume, iso, start, end, edges, dtype), edges


def _endpoints(shape, edges):
    C, D, H, W = shape
    cell, e = np.divmod(edges, 12)
    z, rem = np.divmod(cell, (H - 1) * (W - 1))
    y, x = np.divmod(rem, W - 1)
    ca = np.array([EDGES[k][0] for k in range(12)])[e]
    cb = np.array([EDGES[k][1] for k in range(12)])[e]
    pa = [x + (ca & 1), y + ((ca >> 1) & 1), z + (ca >> 2)]
    pb = [x + (cb & 1), y + ((cb >> 1) & 1), z + (cb >> 2)]
    return pa, pb


def _vertices(volume, iso, start, end, edges, dtype):
    C, D, H, W = volume.shape
    pa, pb = _endpoints(volume.shape, edges)
    vol = volume.astype(dtype)
    va = vol[0][pa[2], pa[1], pa[0]]
    vb = vol[0][pb[2], pb[1], pb[0]]
    t = ((dtype(iso) - va) / (vb - va)).astype(dtype)
    out = np.zeros((edges.size, 2 + C), dtype)
    for k, n in enumerate((W, H, D)):
        g = grid_coords(n, start[k], end[k], dtype)
        a, b = g[pa[k]], g[pb[k]]
        out[:, k] = a + t * (b - a)
    for c in range(1, C):
        a = vol[c][pa[2], pa[1], pa[0]]
        b = vol[c][pb[2], pb[1], pb[0]]
        out[:, 2 + c] = a + t * (b - a)
    return out


def marching_cubes_grad(volume, iso, start, end, edges, verts_grad):
    """d loss / d volume [C, D, H, W] (float64) for verts_grad [N, 3 + C - 1]
    at the vertices of ``edges`` (case table held constant)."""
    volume = np.asarray(volume, np.float64)
    C, D, H, W = volume.shape
    g = np.asarray(verts_grad, np.float64)
    out = np.zeros_like(volume)
    if edges.size == 0:
        return out
    pa, pb = _endpoints(volume.shape, edges)
    va = volume[0][pa[2], pa[1], pa[0]]
    vb = volume[0][pb[2], pb[1], pb[0]]
    den = vb - va
    t = (iso - va) / den
    gt = np.zeros(edges.size)
    for k, n in enumerate((W, H, D)):
        c = grid_coords(n, start[k], end[k], np.float64)
        gt += g[:, k] * (c[pb[k]] - c[pa[k]])
    for ch in range(1, C):
        a = volume[ch][pa[2], pa[1], pa[0]]
        b = volume[ch][pb[2], pb[1], pb[0]]
        gt += g[:, 2 + ch] * (b - a)
        np.add.at(out[ch], (pa[2], pa[1], pa[0]), g[:, 2 + ch] * (1 - t))
        np.add.at(out[ch], (pb[2], pb[1], pb[0]), g[:, 2 + ch] * t)
    np.add.at(out[0], (pa[2], pa[1], pa[0]), gt * (iso - vb) / (den * den))
    np.add.at(out[0], (pb[2], pb[1], pb[0]), -gt * (iso - va) / (den * den))
    return out
