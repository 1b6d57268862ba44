"""CPU oracle for the shaded perspective rasteriser (TEST INFRASTRUCTURE).

Restates csrc/shade.cu: the decisions (vertex projection, coverage, the
perspective-corrected barycentrics, depth and the nearest face) in numpy FP32
with the kernel's operation order and one rounding per operation, so that the
face map is bit-exact; the shading values (vertex normals, interpolation,
Phong lighting, blend) in FP64. The reference's renderer is pytorch3d's
(totri/util/render.py:17-81: FoVPerspectiveCameras, MeshRasterizer with one
face per pixel and no blur, SoftPhongShader), which is not installed here, so
parity is unpinned against it: this oracle pins the kernels to the restated
rules only.

``settings`` is a dict with the fields of totri_shading_t (rotation [9]
row-major, translation, focal, znear, zfar, camera_center, light_location,
light_ambient, light_diffuse, light_specular, material_ambient,
material_diffuse, material_specular, shininess, background, sigma, gamma).
"""
import numpy as np

f32 = np.float32
EPS = f32(1e-8)


def _edge(px, py, ax, ay, bx, by):
    return f32(f32(f32(px - ax) * f32(by - ay)) - f32(f32(py - ay) * f32(bx - ax)))


def _pix_ndc(i, S1, S2):
    n = f32(f32(-1) + f32(f32(2 * i + 1) / f32(S1)))
    if S1 > S2:
        n = f32(f32(n * f32(S1)) / f32(S2))
    return n


def project(verts, settings):
    """[V, 4] (ndc x, ndc y, view z, 0) of every vertex, FP32."""
    v = np.asarray(verts, np.float32)
    R = np.asarray(settings["rotation"], np.float32).reshape(3, 3)
    T = np.asarray(settings["translation"], np.float32)
    view = []
    for i in range(3):
        a = f32(v[:, 0] * R[0, i])
        a = f32(a + f32(v[:, 1] * R[1, i]))
        a = f32(a + f32(v[:, 2] * R[2, i]))
        view.append(f32(a + T[i]))
    fx, fy = (f32(x) for x in settings["focal"])
    with np.errstate(all="ignore"):
        nx = f32(f32(fx * view[0]) / view[2])
        ny = f32(f32(fy * view[1]) / view[2])
    return np.stack([nx, ny, view[2], np.zeros_like(nx)], axis=1).astype(np.float32)


def _bary(px, py, a, b, c):
    area = f32(_edge(c[0], c[1], a[0], a[1], b[0], b[1]) + EPS)
    w0 = f32(_edge(px, py, b[0], b[1], c[0], c[1]) / area)
    w1 = f32(_edge(px, py, c[0], c[1], a[0], a[1]) / area)
    w2 = f32(_edge(px, py, a[0], a[1], b[0], b[1]) / area)
    t0 = f32(f32(w0 * b[2]) * c[2])
    t1 = f32(f32(a[2] * w1) * c[2])
    t2 = f32(f32(a[2] * b[2]) * w2)
    d = np.fmax(f32(f32(t0 + t1) + t2), EPS).astype(np.float32)
    return f32(t0 / d), f32(t1 / d), f32(t2 / d)


def rasterize(verts, faces, H, W, settings):
    """(pix_to_face [H, W] int64, depth [H, W] FP32, inf where empty)."""
    fc = np.asarray(faces, np.int64)
    V = np.asarray(verts).shape[0]
    proj = project(verts, settings)
    xs = np.array([_pix_ndc(i, W, H) for i in range(W)], np.float32)  # by ndc index
    ys = np.array([_pix_ndc(i, H, W) for i in range(H)], np.float32)
    PX, PY = np.meshgrid(xs, ys)  # [yi, xi]
    depth = np.full((H, W), np.inf, np.float32)
    face = np.full((H, W), -1, np.int64)
    for k in range(fc.shape[0]):
        idx = fc[k]
        if np.any(idx < 0) or np.any(idx >= V):
            continue
        a, b, c = proj[idx[0]], proj[idx[1]], proj[idx[2]]
        if np.fmax(np.fmax(a[2], b[2]), c[2]) < 0:
            continue
        area = _edge(a[0], a[1], b[0], b[1], c[0], c[1])
        if area <= EPS and area >= -EPS:
            continue
        xmin = np.fmin(np.fmin(a[0], b[0]), c[0])
        xmax = np.fmax(np.fmax(a[0], b[0]), c[0])
        ymin = np.fmin(np.fmin(a[1], b[1]), c[1])
        ymax = np.fmax(np.fmax(a[1], b[1]), c[1])
        if not (xmin <= xmax and ymin <= ymax):
            continue
        box = (PX <= xmax) & (PX >= xmin) & (PY <= ymax) & (PY >= ymin)
        if not box.any():
            continue
        yy, xx = np.nonzero(box)
        px, py = PX[yy, xx], PY[yy, xx]
        with np.errstate(all="ignore"):
            b0, b1, b2 = _bary(px, py, a, b, c)
            pz = f32(f32(f32(b0 * a[2]) + f32(b1 * b[2])) + f32(b2 * c[2]))
        ok = (pz >= 0) & (b0 > 0) & (b1 > 0) & (b2 > 0)
        rows, cols = H - 1 - yy[ok], W - 1 - xx[ok]
        z = f32(pz[ok] + f32(0))
        better = z < depth[rows, cols]  # faces in index order: ties keep the lower
        depth[rows[better], cols[better]] = z[better]
        face[rows[better], cols[better]] = k
    return face, depth


def vertex_normals(verts, faces):
    """Unit vertex normals [V, 3] (FP64): each the normalised sum over its
    faces of (v2 - v1) x (v0 - v1)."""
    v = np.asarray(verts, np.float64)
    fc = np.asarray(faces, np.int64)
    ok = np.all((fc >= 0) & (fc < v.shape[0]), axis=1)
    fc = fc[ok]
    n = np.cross(v[fc[:, 2]] - v[fc[:, 1]], v[fc[:, 0]] - v[fc[:, 1]])
    acc = np.zeros_like(v)
    for k in range(3):
        np.add.at(acc, fc[:, k], n)
    return acc / np.maximum(np.linalg.norm(acc, axis=1, keepdims=True), 1e-6)


def _seg_dist2(p, a, b):
    e = b - a
    q = p - a
    bot = (e * e).sum(-1)
    with np.errstate(all="ignore"):
        t = np.where(bot > 1e-8, (e * q).sum(-1) / bot, 0.0)
    t = np.clip(t, 0.0, 1.0)[..., None]
    d = p - ((1 - t) * a + t * b)
    return (d * d).sum(-1)


def _unit(x):
    return x / np.maximum(np.linalg.norm(x, axis=-1, keepdims=True), 1e-6)


def shaded_raster(verts, faces, colors, H, W, settings):
    """(image [3, H, W] FP64, pix_to_face [H, W] int64)."""
    s = {k: np.asarray(v, np.float64) for k, v in settings.items()}
    face, depth = rasterize(verts, faces, H, W, settings)
    v32 = np.asarray(verts, np.float32)
    v = v32.astype(np.float64)
    fc = np.asarray(faces, np.int64)
    col = np.broadcast_to(np.asarray(colors, np.float64), v.shape)
    nrm = vertex_normals(v32, fc)
    proj = project(v32, settings)
    img = np.empty((3, H, W), np.float64)
    img[:] = s["background"][:, None, None]
    rows, cols = np.nonzero(face >= 0)
    if rows.size == 0:
        return img, face
    f = face[rows, cols]
    idx = fc[f]  # [n, 3]
    px = np.array([_pix_ndc(W - 1 - c, W, H) for c in cols], np.float32)
    py = np.array([_pix_ndc(H - 1 - r, H, W) for r in rows], np.float32)
    a, b, c = proj[idx[:, 0]].T, proj[idx[:, 1]].T, proj[idx[:, 2]].T
    with np.errstate(all="ignore"):
        b0, b1, b2 = _bary(px, py, a, b, c)
    w = np.stack([b0, b1, b2], axis=1).astype(np.float64)[..., None]  # [n, 3, 1]
    P = (w * v[idx]).sum(1)
    N = _unit((w * nrm[idx]).sum(1))
    C = (w * col[idx]).sum(1)
    L = _unit(s["light_location"] - P)
    E = _unit(s["camera_center"] - P)
    cs = (N * L).sum(-1)
    Rf = 2 * cs[:, None] * N - L
    er = np.maximum((E * Rf).sum(-1), 0) * (cs > 0)
    spec = er ** s["shininess"]
    diff = np.maximum(cs, 0)
    shaded = (s["material_ambient"] * s["light_ambient"]
              + s["material_diffuse"] * s["light_diffuse"] * diff[:, None]) * C \
        + s["material_specular"] * s["light_specular"] * spec[:, None]
    pp = np.stack([px, py], 1).astype(np.float64)
    A, B, Cc = a[:2].T.astype(np.float64), b[:2].T.astype(np.float64), c[:2].T.astype(np.float64)
    d = np.minimum(np.minimum(_seg_dist2(pp, A, B), _seg_dist2(pp, B, Cc)), _seg_dist2(pp, Cc, A))
    prob = 1 / (1 + np.exp(-d / s["sigma"]))
    zinv = np.maximum((s["zfar"] - depth[rows, cols]) / (s["zfar"] - s["znear"]), 1e-10)
    delta = np.maximum(np.exp((1e-10 - zinv) / s["gamma"]), 1e-10)
    out = (prob[:, None] * shaded + delta[:, None] * s["background"]) / (prob + delta)[:, None]
    img[:, rows, cols] = out.T
    return img, face
