"""CPU oracle for the orthographic depth rasteriser (TEST INFRASTRUCTURE).

Restates the rasteriser of csrc/raster.cu in numpy FP32 with the same
operation order (one rounding per operation): for every pixel centre,
x = max_x - (j + 1/2) sx, y = max_y - (i + 1/2) sy, every face whose edge
functions at the centre are all >= 0 or all <= 0 (non-degenerate faces)
contributes its z interpolated with those edge functions, kept within
[znear, zfar] and >= 0; the nearest wins, the lower face index on ties.
The reference's rasteriser is pytorch3d's (totri/util/depthmap.py:6-36),
which is not installed here: parity is unpinned against it.
"""
import numpy as np

f32 = np.float32


def _edge(ax, ay, bx, by, px, py):
    return f32(f32(f32(bx - ax) * f32(py - ay)) - f32(f32(by - ay) * f32(px - ax)))


def depth_raster(verts, faces, H, W, min_x, max_x, min_y, max_y, znear, zfar):
    v = np.asarray(verts, np.float32)
    fc = np.asarray(faces, np.int64)
    sx = f32(f32(f32(max_x) - f32(min_x)) / f32(W))
    sy = f32(f32(f32(max_y) - f32(min_y)) / f32(H))
    px = f32(max_x) - f32(f32(np.arange(W, dtype=np.float32) + f32(0.5)) * sx)
    py = f32(max_y) - f32(f32(np.arange(H, dtype=np.float32) + f32(0.5)) * sy)
    PX, PY = np.meshgrid(px.astype(np.float32), py.astype(np.float32))
    depth = np.full((H, W), np.inf, np.float32)
    face = np.full((H, W), -1, np.int64)
    for k in range(fc.shape[0]):
        idx = fc[k]
        if np.any(idx < 0) or np.any(idx >= v.shape[0]):
            continue
        x, y, z = v[idx, 0], v[idx, 1], v[idx, 2]
        area = _edge(x[0], y[0], x[1], y[1], x[2], y[2])
        if area == 0 or not np.isfinite(area):
            continue
        w0 = _edge(x[1], y[1], x[2], y[2], PX, PY)
        w1 = _edge(x[2], y[2], x[0], y[0], PX, PY)
        w2 = _edge(x[0], y[0], x[1], y[1], PX, PY)
        inside = ((w0 >= 0) & (w1 >= 0) & (w2 >= 0)) | ((w0 <= 0) & (w1 <= 0) & (w2 <= 0))
        with np.errstate(all="ignore"):
            zz = f32(f32(f32(f32(w0 * z[0]) + f32(w1 * z[1])) + f32(w2 * z[2])) / area)
        ok = inside & (zz >= znear) & (zz <= zfar) & (zz >= 0)
        better = ok & (zz < depth)  # faces are visited in index order: ties keep the lower
        depth[better] = zz[better]
        face[better] = k
    mask = face >= 0
    return np.where(mask, depth, np.float32(-1)), mask
