"""Orthographic depth rasteriser oracle on the CPU: a plane's depth, a
sphere's covered area, and the nearest-face rule."""
import numpy as np

import oracle
from totri_gb300 import scenes


def test_tilted_plane_depth_and_coverage():
    # square [-0.5, 0.5]^2 at z = 1 + 0.2 x, two triangles
    v = np.array([[-0.5, -0.5, 0.9], [0.5, -0.5, 1.1], [0.5, 0.5, 1.1], [-0.5, 0.5, 0.9]],
                 np.float32)
    f = np.array([[0, 1, 2], [0, 2, 3]])
    depth, mask = oracle.depth_raster(v, f, 32, 32, -1, 1, -1, 1, 0, 2)
    assert mask.sum() == 16 * 16
    j = np.arange(32)
    x = 1 - (j + 0.5) * (2 / 32)
    cols = mask.any(0)
    assert np.allclose(depth[16, cols], 1 + 0.2 * x[cols], atol=1e-6)
    assert np.all(depth[~mask] == -1)


def test_sphere_area_and_nearest_surface():
    s = scenes.confocal_small()
    v, f = s["verts"][0].numpy(), s["faces"][0].numpy()
    depth, mask = oracle.depth_raster(v, f, 96, 96, -1, 1, -1, 1, 0, 2)
    pix = (2 / 96) ** 2
    assert abs(mask.sum() * pix / (np.pi * 0.3 ** 2) - 1) < 0.05
    # the near side (z ~ 0.7 at the centre), not the far side
    assert abs(depth[48, 48] - 0.7) < 0.03
