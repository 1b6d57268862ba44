"""Shaded preview rasteriser oracle on the CPU: the camera matrices, coverage
of a square (including pytorch3d's strict inside rule on a shared edge), the
Phong colour of a lit face against the lighting formula, the nearest-face
rule and faces behind the camera."""
import math

import numpy as np
import pytest

import oracle
from totri_gb300.util.render import UnitCubeMeshRender, fov_focal, look_at_view_transform


def settings_of(renderer):
    s = renderer.shading
    out = {}
    for name, _ in s._fields_:
        v = getattr(s, name)
        out[name] = list(v) if hasattr(v, "__len__") else v
    return out


def test_camera_matrices():
    R, T = look_at_view_transform([0.0, 0.0, -0.5])
    assert np.allclose(R.numpy(), np.eye(3)) and np.allclose(T.numpy(), [0, 0, 0.5])
    # an eye on +x looking at (0, 0, 1): view z points from the eye to the target
    R, T = look_at_view_transform([1.0, 0.0, 1.0])
    eye = np.array([1.0, 0.0, 1.0])
    assert np.allclose(R.numpy()[:, 2], [-1, 0, 0], atol=1e-6)
    assert np.allclose(eye @ R.numpy() + T.numpy(), 0, atol=1e-6)
    fx, fy = fov_focal(60.0, 0.1, 1.0)
    assert fx == fy and abs(fx - 1 / math.tan(math.pi / 6)) < 1e-6
    s = settings_of(UnitCubeMeshRender(resolution=8, distance=0.7))
    assert np.allclose(s["camera_center"], [0, 0, -0.7], atol=1e-6)


def _square(z=1.0, h=0.2, flip=False):
    v = np.array([[-h, -h, z], [h, -h, z], [h, h, z], [-h, h, z]], np.float32)
    f = np.array([[0, 2, 1], [0, 3, 2]]) if flip else np.array([[0, 1, 2], [0, 2, 3]])
    return v, f


def test_square_coverage_and_shared_edge():
    s = settings_of(UnitCubeMeshRender(resolution=64))
    v, f = _square()
    img, face = oracle.shaded_raster(v, f, np.ones((1, 3)), 64, 64, s)
    # half-width 0.2 * focal / 1.5 in ndc: 7 pixel centres each side of the axis,
    # 14 x 14 pixels less the 14 centres exactly on the shared diagonal
    assert (face >= 0).sum() == 14 * 14 - 14
    assert face[32, 32] == -1 and face[30, 33] >= 0
    assert np.all(img[:, face < 0] == 1.0)


@pytest.mark.parametrize("flip", [False, True])
def test_phong_colour_of_a_face(flip):
    s = settings_of(UnitCubeMeshRender(resolution=64, specular=0.3))
    v, f = _square(flip=flip)
    colour = np.array([0.9, 0.6, 0.3])
    img, face = oracle.shaded_raster(v, f, colour[None], 64, 64, s)
    r, c = 30, 36
    assert face[r, c] >= 0
    # the ray through the pixel centre meets the plane z = 1 (view depth 1.5)
    ndc_x = 1 - (2 * c + 1) / 64
    ndc_y = 1 - (2 * r + 1) / 64
    P = np.array([ndc_x * 1.5 / s["focal"][0], ndc_y * 1.5 / s["focal"][1], 1.0])
    n = np.array([0, 0, -1.0 if flip else 1.0])
    L = np.array([2.0, 2, -2]) - P
    L /= np.linalg.norm(L)
    E = np.array([0, 0, -0.5]) - P
    E /= np.linalg.norm(E)
    cs = n @ L
    Rf = 2 * cs * n - L
    spec = (max(E @ Rf, 0) * (cs > 0)) ** 64
    want = (0.5 + 0.3 * max(cs, 0)) * colour + 0.3 * spec
    assert np.allclose(img[:, r, c], want, atol=2e-6)
    assert (cs > 0) == flip  # the winding decides the lit side


def test_nearest_face_and_behind_camera():
    s = settings_of(UnitCubeMeshRender(resolution=32))
    v1, f1 = _square(z=1.0, h=0.3)
    v2, f2 = _square(z=0.8, h=0.1)
    v3, f3 = _square(z=-1.0, h=5.0)  # behind the eye (view z < 0): never drawn
    v = np.concatenate([v1, v2, v3])
    f = np.concatenate([f1, f2 + 4, f3 + 8])
    _, face = oracle.shaded_raster(v, f, np.ones((1, 3)), 32, 32, s)
    assert set(np.unique(face)) <= {-1, 0, 1, 2, 3}
    assert face[15, 16] in (2, 3)  # the nearer, smaller square
    assert face[12, 16] in (0, 1)  # outside it: the larger one behind
    # equal depths: the lower face index wins
    _, face2 = oracle.shaded_raster(np.concatenate([v2, v2]), np.concatenate([f2, f2 + 4]),
                                    np.ones((1, 3)), 32, 32, s)
    assert set(np.unique(face2)) == {-1, 0, 1}
