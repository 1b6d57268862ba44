"""Shaded preview rasteriser on the GPU against the oracle: the face map bit
for bit (FP32 decisions, one rounding per operation on both sides) and the
image within rel-L2 1e-5 of the FP64 shading, square and non-square images,
the volume-box mapping and the default faces and colours."""
import ctypes

import numpy as np
import pytest
import torch

import oracle
from totri_gb300 import _lib, scenes
from totri_gb300.types import VolumeDef
from totri_gb300.util import UnitCubeMeshRender

from test_shaded_raster import settings_of

pytestmark = pytest.mark.gpu


def _scene(seed=2):
    s = scenes.displaced_sphere(3, 4)
    v, f = s[0][0].numpy(), s[1][0].numpy()
    g = np.random.default_rng(seed)
    soup = g.uniform(-0.6, 0.6, (300, 3)).astype(np.float32)
    soup[:, 2] = g.uniform(0.3, 1.6, 300)
    verts = np.concatenate([v, soup]).astype(np.float32)
    faces = np.concatenate([f, v.shape[0] + np.arange(300).reshape(100, 3)])
    colors = g.uniform(0.2, 1.0, (verts.shape[0], 3)).astype(np.float32)
    return verts, faces, colors


def _compare(img, pix, ref_img, ref_face):
    assert np.array_equal(pix, ref_face)
    err = np.linalg.norm(img - ref_img) / np.linalg.norm(ref_img)
    assert err < 1e-5, err
    assert np.abs(img - ref_img).max() < 1e-4


@pytest.mark.parametrize("res", [64, 97])
def test_matches_oracle(cuda_lib, res):
    verts, faces, colors = _scene()
    r = UnitCubeMeshRender(resolution=res, specular=0.4)
    img, pix = r.render(torch.tensor(verts).cuda(), torch.tensor(faces).cuda(),
                        torch.tensor(colors).cuda())
    ref_img, ref_face = oracle.shaded_raster(verts, faces, colors, res, res, settings_of(r))
    assert 0.1 < (ref_face >= 0).mean() < 0.9
    _compare(img.cpu().numpy(), pix.cpu().numpy(), ref_img, ref_face)


@pytest.mark.parametrize("hw", [(48, 80), (81, 40)])
def test_non_square_image(cuda_lib, hw):
    H, W = hw
    verts, faces, colors = _scene(3)
    r = UnitCubeMeshRender(resolution=8, eye=[0.3, -0.2, -0.6])
    v, f = torch.tensor(verts).cuda(), torch.tensor(faces).cuda()
    c = torch.tensor(colors).cuda()
    img = torch.empty((3, H, W), device="cuda")
    pix = torch.empty((H, W), dtype=torch.int32, device="cuda")
    n = int(cuda_lib.totri_shaded_raster_workspace(v.shape[0], H, W))
    ws = torch.empty(n, dtype=torch.uint8, device="cuda")
    _lib.check(cuda_lib.totri_shaded_raster(
        _lib.array(v), _lib.array(f), _lib.array(c), ctypes.byref(r.shading), _lib.array(img),
        _lib.array(pix), ctypes.c_void_p(ws.data_ptr()), n, _lib.stream_of(v.device)))
    ref_img, ref_face = oracle.shaded_raster(verts, faces, colors, H, W, settings_of(r))
    _compare(img.cpu().numpy(), pix.cpu().numpy(), ref_img, ref_face)


def test_volume_box_and_defaults(cuda_lib):
    g = np.random.default_rng(5)
    soup = g.uniform(-0.4, 0.4, (600, 3)).astype(np.float32)
    soup[:, 2] = g.uniform(0.6, 1.4, 600)
    vd = VolumeDef((-0.5, -0.5, 0.5), (0.5, 0.5, 1.5), (8, 8, 8))
    r = UnitCubeMeshRender(resolution=72)
    v = torch.tensor(soup).cuda()
    img, pix = r.render(v, volume_def=vd)  # consecutive triples, white vertices
    mapped = UnitCubeMeshRender.fit_volume(v, vd).cpu().numpy()
    faces = np.arange(600).reshape(200, 3)
    ref_img, ref_face = oracle.shaded_raster(mapped, faces, np.ones((1, 3)), 72, 72,
                                             settings_of(r))
    assert (ref_face >= 0).mean() > 0.05
    _compare(img.cpu().numpy(), pix.cpu().numpy(), ref_img, ref_face)
    assert torch.equal(r.apply(v, volume_def=vd), img)
