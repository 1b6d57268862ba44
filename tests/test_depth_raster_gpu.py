"""Orthographic depth rasteriser on the GPU against the numpy oracle: depth
and mask bit for bit (FP32, one rounding per operation on both sides)."""
import numpy as np
import pytest
import torch

import oracle
from totri_gb300 import scenes
from totri_gb300.util import UnitDepthMapRender

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("res", [64, 97])
def test_matches_oracle(cuda_lib, res):
    s = scenes.displaced_sphere(3, 4)
    v, f = s[0][0], s[1][0]
    g = np.random.default_rng(2)
    soup = g.uniform(-0.8, 0.8, (300, 3)).astype(np.float32)
    soup[:, 2] = g.uniform(0.2, 1.8, 300)
    verts = np.concatenate([v.numpy(), soup])
    faces = np.concatenate([f.numpy(), v.shape[0] + np.arange(300).reshape(100, 3)])
    r = UnitDepthMapRender(resolution=res, xysize=2, znear=0, zfar=2)
    depth, mask = r.apply(torch.tensor(verts).cuda(), torch.tensor(faces).cuda())
    ref_d, ref_m = oracle.depth_raster(verts, faces, res, res, -1, 1, -1, 1, 0, 2)
    assert np.array_equal(mask.cpu().numpy(), ref_m)
    assert np.array_equal(depth.cpu().numpy(), ref_d)
    assert 0.1 < ref_m.mean() < 0.9
