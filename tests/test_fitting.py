"""Pose-fitting building blocks on the CPU: the quaternion rotation against the
rotation matrix of the same unit quaternion, the normalising Rotation module,
Translation, and the mesh merge used by the fit."""
import numpy as np
import torch

from totri_gb300.data.util import merge_meshes
from totri_gb300.fitting import Rotation, Translation, apply_transform, quaternion_apply


def _matrix(q):
    w, x, y, z = q
    return np.array([
        [1 - 2 * (y * y + z * z), 2 * (x * y - w * z), 2 * (x * z + w * y)],
        [2 * (x * y + w * z), 1 - 2 * (x * x + z * z), 2 * (y * z - w * x)],
        [2 * (x * z - w * y), 2 * (y * z + w * x), 1 - 2 * (x * x + y * y)]])


def test_quaternion_apply_is_the_rotation_matrix():
    g = np.random.default_rng(0)
    for _ in range(5):
        q = g.standard_normal(4)
        q /= np.linalg.norm(q)
        p = g.standard_normal((7, 3))
        got = quaternion_apply(torch.tensor(q)[None], torch.tensor(p)).numpy()
        assert np.allclose(got, p @ _matrix(q).T, atol=1e-12)


def test_rotation_normalises_and_translation_adds():
    rot = Rotation((2.0, 0.0, 0.0, 2.0), device="cpu")  # 90 degrees about z
    tr = Translation((0.1, -0.2, 0.3), device="cpu")
    p = torch.tensor([[1.0, 0.0, 0.0]])
    out = apply_transform([p], [tr], [rot])[0]
    assert torch.allclose(out, torch.tensor([[0.1, 0.8, 0.3]]), atol=1e-6)
    out.sum().backward()
    assert rot.quaternion.grad is not None and tr.translation.grad is not None


def test_merge_meshes_offsets_faces():
    v0, v1 = torch.zeros(4, 3), torch.ones(5, 3)
    f0 = torch.tensor([[0, 1, 2]])
    f1 = torch.tensor([[0, 1, 2], [2, 3, 4]])
    v, f = merge_meshes([v0, v1], [f0, f1])
    assert v.shape == (9, 3)
    assert f.tolist() == [[0, 1, 2], [4, 5, 6], [6, 7, 8]]


def test_depth_map_geometry_and_clamps():
    from totri_gb300.fitting import DepthMap
    from totri_gb300.types import VolumeDef
    dm = DepthMap(VolumeDef((-0.5, -0.5, 0.5), (0.5, 0.5, 1.5), (8, 4, 5)), device="cpu")
    v = dm.verts()
    assert v.shape == (20, 3) and dm.faces.shape == (24, 3)
    assert v[:5, 0].tolist() == [-0.5, -0.25, 0.0, 0.25, 0.5]
    assert abs(float(v[5, 1]) - (-0.5 + 1 / 3)) < 1e-6
    assert torch.all(v[:, 2] == 1.0)
    assert dm.faces[:2].tolist() == [[0, 6, 1], [0, 5, 6]]
    with torch.no_grad():
        dm.depth[:] = 2.0
        dm.color[:] = 4.0
    intensity = torch.ones(1)
    dm.clamp_params(intensity)
    assert dm.depth[1, 1] == 1.0 and dm.depth[0, 0] == 0.5
    assert dm.color[1, 1] == 1.0 and float(intensity) == 4.0


def test_tv_loss_and_blur():
    from totri_gb300.fitting import tv_loss
    from totri_gb300.fitting.depth_map import gaussian_blur
    assert abs(float(tv_loss(torch.ones(6, 7)))) < 1e-7
    t = torch.zeros(4, 4)
    t[1, 1] = 1.0
    # nonzero differences: dx at (1,0) and (1,1), dy at (0,1) and (1,1)
    eps = 1e-3
    expect = (2 * (1 + eps) ** 0.5 + (2 + eps) ** 0.5 - 3 * eps ** 0.5) / 16
    assert abs(float(tv_loss(t)) - expect) < 1e-6
    img = torch.rand(2, 11, 13, dtype=torch.float64)
    out = gaussian_blur(img, 9)
    assert out.shape == img.shape
    assert torch.allclose(gaussian_blur(torch.ones(1, 9, 9), 9), torch.ones(1, 9, 9))
    assert abs(float(out.mean() - img.mean())) < 0.05


def test_optimizer_schedule():
    from totri_gb300.util.optim import (LinearInterpolator, MultiplicativeInterpolator,
                                        TotriOptimizer)
    p = torch.zeros(2, requires_grad=True)
    opt = TotriOptimizer([p], 1.0, warmup=3)
    assert opt.lr == (1 / 4) ** 2
    rates = []
    for _ in range(4):
        p.sum().backward()
        opt.step()
        rates.append(opt.optim.param_groups[0]["lr"])
    assert rates == [(2 / 4) ** 2, (3 / 4) ** 2, 1.0, 1.0]
    lin = LinearInterpolator(1.0, 3.0, 5)
    assert [lin(i) for i in (0, 2, 4, 9)] == [1.0, 2.0, 3.0, 3.0]
    mul = MultiplicativeInterpolator(1.0, 0.0, 0.5)
    assert [mul(0), mul(0)] == [0.5, 0.25]


def test_rbf_fitting_reduce_transient_crops_silent_bins():
    """Bin cropping of RbfFitting.reduce_transient (reference rbf.py:218-243):
    bins whose 0.95-quantile stays below a tenth of the largest are cut from
    both ends, widened by the margin; the bin definition follows."""
    from totri_gb300.fitting import RbfFitting
    from totri_gb300.types import BinDef
    tr = torch.zeros((400, 16))
    tr[150:201] = torch.linspace(1.0, 2.0, 16)
    tr[120] = 0.1  # below the threshold: still cropped
    fit = RbfFitting(BinDef(0.01, 0.5, 400), torch.zeros((16, 3)))
    out = fit.reduce_transient(tr)
    assert (fit.bin_def.num, out.shape[0]) == (115, 115)
    assert abs(fit.bin_def.offset - (0.5 + 0.01 * 118)) < 1e-9
    assert torch.equal(out, tr[118:233])
    out = fit.reduce_transient(tr, margin=0)
    assert out.shape[0] == 51 and torch.equal(out, tr[150:201])
