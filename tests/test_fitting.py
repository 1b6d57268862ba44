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
