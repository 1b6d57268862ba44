"""Helpers shared by the mesh tests."""
import numpy as np


def unpack_mask(words, num_faces):
    """int32 words [P, ceil(F/32)] -> uint8 [P, F] (bit f % 32 of word f // 32)."""
    w = np.ascontiguousarray(words).view(np.uint32)
    bits = (w[:, :, None] >> np.arange(32, dtype=np.uint32)) & np.uint32(1)
    return bits.astype(np.uint8).reshape(w.shape[0], -1)[:, :num_faces]


def rel_l2(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def np_scene(s):
    """numpy views of a single-item scene dict (batch index 0)."""
    out = {}
    for k in ("verts", "faces", "colors", "scan_points", "laser_points"):
        if k in s:
            out[k] = s[k][0].cpu().numpy()
    return out
