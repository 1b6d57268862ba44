"""Golden vectors for f-k migration from the reference's own implementation.

The reference's f-k migration (totri/reconstruct/fk_migration.py) is plain
PyTorch; this script loads that file directly from the reference tree (the
package itself does not import here: totri/util pulls in pytorch3d and cv2),
runs it on the CPU on seeded inputs and stores inputs and outputs in
tests/golden/fk_migration.npz.

Run: python tests/golden/make_golden_fk.py [reference root]
"""
import importlib.util
import os
import sys

import numpy as np
import torch

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
from oracle.ref_harness import REF_ROOT  # noqa: E402

REF = sys.argv[1] if len(sys.argv) > 1 else REF_ROOT


def load():
    path = os.path.join(REF, "totri", "reconstruct", "fk_migration.py")
    spec = importlib.util.spec_from_file_location("ref_fk_migration", path)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def main():
    fk = load()
    g = torch.Generator().manual_seed(11)
    out = {}
    cases = [((32, 16, 16), (0.64, 2.0, 2.0)), ((20, 9, 12), (0.5, 1.6, 2.2))]
    for i, (shape, dims) in enumerate(cases):
        tr = torch.rand((1,) + shape, generator=g) ** 4
        vol = fk.FkMigration(*dims)(tr)
        out["transient_%d" % i] = tr.numpy()
        out["dims_%d" % i] = np.array(dims, np.float64)
        out["volume_%d" % i] = vol.numpy()
    # the Stolt resampling alone, on a complex volume [N, C, 2D, H, W]
    re = torch.randn((1, 2, 24, 10, 7), generator=g)
    im = torch.randn((1, 2, 24, 10, 7), generator=g)
    f = torch.complex(re, im)
    s = fk.StoltInterpolation(0.7, 1.9, 2.3)(f)
    out["stolt_in"] = torch.view_as_real(f).numpy()
    out["stolt_dims"] = np.array((0.7, 1.9, 2.3), np.float64)
    out["stolt_out"] = torch.view_as_real(s).numpy()
    np.savez_compressed(os.path.join(HERE, "fk_migration.npz"), **out)
    print({k: v.shape for k, v in out.items()})


if __name__ == "__main__":
    main()
