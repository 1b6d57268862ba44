"""Golden vectors for the fitting loops' learned backgrounds, from the
reference's own modules (totri/fitting/background.py, plain PyTorch): the
file is loaded directly from the reference tree, each module is built with
seeded weights and evaluated on seeded wall points; weights, inputs and
outputs go to tests/golden/background.npz.

Run: python tests/golden/make_golden_background.py [reference root]
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


def main():
    path = os.path.join(REF, "totri", "fitting", "background.py")
    spec = importlib.util.spec_from_file_location("ref_background", path)
    bg = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(bg)
    torch.manual_seed(3)
    out = {}
    conf = bg.TransientBackgroundConfocal(40, wall_start=(-1, -0.8), wall_end=(1.2, 1))
    ex = bg.TransientBackgroundExhaustive(24, wall_start=(-1, -1), wall_end=(1, 1))
    g = torch.Generator().manual_seed(5)
    sp = torch.rand((2, 7, 3), generator=g) * 2 - 1
    lp = torch.rand((2, 3, 3), generator=g) * 2 - 1
    with torch.no_grad():
        conf.intensity[:] = 1.7
        out["conf_out"] = conf(sp).numpy()
        out["ex_out"] = ex(sp, lp).numpy()
    for name, m in (("conf", conf), ("ex", ex)):
        for k, v in m.state_dict().items():
            out["%s.%s" % (name, k)] = v.numpy()
    out["scan"] = sp.numpy()
    out["laser"] = lp.numpy()
    np.savez_compressed(os.path.join(HERE, "background.npz"), **out)
    print(sorted(out))


if __name__ == "__main__":
    main()
