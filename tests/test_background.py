"""The fitting loops' learned backgrounds against the reference's own modules
evaluated with the same weights (tests/golden/background.npz)."""
import os

import numpy as np
import torch

from totri_gb300.fitting.background import (TransientBackgroundConfocal,
                                            TransientBackgroundExhaustive)

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "background.npz")


def _load(module, g, prefix):
    state = {k[len(prefix) + 1:]: torch.tensor(g[k]) for k in g.files
             if k.startswith(prefix + ".")}
    module.load_state_dict(state)


def test_backgrounds_match_reference():
    g = np.load(GOLDEN)
    conf = TransientBackgroundConfocal(40, wall_start=(-1, -0.8), wall_end=(1.2, 1))
    ex = TransientBackgroundExhaustive(24, wall_start=(-1, -1), wall_end=(1, 1))
    _load(conf, g, "conf")
    _load(ex, g, "ex")
    sp, lp = torch.tensor(g["scan"]), torch.tensor(g["laser"])
    with torch.no_grad():
        assert np.allclose(conf(sp).numpy(), g["conf_out"], rtol=1e-5, atol=1e-7)
        assert np.allclose(ex(sp, lp).numpy(), g["ex_out"], rtol=1e-5, atol=1e-7)


def test_clamp_caps_background_energy():
    conf = TransientBackgroundConfocal(16)
    fg = torch.ones(16, 5)
    conf.clamp_parameters(fg, 3 * torch.ones(16, 5))
    assert abs(float(conf.intensity.detach()) - 1 / 3) < 1e-6
