"""Golden vectors for the MATLAB-format dataset loaders, from the
reference's own loaders (totri/data/veltennc2012.py, otooleconfocal2018.py).

Small synthetic files in the two formats are written to tests/golden/ and
read by the reference's loader modules, loaded directly from the reference
tree with the reference's own totri/types.py and totri/data/util.py standing
in for the package (importing the package itself needs pytorch3d and cv2).
Outputs go to tests/golden/datasets.npz.

Run: python tests/golden/make_golden_datasets.py [reference root]
"""
import importlib.util
import os
import sys
import types

import numpy as np
import torch
from scipy.io import savemat

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
from oracle.ref_harness import REF_ROOT  # noqa: E402

REF = sys.argv[1] if len(sys.argv) > 1 else REF_ROOT


def _load(name, rel):
    spec = importlib.util.spec_from_file_location(name, os.path.join(REF, rel))
    mod = importlib.util.module_from_spec(spec)
    sys.modules[name] = mod
    spec.loader.exec_module(mod)
    return mod


def write_inputs():
    g = np.random.default_rng(17)
    L, S, N = 3, 5, 16
    velten = {
        "deltat": np.array([[0.7]]), "t0": np.array([[12.5]]), "t": np.array([[N]], np.int32),
        "data": g.random((L, S * N)),
        "cameraPos": g.uniform(-50, 50, (S, 3)) + np.array([375.0, 220.0, 0.0]),
        "laserPos": g.uniform(-50, 50, (L, 3)) + np.array([375.0, 220.0, 0.0]),
        "cameraOrigin": np.array([[300.0, 150.0, 20.0]]),
        "laserOrigin": np.array([[320.0, 140.0, -10.0]]),
    }
    savemat(os.path.join(HERE, "velten_nc2012_small.mat"), {"dataset": velten})
    savemat(os.path.join(HERE, "otoole_confocal2018_small.mat"),
            {"rect_data": g.random((4, 3, 640)).astype(np.float32)})


def main():
    write_inputs()
    totri = types.ModuleType("totri")
    totri.__path__ = []
    sys.modules["totri"] = totri
    data_pkg = types.ModuleType("totri.data")
    data_pkg.__path__ = []
    sys.modules["totri.data"] = data_pkg
    _load("totri.types", "totri/types.py")
    util = _load("totri.data.util", "totri/data/util.py")
    grid = util.make_wall_grid  # its default device is CUDA; this container has none
    util.make_wall_grid = lambda *a, **k: grid(*a, **{**k, "device": torch.device("cpu")})
    velten = _load("totri.data.veltennc2012", "totri/data/veltennc2012.py")
    otoole = _load("totri.data.otooleconfocal2018", "totri/data/otooleconfocal2018.py")
    out = {}
    v = velten.VeltenNc2012(os.path.join(HERE, "velten_nc2012_small.mat"))
    out["velten_transient"] = v.transient.numpy().copy()  # rectify() writes in place
    out["velten_scan"] = v.scan_points.numpy()
    out["velten_laser"] = v.laser_points.numpy()
    out["velten_scan_origin"] = v.scan_origin.numpy()
    out["velten_laser_origin"] = v.laser_origin.numpy()
    out["velten_bins"] = np.array([v.bin_def.width, v.bin_def.offset, v.bin_def.num])
    v.rectify()
    out["velten_rectified"] = v.transient.numpy()
    o = otoole.OTooleConfocal2018(os.path.join(HERE, "otoole_confocal2018_small.mat"))
    out["otoole_transient"] = o.transient.numpy().copy()
    out["otoole_scan"] = o.scan_points.cpu().numpy()
    o.downsample_temporal(4)
    out["otoole_down4"] = o.transient.numpy()
    out["otoole_bins4"] = np.array([o.bin_def.width, o.bin_def.offset, o.bin_def.num])
    np.savez_compressed(os.path.join(HERE, "datasets.npz"), **out)
    print({k: a.shape for k, a in out.items()})


if __name__ == "__main__":
    main()
