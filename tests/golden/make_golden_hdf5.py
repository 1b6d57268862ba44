"""Golden vectors for the HDF5 dataset loaders, from the reference's own
loaders (totri/data/zaragoza.py, totri/data/lindellfk2019.py).

h5py is not installed here, and the loaders only index datasets by name
(file['x'][()], torch.tensor(file['x']), f.get('x')), so a stand-in h5py whose
File is a dict of numpy arrays read from an .npz serves them the inputs. The
reference's totri/types.py and totri/data/util.py stand in for the package
(importing the package itself needs pytorch3d and cv2). Inputs and outputs
go to tests/golden/zaragoza.npz and tests/golden/lindellfk2019.npz (inputs
under "in_<name>").

Run: python tests/golden/make_golden_hdf5.py [reference root]
"""
import os
import sys
import tempfile
import types

import numpy as np
import torch

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
sys.path.insert(0, HERE)
from oracle.ref_harness import REF_ROOT  # noqa: E402

REF = sys.argv[1] if len(sys.argv) > 1 else REF_ROOT


class _File(dict):
    """h5py.File stand-in: the arrays of one .npz, read-only."""

    def __init__(self, path, mode="r"):
        assert mode == "r"
        with np.load(path) as z:
            super().__init__({k: z[k] for k in z.files})

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        return False


def zaragoza_inputs(seed, N, H, W):
    """A confocal capture in the file's frame (y up, the wall at y = 0)."""
    g = np.random.default_rng(seed)
    x, z = np.meshgrid(np.linspace(-0.9, 0.9, W), np.linspace(-0.8, 0.8, H))
    pos = np.stack([x.ravel(), g.uniform(-0.01, 0.01, H * W), z.ravel()])
    nrm = np.tile([[0.0], [1.0], [0.0]], H * W) + g.normal(0, 0.01, (3, H * W))
    return {
        "isConfocal": np.array(1), "deltaT": np.array(0.0075), "t0": np.array(0.31),
        "t": np.array([[N]]), "hiddenVolumePosition": np.array([[0.05], [0.9], [-0.1]]),
        "hiddenVolumeSize": np.array(0.65), "cameraGridPoints": np.array([[W], [H]]),
        "cameraGridSize": np.array([[1.8], [1.6]]),
        "data": g.random((N, 6, H, W)).astype(np.float32),
        "cameraGridPositions": pos, "cameraGridNormals": nrm,
        "cameraPosition": np.array([[0.4], [-0.3], [1.7]]),
    }


def lindell_inputs(seed, T, W, H):
    g = np.random.default_rng(seed)
    return {"meas": g.random((T, W, H)).astype(np.float32),
            "tofgrid": g.uniform(-100, 700, (W, H)).astype(np.float32)}


def main():
    h5 = types.ModuleType("h5py")
    h5.File = _File
    sys.modules["h5py"] = h5
    from make_golden_datasets import _load
    import make_golden_datasets
    make_golden_datasets.REF = REF
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
    zaragoza = _load("totri.data.zaragoza", "totri/data/zaragoza.py")
    lindell = _load("totri.data.lindellfk2019", "totri/data/lindellfk2019.py")
    with tempfile.TemporaryDirectory() as tmp:
        out = {}
        for case, (seed, N, H, W) in enumerate(((21, 48, 5, 7), (22, 30, 4, 4))):
            m = zaragoza_inputs(seed, N, H, W)
            path = os.path.join(tmp, "z%d.npz" % case)
            np.savez(path, **m)
            out.update({"in%d_%s" % (case, k): v for k, v in m.items()})
            d = zaragoza.Zaragoza(path)
            p = "out%d_" % case
            out[p + "bins"] = np.array([d.bin_def.width, d.bin_def.offset, d.bin_def.num])
            out[p + "volume"] = np.array([d.volume_def.start, d.volume_def.end])
            out[p + "resolution"] = np.array(d.volume_def.resolution)
            out[p + "extent"] = np.array(d.scan_point_extent)
            out[p + "transient"] = d.transient.numpy().copy()  # rectify() writes in place
            out[p + "scan_points"] = d.scan_points.numpy()
            out[p + "scan_normals"] = d.scan_normals.numpy()
            out[p + "scan_origin"] = d.scan_origin.numpy()
            d.rectify()
            out[p + "rectified"] = d.transient.numpy()
        np.savez_compressed(os.path.join(HERE, "zaragoza.npz"), **out)
        print({k: a.shape for k, a in out.items() if k.startswith("out")})
        out = {}
        for case, (seed, T, W, H, crop) in enumerate(((31, 40, 5, 6, 32), (32, 24, 3, 3, 24))):
            m = lindell_inputs(seed, T, W, H)
            np.savez(os.path.join(tmp, "meas%d.npz" % case), meas=m["meas"])
            np.savez(os.path.join(tmp, "tof%d.npz" % case), tofgrid=m["tofgrid"])
            out.update({"in%d_%s" % (case, k): v for k, v in m.items()})
            out["in%d_crop" % case] = np.array(crop)
            d = lindell.LindellFk2019(os.path.join(tmp, "meas%d.npz" % case),
                                      os.path.join(tmp, "tof%d.npz" % case), crop=crop)
            p = "out%d_" % case
            out[p + "transient"] = d.transient.numpy()
            out[p + "scan_points_every64"] = d.scan_points[0, ::64, ::64].numpy()
            out[p + "bins"] = np.array([d.bin_def.width_s, d.bin_def.offset, d.bin_def.num])
        np.savez_compressed(os.path.join(HERE, "lindellfk2019.npz"), **out)
        print({k: a.shape for k, a in out.items() if k.startswith("out")})


if __name__ == "__main__":
    main()
