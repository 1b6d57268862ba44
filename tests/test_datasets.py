"""Dataset loaders against the reference's own loaders run on the same small
inputs: the MATLAB formats (tests/golden/make_golden_datasets.py) and the
HDF5 formats (tests/golden/make_golden_hdf5.py); plus the Zaragoza and Lindell
layouts checked directly on synthetic arrays."""
import os

import numpy as np
import torch

from totri_gb300.data import OTooleConfocal2018, VeltenNc2012

HERE = os.path.join(os.path.dirname(__file__), "golden")


def test_velten_nc2012_matches_reference():
    g = np.load(os.path.join(HERE, "datasets.npz"))
    d = VeltenNc2012(os.path.join(HERE, "velten_nc2012_small.mat"))
    assert np.array_equal(d.transient.numpy(), g["velten_transient"])
    assert np.allclose(d.scan_points.numpy(), g["velten_scan"], atol=1e-6)
    assert np.allclose(d.laser_points.numpy(), g["velten_laser"], atol=1e-6)
    assert np.allclose(d.scan_origin.numpy(), g["velten_scan_origin"], atol=1e-6)
    assert np.allclose(d.laser_origin.numpy(), g["velten_laser_origin"], atol=1e-6)
    assert np.allclose([d.bin_def.width, d.bin_def.offset, d.bin_def.num], g["velten_bins"])
    d.rectify()
    assert d.scan_origin is None and d.laser_origin is None
    assert np.array_equal(d.transient.numpy(), g["velten_rectified"])


def test_otoole_confocal2018_matches_reference():
    g = np.load(os.path.join(HERE, "datasets.npz"))
    d = OTooleConfocal2018(os.path.join(HERE, "otoole_confocal2018_small.mat"))
    assert np.array_equal(d.transient.numpy(), g["otoole_transient"])
    assert np.allclose(d.scan_points.numpy(), g["otoole_scan"], atol=1e-7)
    d.downsample_temporal(4)
    assert np.allclose(d.transient.numpy(), g["otoole_down4"], rtol=1e-6, atol=1e-6)
    assert np.allclose([d.bin_def.width, d.bin_def.offset, d.bin_def.num], g["otoole_bins4"])


def _zaragoza_mapping(N=64, H=4, W=5, seed=0):
    g = np.random.default_rng(seed)
    x, y = np.meshgrid(np.linspace(-1, 1, W), np.linspace(-1, 1, H))
    pos = np.stack([x.ravel(), np.zeros(H * W), y.ravel()])  # file frame: the wall at y = 0
    return {
        "isConfocal": np.array(1), "deltaT": np.array(0.01), "t0": np.array(0.2),
        "t": np.array([[N]]), "hiddenVolumePosition": np.array([[0.1], [-1.0], [0.2]]),
        "hiddenVolumeSize": np.array(0.8), "cameraGridPoints": np.array([[W], [H]]),
        "cameraGridSize": np.array([[2.0], [2.0]]),
        "data": g.random((N, 6, H, W)).astype(np.float32),
        "cameraGridPositions": pos, "cameraGridNormals": np.tile([[0.0], [1.0], [0.0]], H * W),
        "cameraPosition": np.array([[0.3], [-0.4], [0.5]]),
    }


def test_zaragoza_mapping_layout_and_rectify():
    """Zaragoza (reference totri/data/zaragoza.py:57-128) from a mapping of
    its datasets: bins, volume box, summed transient, wall-frame grids, and
    rectification by the per-column origin round trip (zaragoza.py:38-50)."""
    from totri_gb300.data import Zaragoza
    m = _zaragoza_mapping()
    ds = Zaragoza(m)
    assert (ds.bin_def.width, ds.bin_def.offset, ds.bin_def.num) == (0.01, 0.2, 64)
    # position (0.1, -1.0, 0.2) in the file frame is (0.1, 0.2, 1.0) on the wall
    assert np.allclose(ds.volume_def.start, (-0.3, -0.2, 0.6))
    assert np.allclose(ds.volume_def.end, (0.5, 0.6, 1.4))
    assert tuple(ds.volume_def.resolution) == (64, 4, 5)
    assert torch.allclose(ds.transient[0], torch.tensor(m["data"].sum(axis=1)))
    assert ds.scan_points.shape == (1, 4, 5, 3)
    assert torch.allclose(ds.scan_points[0, 1, 2], torch.tensor([0.0, -1 / 3, 0.0]), atol=1e-6)
    assert torch.allclose(ds.scan_normals[0, 0, 0], torch.tensor([0.0, 0.0, -1.0]))
    assert torch.allclose(ds.scan_origin, torch.tensor([[0.3, 0.5, 0.4]]))
    r = Zaragoza(m, rectify=True)
    assert r.scan_origin is None
    for yy, xx in ((0, 0), (3, 4), (2, 1)):
        d = float(((ds.scan_points[0, yy, xx] - ds.scan_origin[0]) ** 2).sum() ** 0.5)
        k = int(2 * d / 0.01)
        assert torch.equal(r.transient[0, :, yy, xx], torch.roll(ds.transient[0, :, yy, xx], -k))


def test_lindell_fk2019_arrays():
    """LindellFk2019 (reference totri/data/lindellfk2019.py:33-57) from its two
    arrays: per-column roll by floor(tof / 32 ps), crop, [1, T, H, W] with
    rows and columns flipped, the fixed 512 x 512 wall grid."""
    from totri_gb300.data import LindellFk2019
    g = np.random.default_rng(3)
    T, W, H = 20, 3, 4
    meas = g.random((T, W, H)).astype(np.float32)
    tof = g.uniform(-40, 120, (W, H)).astype(np.float32)
    ds = LindellFk2019(meas, tof, crop=16)
    want = np.empty_like(meas)
    for x in range(W):
        for y in range(H):
            want[:, x, y] = np.roll(meas[:, x, y], -int(np.floor(tof[x, y] / 32.0)))
    want = want[:16].transpose(0, 2, 1)[:, ::-1, ::-1][None]
    assert ds.transient.shape == (1, 16, H, W)
    assert np.array_equal(ds.transient.numpy(), want)
    assert ds.scan_points.shape == (1, 512, 512, 3)
    assert abs(ds.bin_def.width_s - 32e-12) < 1e-20


def _golden_cases(name):
    z = dict(np.load(os.path.join(HERE, name)))
    cases = sorted({k.split("_", 1)[0][2:] for k in z if k.startswith("in")})
    for c in cases:
        inputs = {k.split("_", 1)[1]: v for k, v in z.items() if k.startswith("in%s_" % c)}
        outputs = {k.split("_", 1)[1]: v for k, v in z.items() if k.startswith("out%s_" % c)}
        yield inputs, outputs


def test_zaragoza_matches_reference_loader():
    """Zaragoza against the reference's own loader (totri/data/zaragoza.py:57-128)
    run on the same datasets (tests/golden/make_golden_hdf5.py): bins, volume
    box, grid extent, summed transient, wall-frame points, normals and origin,
    and the rectified transient (its rolls wrap: 2 d / bin width > T)."""
    from totri_gb300.data import Zaragoza
    n = 0
    for m, ref in _golden_cases("zaragoza.npz"):
        ds = Zaragoza(m)
        assert np.allclose([ds.bin_def.width, ds.bin_def.offset, ds.bin_def.num], ref["bins"])
        assert np.allclose([ds.volume_def.start, ds.volume_def.end], ref["volume"])
        assert tuple(ds.volume_def.resolution) == tuple(ref["resolution"])
        assert np.allclose(ds.scan_point_extent, ref["extent"])
        assert np.array_equal(ds.transient.numpy(), ref["transient"])
        assert np.array_equal(ds.scan_points.numpy(), ref["scan_points"])
        assert np.array_equal(ds.scan_normals.numpy(), ref["scan_normals"])
        assert np.array_equal(ds.scan_origin.numpy(), ref["scan_origin"])
        assert np.array_equal(Zaragoza(m, rectify=True).transient.numpy(), ref["rectified"])
        assert not np.array_equal(ref["rectified"], ref["transient"])
        n += 1
    assert n == 2


def test_lindell_fk2019_matches_reference_loader():
    """LindellFk2019 against the reference's own loader
    (totri/data/lindellfk2019.py:33-57) on the same arrays: rolled, cropped,
    flipped transient, the wall grid (every 64th point) and the bins."""
    from totri_gb300.data import LindellFk2019
    n = 0
    for m, ref in _golden_cases("lindellfk2019.npz"):
        ds = LindellFk2019(m["meas"], m["tofgrid"], crop=int(m["crop"]))
        assert np.array_equal(ds.transient.numpy(), ref["transient"])
        assert np.array_equal(ds.scan_points[0, ::64, ::64].numpy(), ref["scan_points_every64"])
        assert np.allclose([ds.bin_def.width_s, ds.bin_def.offset, ds.bin_def.num], ref["bins"])
        n += 1
    assert n == 2
