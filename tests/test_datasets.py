"""MATLAB-format dataset loaders against the reference's own loaders run on
the same small files (tests/golden/make_golden_datasets.py)."""
import os

import numpy as np

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
