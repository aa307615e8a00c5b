"""Seeded initial-condition generators (shapes, ranges, conservation)."""
import numpy as np

from swift_gb300 import ics


def test_lattice_shape_and_jitter():
    b = ics.lattice(10, seed=4)
    assert b["x"].shape == (1000, 3) and b["x"].dtype == np.float64
    assert (b["x"] >= 0).all() and (b["x"] < 1).all()
    g = (np.floor(b["x"] * 10) + 0.5) / 10
    assert np.abs(b["x"] - g).max() <= 0.6 / 10
    assert np.allclose(b["m"].sum(), 1.0, rtol=1e-6)
    assert np.allclose(b["h"], 1.2348 / 10)
    assert abs(b["v"].std() - 0.05) < 0.01
    assert np.array_equal(ics.lattice(10, seed=4)["x"], b["x"])


def test_clustered_rms_displacement():
    n = 24
    psi = ics.grf_displacement(n, 0.3, seed=1)
    assert abs(np.sqrt((psi ** 2).sum(axis=1).mean()) - 0.3) < 1e-9
    b = ics.clustered(n, seed=1)
    assert (b["x"] >= 0).all() and (b["x"] < 1).all()


def test_sedov_energy_and_bins():
    b = ics.sedov(20, seed=2)
    e = (b["u"] * b["m"]).astype(np.float64)
    hot = b["u"] > 1e-3
    assert hot.sum() == 33
    assert abs(e[hot].sum() - 1.0) < 1e-5
    tb = b["time_bin"]
    frac = [(tb <= 20 + k).mean() for k in range(7)]
    assert 0.005 < frac[0] < 0.02 and 0.05 < frac[6] < 0.2
    assert ics.max_active_bin_for_step(1) == 20
    assert ics.max_active_bin_for_step(4) == 22
