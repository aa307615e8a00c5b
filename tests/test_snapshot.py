"""Snapshots (swift_gb300.snapshot): the reference's PartType0 fields in an
.npz container (HDF5 is not available here), read back as initial
conditions, and an integrator restart that continues bit for bit."""
import numpy as np
import pytest

from swift_gb300 import ics, snapshot


def test_write_read_roundtrip(tmp_path):
    box = ics.clustered(12, seed=4)
    n = box["x"].shape[0]
    rho = np.full(n, 1.5, np.float32)
    path = str(tmp_path / "snap_0000.npz")
    snapshot.write(path, dict(box, rho=rho), box_size=(1.0, 1.0, 1.0), time=0.25)
    back = snapshot.read(path)
    for k in ("x", "v", "m", "h", "u", "rho"):
        assert np.array_equal(back[k], np.asarray(box[k] if k != "rho" else rho)), k
    assert back["x"].dtype == np.float64
    assert np.array_equal(back["ids"], np.arange(1, n + 1))
    assert back["dim"] == (1.0, 1.0, 1.0) and back["time"] == 0.25
    assert back["restart"] == {}
    with np.load(path) as z:
        assert "PartType0/Entropies" in z.files
        assert z["Header/NumPart_ThisFile"][0] == n
        # ideal gas: A = (gamma - 1) u rho^(1 - gamma)
        a = z["PartType0/Entropies"].astype(np.float64)
        ref = (2.0 / 3.0) * box["u"].astype(np.float64) * 1.5 ** (-2.0 / 3.0)
        assert np.allclose(a, ref, rtol=1e-6)


def test_initial_conditions_field_names(tmp_path):
    """The reference's initial-condition names (SmoothingLength,
    InternalEnergy) are read as well."""
    box = ics.lattice(8, seed=2)
    path = str(tmp_path / "ics.npz")
    np.savez(path, **{"Header/BoxSize": np.array([1.0]),
                      "PartType0/Coordinates": box["x"], "PartType0/Velocities": box["v"],
                      "PartType0/Masses": box["m"], "PartType0/SmoothingLength": box["h"],
                      "PartType0/InternalEnergy": box["u"],
                      "PartType0/ParticleIDs": np.arange(box["x"].shape[0], dtype=np.uint64)})
    back = snapshot.read(path)
    assert back["dim"] == (1.0, 1.0, 1.0)
    assert np.array_equal(back["h"], box["h"]) and np.array_equal(back["u"], box["u"])


def test_missing_field_is_an_error(tmp_path):
    path = str(tmp_path / "bad.npz")
    np.savez(path, **{"Header/BoxSize": np.array([1.0]),
                      "PartType0/Coordinates": np.zeros((2, 3))})
    with pytest.raises(KeyError):
        snapshot.read(path)


@pytest.mark.gpu
def test_integrator_restart_is_bit_identical(tmp_path):
    from swift_gb300.integrate import Integrator
    box = ics.lattice(12, seed=6, sigma_v=0.3)
    box["u"][::5] *= 6.0
    a = Integrator(box, time_end=1.0, dt_max=0.05).init()
    for _ in range(2):
        a.step()
    path = str(tmp_path / "restart.npz")
    a.save(path)
    b = Integrator.restart(path)
    assert (b.ti_current, b.ti_end_min, b.steps) == (a.ti_current, a.ti_end_min, a.steps)
    for _ in range(3):
        assert a.step() == b.step()
    sa, sb = a.state(), b.state()
    for k in sa:
        assert np.array_equal(np.asarray(sa[k]).view(np.uint8), np.asarray(sb[k]).view(np.uint8)), k
    assert a.ti_current == b.ti_current
