"""A space's particles moved without a rebuild (sphgpu_space_drift,
swift_gb300/csrc/drift.cu).

Between rebuilds the reference keeps each particle in its cell, measures each
cell's largest motion since the rebuild (dx_max_part, cell_drift.c:330-382),
adds it to the recursions' cut-offs (cell.h:934-1010) and rebuilds once
cell_need_rebuild_for_hydro_pair (cell.h:1237) holds.  A drifted space must
give the physics of a space rebuilt from the moved positions (the same
neighbours, up to pairs within FP32 rounding of the kernel's edge, whose
frames differ between the two trees), its device plans must equal the host
planner's with the same dx_max, and a drift too large for the tree must be
refused without changing the space.
"""
import numpy as np
import pytest

from swift_gb300 import api, ics

pytestmark = pytest.mark.gpu


def scaled_err(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return np.abs(a - b) / (np.max(np.abs(b)) + 1e-30)


def rel_err(a, b, floor_frac=1e-3):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    scale = np.maximum(np.abs(b), floor_frac * np.max(np.abs(b)) + 1e-30)
    return np.abs(a - b) / scale


def _box(cfg, seed):
    box = ics.make(cfg, seed=seed)
    if not cfg.startswith("sedov"):
        n = box["x"].shape[0]
        box["time_bin"][:] = 20 + (np.arange(n) * 7919) % 4
    return box


def _moved(box, frac, seed):
    """Positions displaced by about frac mean spacings in random directions."""
    n = box["x"].shape[0]
    spacing = float(box.get("dim", 1.0)) / round(n ** (1.0 / 3.0))
    rng = np.random.default_rng(seed)
    return box["x"] + frac * spacing * rng.standard_normal((n, 3)) / np.sqrt(3.0)


def _steps(sp, seq):
    for b in seq:
        sp.set_active(b)
        sp.step()
    return sp.download()


def test_zero_drift_changes_nothing():
    """A drift to the rebuild's own positions and h: every later step equals
    the undrifted space's bit for bit (the steps plan on the device with
    dx_max = 0, the undrifted ones on the host)."""
    box = _box("sedov:24", 3)
    seq = (api.ALL_ACTIVE, 22, 20, 23)
    with api.Space(box) as sp:
        a = _steps(sp, seq)
    with api.Space(box) as sp:
        sp.drift(box["x"], box["h"])
        b = _steps(sp, seq)
    for k in a:
        assert np.array_equal(a[k], b[k], equal_nan=True), k


@pytest.mark.parametrize("cfg", ["clustered:24", "sedov:32"])
def test_drifted_space_matches_a_rebuilt_space(cfg):
    box = _box(cfg, 4)
    x2 = _moved(box, 0.05, 1)
    moved = dict(box, x=x2)
    with api.Space(box) as sp:
        sp.set_active(api.ALL_ACTIVE)
        sp.step()
        sp.drift(x2, box["h"])
        a = _steps(sp, (api.ALL_ACTIVE,))
        # the device's lists equal the host planner's with the same dx_max
        sp.set_active(22)
        sp.step()
        chk = sp.check_device_plans()
    assert all(bad == 0 for bad, _ in chk.values()), chk
    with api.Space(moved) as sp:
        b = _steps(sp, (api.ALL_ACTIVE,))
    # the same neighbours but for pairs at the kernel's edge in FP32
    assert np.mean(a["ngb_first"] == b["ngb_first"]) > 0.999
    assert rel_err(a["h"], b["h"]).max() < 2e-4
    for k in ("rho", "pressure", "soundspeed", "v_sig"):
        assert rel_err(a[k], b[k]).max() < 3e-4, k
    for k in ("ax", "ay", "az", "u_dt", "h_dt"):
        assert scaled_err(a[k], b[k]).max() < 1e-3, k


def test_large_drift_asks_for_a_rebuild_and_changes_nothing():
    box = _box("clustered:24", 5)
    n = box["x"].shape[0]
    far = box["x"] + 0.25 * float(box.get("dim", 1.0)) * (np.arange(n) % 2)[:, None]
    with api.Space(box) as sp:
        sp.set_active(api.ALL_ACTIVE)
        sp.step()
        with pytest.raises(api.SphGpuError) as e:
            sp.drift(far, box["h"])
        assert e.value.code == api.EREBUILD
        a = _steps(sp, (21, api.ALL_ACTIVE))
    with api.Space(box) as sp:
        b = _steps(sp, (api.ALL_ACTIVE, 21, api.ALL_ACTIVE))
    for k in a:
        assert np.array_equal(a[k], b[k], equal_nan=True), k


def test_step_host_takes_moved_positions():
    """sphgpu_step_host with moved x drifts the space first: the same as an
    explicit drift followed by the step."""
    box = _box("sedov:24", 6)
    x2 = _moved(box, 0.03, 2)
    moved = dict(box, x=x2)
    with api.Space(box) as sp:
        sp.step()
        out = np.zeros((box["x"].shape[0], 24), np.float32)
        sp.step_host(moved, out)
        a = sp.download()
    with api.Space(box) as sp:
        sp.step()
        sp.drift(x2, box["h"])
        sp.step()
        b = sp.download()
    for k in a:
        assert np.array_equal(a[k], b[k], equal_nan=True), k


def test_plain_form_on_a_drifted_space():
    """The host planner takes the drifted state (dx_max, h) for the plain
    form."""
    box = _box("clustered:24", 7)
    x2 = _moved(box, 0.05, 3)
    with api.Space(box) as sp:
        sp.step()
        sp.drift(x2, box["h"])
        sp.set_active(api.ALL_ACTIVE)
        sp.step()
        a = sp.download()
        sp.step_plain()
        b = sp.download()
    assert np.array_equal(a["ngb_first"], b["ngb_first"])
    assert rel_err(b["h"], a["h"]).max() < 2e-4
    for k in ("rho", "v_sig"):
        assert rel_err(b[k], a[k]).max() < 3e-4, k
    for k in ("ax", "ay", "az", "u_dt", "h_dt"):
        assert scaled_err(b[k], a[k]).max() < 1e-3, k
