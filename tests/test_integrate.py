"""Time integration: the oracle's restatement of the kicks, the drift and the
time steps against the reference's own functions (oracle/_ref, where it is
built), the engine sequence on the oracle, and the GPU integrator
(sphgpu_integ_* kernels, swift_gb300.integrate) against the oracle."""
import os
import tempfile

import numpy as np
import pytest

from swift_gb300 import ics

from oracle import integrate as oi  # noqa: E402

HAVE_REF = os.path.exists(oi.ref_integrate_path("parity"))
LMHC = float(np.log(np.power(np.float32(1.4), np.float32(1.0) / np.float32(3.0),
                             dtype=np.float32), dtype=np.float32))


def random_state(n, seed, bins=(18, 26)):
    """A post-force state with the spread of a real one: positions in the
    unit box, O(1) velocities and accelerations, h ~ 0.03, a few large h_dt
    (the expf branch of the drift), u_dt that would drive u negative on some
    particles (the kick's floor), mixed time bins."""
    rng = np.random.default_rng(seed)
    f = lambda *s: rng.standard_normal(s).astype(np.float32)  # noqa: E731
    h = (0.03 * (1 + 0.3 * rng.random(n))).astype(np.float32)
    st = {"x": rng.random((n, 3)), "v_full": f(n, 3), "v": f(n, 3), "a": 10 * f(n, 3),
          "u_full": (1 + rng.random(n)).astype(np.float32),
          "u": (1 + rng.random(n)).astype(np.float32), "u_dt": 50 * f(n),
          "h": h, "h_dt": (h * f(n) * 5).astype(np.float32),
          "rho": (1 + rng.random(n)).astype(np.float32),
          "P": np.ones(n, np.float32), "c": np.ones(n, np.float32),
          "v_sig": (2 + 3 * rng.random(n)).astype(np.float32),
          "time_bin": rng.integers(bins[0], bins[1], n).astype(np.int8),
          "min_ngb_bin": rng.integers(bins[0] - 1, bins[1] + 3, n).astype(np.int8)}
    st["h_dt"][::37] *= 40.0   # |w| >= 0.2 in the drift for some
    st["u_dt"][::11] *= -400.0  # u_full would fall below half: the floor
    return st


def params(time_end=float(1 << 37) * 1e-3):
    """A time line on which the 2^20-tick intervals of the tests are 1e-3
    (drifts that move h by up to ~25 %, time steps near bins 20-23)."""
    return oi.IntegParams(time_end / oi.MAX_NR_TIMESTEPS, 1e-14, 1e-2, 0.1, LMHC, 0.0,
                          3.4e38, 0.0)


def copy_state(st):
    return {k: np.array(v, copy=True) for k, v in st.items()}


# ti_current values at which bins 18..25 are active (multiples of 2^19)
TI = 3 << 22


@pytest.mark.skipif(not HAVE_REF, reason="reference build (oracle/_ref) absent")
@pytest.mark.parametrize("op", ["kick1", "kick2", "drift", "timestep"])
def test_oracle_integration_matches_reference(op):
    """Every operation, bit for bit against the reference's kick_part,
    drift_part / hydro_predict_extra, hydro_reset_predicted_values and
    get_part_timestep."""
    st = random_state(4000, seed=5)
    ip = params()
    mab = oi.max_active_bin(TI)
    ti_old = TI - (1 << 20)
    with tempfile.TemporaryDirectory() as wd:
        ref = oi.run_reference_op(ip, st, op, ti_old, TI, mab, wd)
    mine = copy_state(st)
    if op in ("kick1", "kick2"):
        oi.kick(ip, mine, 1 if op == "kick1" else 2, TI, mab)
    elif op == "drift":
        oi.drift(ip, mine, ti_old, TI)
    else:
        assert oi.timestep(ip, mine, TI, mab) == 0
    for k in oi.STATE_KEYS:
        assert np.array_equal(np.asarray(mine[k]).view(np.uint8),
                              np.asarray(ref[k]).view(np.uint8)), (op, k)
    if op == "timestep":  # bins did change
        assert np.mean(mine["time_bin"] != st["time_bin"]) > 0.3


def test_integer_time_line():
    assert oi.max_active_bin(0) == 56
    assert oi.max_active_bin(1 << 20) == 19
    assert oi.max_active_bin(3 << 22) == 21
    L = oi._lib()
    assert L.sph_integ_time_end(5, 1) == 8 and L.sph_integ_time_end(8, 1) == 8
    assert L.sph_integ_time_end(9, 2) == 16


def test_box_wrap():
    x = np.array([[-0.25, 1.0, 0.5], [1.5, -1e-300, 0.999]])
    y = oi.box_wrap(x, (1.0, 1.0, 1.0))
    assert np.array_equal(y, [[0.75, 0.0, 0.5], [0.5, 0.0, 0.999]])


def test_oracle_engine_sequence_runs():
    """A few steps of the oracle's integrator on a box with uneven sound
    speeds: time advances, bins differ, activity varies, energy stays
    finite."""
    box = ics.lattice(10, seed=3, sigma_v=0.3)
    box["u"][::7] *= 8.0
    it = oi.OracleIntegrator(box, time_end=1.0, log_max_h_change=LMHC, dt_max=0.05).init()
    nact = []
    for _ in range(6):
        mab = it.step()
        nact.append(int(np.sum(it.st["time_bin"] <= mab)))
    assert it.ti_current > 0
    assert len(set(it.st["time_bin"].tolist())) >= 2
    assert min(nact) < box["x"].shape[0]
    for k in ("x", "v_full", "u_full", "h", "rho"):
        assert np.isfinite(it.st[k]).all(), k


@pytest.mark.skipif(not HAVE_REF, reason="reference build (oracle/_ref) absent")
def test_oracle_min_ngb_bin_matches_reference():
    """The force loop's smallest neighbour time bin (runner_iact_timebin),
    oracle against the reference's loops."""
    from oracle import io, oracle
    box = ics.lattice(12, seed=8)
    rng = np.random.default_rng(8)
    box["time_bin"] = rng.integers(20, 26, box["x"].shape[0]).astype(np.int8)
    kw = {"max_active_bin": 23}
    with tempfile.TemporaryDirectory() as wd:
        ref = io.run_reference(box, wd, **kw)
    mine = oracle.run(box, **kw)
    act = box["time_bin"] <= 23
    assert np.array_equal(mine["min_ngb_bin"][act], ref["min_ngb_bin"][act])
    assert mine["min_ngb_bin"][act].min() >= 20


# --- GPU ---------------------------------------------------------------------

def gpu_state(st):
    import torch
    return {k: torch.as_tensor(np.ascontiguousarray(v), device="cuda") for k, v in st.items()}


@pytest.mark.gpu
@pytest.mark.parametrize("op", ["kick1", "kick2", "drift", "timestep"])
def test_gpu_integration_kernels_match_oracle(op):
    """The sphgpu_integ_* kernels against the oracle: bit for bit, except
    the drift's expf branch (|w| >= 0.2) where h and rho may differ by the
    device expf's last bits."""
    import ctypes

    import torch

    from swift_gb300 import api
    st = random_state(50000, seed=11)
    ip = params()
    mab = oi.max_active_bin(TI)
    ti_old = TI - (1 << 20)
    mine = copy_state(st)
    if op in ("kick1", "kick2"):
        oi.kick(ip, mine, 1 if op == "kick1" else 2, TI, mab)
    elif op == "drift":
        oi.drift(ip, mine, ti_old, TI)
    else:
        oi.timestep(ip, mine, TI, mab)
    g = gpu_state(st)
    gp = api.IntegParams()
    for k in ("time_base", "dt_min", "dt_max", "CFL", "log_max_h_change", "h_min", "h_max",
              "minimal_u"):
        setattr(gp, k, getattr(ip, k))
    gp.dim[:] = [1.0, 1.0, 1.0]
    gp.periodic = 0
    s = api.IntegState()
    for k in api.INTEG_FIELDS:
        setattr(s, k, ctypes.c_void_p(g[k].data_ptr()))
    L = api.lib()
    if op in ("kick1", "kick2"):
        api._check(L.sphgpu_integ_kick(ctypes.byref(gp), ctypes.byref(s), len(st["h"]),
                                       1 if op == "kick1" else 2, TI, mab, None))
    elif op == "drift":
        api._check(L.sphgpu_integ_drift(ctypes.byref(gp), ctypes.byref(s), len(st["h"]),
                                        ti_old, TI, 0, None))
    else:
        tmin, bad = ctypes.c_int64(), ctypes.c_int64()
        api._check(L.sphgpu_integ_timestep(ctypes.byref(gp), ctypes.byref(s), len(st["h"]),
                                           TI, mab, ctypes.byref(tmin), ctypes.byref(bad),
                                           None))
        assert bad.value == 0
        assert tmin.value == oi.ti_end_min(mine, TI)
    torch.cuda.synchronize()
    out = {k: v.cpu().numpy() for k, v in g.items()}
    big = np.zeros(len(st["h"]), bool)
    if op == "drift":
        w1 = st["h_dt"] * (np.float32(1) / st["h"]) * np.float32(ip.time_base * (1 << 20))
        big = np.abs(w1) >= 0.06  # expf for h (|w1| >= 0.2) or rho (|3 w1| >= 0.2)
        assert big.sum() > 10
    for k in oi.STATE_KEYS:
        a, b = out[k], mine[k]
        if k in ("h", "rho", "P", "c", "v_sig") and op == "drift":
            assert np.array_equal(a[~big].view(np.uint8), b[~big].view(np.uint8)), k
            assert np.allclose(a[big], b[big], rtol=1e-6, atol=0), k
        else:
            assert np.array_equal(a.view(np.uint8), b.view(np.uint8)), (op, k)


@pytest.mark.gpu
def test_gpu_integrator_matches_oracle_integrator():
    """Six steps of the engine sequence, GPU against the oracle: the same
    time line (synchronisation points, active sets, time bins) and states
    within the step-to-step FP32 tolerance."""
    from swift_gb300.integrate import Integrator
    box = ics.lattice(12, seed=4, sigma_v=0.3)
    box["u"][::5] *= 6.0
    kw = dict(time_end=1.0, dt_max=0.05)
    ref = oi.OracleIntegrator(box, log_max_h_change=LMHC, **kw).init()
    gpu = Integrator(box, **kw).init()
    assert gpu.ti_end_min == ref.ti_end
    active = []
    for step in range(6):
        mab_r = ref.step()
        mab_g = gpu.step()
        active.append(gpu.last_active)
        assert mab_g == mab_r and gpu.ti_current == ref.ti_current, step
        g = gpu.state()
        assert np.mean(g["time_bin"] == ref.st["time_bin"]) > 0.999, step
        # the oracle wraps every step (it rebuilds every step), the GPU
        # integrator at its rebuilds only
        assert np.abs(oi.box_wrap(g["x"], gpu.dim) - ref.st["x"]).max() < 1e-6, step
        for k in ("v_full", "h", "rho", "u_full"):
            scale = np.abs(ref.st[k]).max()
            assert np.abs(g[k] - ref.st[k]).max() < 2e-4 * scale, (step, k)
    assert min(active) < box["x"].shape[0], active  # some steps were partial
    # the space was drifted between rebuilds (init builds the first one)
    assert 1 <= gpu.rebuilds < 1 + 6, gpu.rebuilds
