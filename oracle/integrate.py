"""The oracle's time integration: ctypes front end of oracle/sph_integrate.c
and the same engine sequence as swift_gb300/integrate.py, restated over the
oracle's loops (oracle.run, sph_oracle_run_state).  Test infrastructure
only: the tests use it as the checker of the GPU integrator.

Engine sequence (engine_init_particles, engine.c:2245-2420; engine_step),
with every particle drifted at every step (the reference's --drift-all) and
a rebuild at every step:
    init:  density + ghost (all active) -> density + ghost + force at
           ti = 0 -> kick2 -> timestep -> kick1
    step:  ti_old = ti_current; ti_current = ti_end_min;
           max_active_bin = get_max_active_bin(ti_current);
           drift all; box_wrap; density + ghost (active); force (active, the
           inactive particles' predicted state); kick2; timestep; kick1.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

from . import oracle

NUM_TIME_BINS = 56
MAX_NR_TIMESTEPS = 1 << (NUM_TIME_BINS + 1)
STATE_KEYS = ("x", "v_full", "v", "a", "u_full", "u", "u_dt", "h", "h_dt", "rho", "P", "c",
              "v_sig", "time_bin")


class IntegParams(ctypes.Structure):
    _fields_ = [("time_base", ctypes.c_double), ("dt_min", ctypes.c_double),
                ("dt_max", ctypes.c_double), ("CFL", ctypes.c_float),
                ("log_max_h_change", ctypes.c_float), ("h_min", ctypes.c_float),
                ("h_max", ctypes.c_float), ("minimal_u", ctypes.c_float)]


class IntegState(ctypes.Structure):
    _fields_ = [(k, ctypes.c_void_p) for k in STATE_KEYS]


def _lib():
    L = oracle.lib()
    if not getattr(L, "_integ_ready", False):
        P, S = ctypes.POINTER(IntegParams), ctypes.POINTER(IntegState)
        L.sph_integ_kick.argtypes = [P, S, ctypes.c_int64, ctypes.c_int, ctypes.c_int64,
                                     ctypes.c_int]
        L.sph_integ_kick.restype = None
        L.sph_integ_drift.argtypes = [P, S, ctypes.c_int64, ctypes.c_int64, ctypes.c_int64]
        L.sph_integ_drift.restype = None
        L.sph_integ_timestep.argtypes = [P, S, ctypes.c_int64, ctypes.c_void_p,
                                         ctypes.c_int64, ctypes.c_int]
        L.sph_integ_timestep.restype = ctypes.c_int64
        L.sph_integ_ti_end_min.argtypes = [S, ctypes.c_int64, ctypes.c_int64]
        L.sph_integ_ti_end_min.restype = ctypes.c_int64
        L.sph_integ_max_active_bin.argtypes = [ctypes.c_int64]
        L.sph_integ_max_active_bin.restype = ctypes.c_int
        L.sph_oracle_run_state.restype = ctypes.c_int
        L._integ_ready = True
    return L


def make_state(box):
    """Initial state of a box (hydro_first_init_part: v_full = v,
    u_full = u; time bins 0)."""
    n = box["x"].shape[0]
    v = np.ascontiguousarray(box["v"], np.float32)
    u = np.ascontiguousarray(box["u"], np.float32)
    z = lambda: np.zeros(n, np.float32)  # noqa: E731
    return {"x": np.ascontiguousarray(box["x"], np.float64).copy(), "v_full": v.copy(),
            "v": v.copy(), "a": np.zeros((n, 3), np.float32), "u_full": u.copy(),
            "u": u.copy(), "u_dt": z(), "h": np.ascontiguousarray(box["h"], np.float32).copy(),
            "h_dt": z(), "rho": z(), "P": z(), "c": z(), "v_sig": z(),
            "time_bin": np.zeros(n, np.int8),
            "min_ngb_bin": np.full(n, NUM_TIME_BINS + 1, np.int8),
            "f": z(), "balsara": z()}


def _struct(st):
    s = IntegState()
    for k in STATE_KEYS:
        setattr(s, k, ctypes.c_void_p(st[k].ctypes.data))
    return s


def kick(ip, st, which, ti_current, max_active_bin):
    _lib().sph_integ_kick(ctypes.byref(ip), ctypes.byref(_struct(st)), len(st["h"]), which,
                          ti_current, max_active_bin)


def drift(ip, st, ti_old, ti_current):
    _lib().sph_integ_drift(ctypes.byref(ip), ctypes.byref(_struct(st)), len(st["h"]),
                           ti_old, ti_current)


def timestep(ip, st, ti_current, max_active_bin):
    """New bins of the active particles; returns the count below dt_min."""
    nb = np.ascontiguousarray(st["min_ngb_bin"], np.int8)
    return _lib().sph_integ_timestep(ctypes.byref(ip), ctypes.byref(_struct(st)),
                                     len(st["h"]), nb.ctypes.data, ti_current, max_active_bin)


def ti_end_min(st, ti_current):
    return _lib().sph_integ_ti_end_min(ctypes.byref(_struct(st)), len(st["h"]), ti_current)


def max_active_bin(ti):
    return _lib().sph_integ_max_active_bin(ti)


def box_wrap(x, dim):
    """The rebuild's periodic wrap (space_cell_index.c:113-123)."""
    D = np.asarray(dim, np.float64)[None, :]
    y = np.where(x < 0.0, x + D, np.where(x >= D, x - D, x))
    return np.where(y == D, 0.0, y)


def run_state_force(box, state6, **kw):
    """sph_oracle_run_state: the force loops on a given state."""
    L = _lib()
    n = box["x"].shape[0]
    arrs = {k: np.ascontiguousarray(box[k], t) for k, t in
            (("x", np.float64), ("v", np.float32), ("m", np.float32), ("u", np.float32),
             ("time_bin", np.int8))}
    st6 = np.ascontiguousarray(state6, np.float32)
    fields = np.zeros((n, oracle.NFIELDS), np.float32)
    ints = np.zeros((n, oracle.NINTS), np.int32)
    res = oracle.Result()
    res.fields = oracle._ptr(fields, ctypes.c_float)
    res.ints = oracle._ptr(ints, ctypes.c_int32)
    prm = oracle.make_params(box, **kw)
    L.sph_oracle_run_state(ctypes.byref(prm), ctypes.c_int(n),
                           oracle._ptr(arrs["x"], ctypes.c_double),
                           oracle._ptr(arrs["v"], ctypes.c_float),
                           oracle._ptr(arrs["m"], ctypes.c_float),
                           oracle._ptr(arrs["u"], ctypes.c_float),
                           oracle._ptr(arrs["time_bin"], ctypes.c_byte),
                           oracle._ptr(st6, ctypes.c_float), ctypes.byref(res))
    out = {"a": fields[:, 15:18].copy(), "u_dt": fields[:, 18].copy(),
           "h_dt": fields[:, 19].copy(), "v_sig": fields[:, 20].copy(),
           "ngb_force": ints[:, 8].copy(), "min_ngb_bin": ints[:, 10].astype(np.int8)}
    return out


class OracleIntegrator:
    """The engine sequence of swift_gb300.integrate.Integrator over the
    oracle's loops (numpy state, the caller's order)."""

    def __init__(self, box, *, time_end=1.0, cfl=0.1, dt_min=1e-12, dt_max=1e-2,
                 log_max_h_change, minimal_u=0.0, **kw):
        self.box = box
        self.kw = kw
        self.m = np.ascontiguousarray(box["m"], np.float32)
        d = box["dim"]
        self.dim = tuple(float(v) for v in (d if np.ndim(d) else (d, d, d)))
        prm = oracle.make_params(box, **kw)
        self.ip = IntegParams(float(time_end) / MAX_NR_TIMESTEPS, dt_min, dt_max, cfl,
                              log_max_h_change, prm.h_min, prm.h_max, minimal_u)
        self.periodic = prm.periodic
        self.st = make_state(box)
        self.ti_current = 0
        self.ti_end = 0

    def _box(self):
        st = self.st
        return dict(x=st["x"], v=st["v"], m=self.m, h=st["h"], u=st["u"],
                    time_bin=st["time_bin"], dim=self.dim,
                    **{k: self.box[k] for k in ("eta",) if k in self.box})

    def _hydro(self, mab, force=True):
        st = self.st
        act = st["time_bin"] <= mab
        r = oracle.run(self._box(), stages=oracle.STAGE_DENSITY | oracle.STAGE_GHOST,
                       max_active_bin=mab, **self.kw)
        assert r["status"] == 0, "ghost did not converge"
        for k, col in (("h", "h"), ("rho", "rho"), ("P", "pressure"), ("c", "soundspeed"),
                       ("f", "f"), ("balsara", "balsara")):
            st[k] = np.where(act, r[col], st[k]).astype(np.float32)
        if not force:
            return
        state6 = np.stack([st["h"], st["rho"], st["f"], st["P"], st["c"], st["balsara"]], 1)
        o = run_state_force(self._box(), state6, max_active_bin=mab, **self.kw)
        st["a"] = np.where(act[:, None], o["a"], st["a"]).astype(np.float32)
        for k in ("u_dt", "h_dt", "v_sig"):
            st[k] = np.where(act, o[k], st[k]).astype(np.float32)
        st["min_ngb_bin"] = np.where(act, o["min_ngb_bin"], st["min_ngb_bin"]).astype(np.int8)

    def init(self):
        mab = NUM_TIME_BINS
        self._hydro(mab, force=False)
        self._hydro(mab)
        kick(self.ip, self.st, 2, 0, mab)
        assert timestep(self.ip, self.st, 0, mab) == 0
        kick(self.ip, self.st, 1, 0, mab)
        self.ti_end = ti_end_min(self.st, 0)
        return self

    def step(self):
        ti_old = self.ti_current
        self.ti_current = self.ti_end
        mab = max_active_bin(self.ti_current)
        drift(self.ip, self.st, ti_old, self.ti_current)
        if self.periodic:
            self.st["x"] = np.ascontiguousarray(box_wrap(self.st["x"], self.dim))
        self._hydro(mab)
        kick(self.ip, self.st, 2, self.ti_current, mab)
        assert timestep(self.ip, self.st, self.ti_current, mab) == 0
        kick(self.ip, self.st, 1, self.ti_current, mab)
        self.ti_end = ti_end_min(self.st, self.ti_current)
        return mab


# ---- the reference's own functions (oracle/_ref/<mode>/bin/ref_integrate) --

OPS = {"kick1": 1, "kick2": 2, "drift": 3, "timestep": 4}


def ref_integrate_path(mode="parity"):
    return os.path.join(os.path.dirname(os.path.abspath(__file__)), "_ref", mode, "bin",
                        "ref_integrate")


def run_reference_op(ip, st, op, ti_old, ti_current, max_active_bin, workdir, mode="parity"):
    """Apply one operation with the reference's functions; returns the new
    state (a copy)."""
    exe = ref_integrate_path(mode)
    n = len(st["h"])
    hdr = np.zeros(1, dtype=[("magic", "S8"), ("n", "<i8"), ("op", "<i8"), ("ti_old", "<i8"),
                             ("ti_current", "<i8"), ("mab", "<i4"), ("pad", "<i4"),
                             ("time_base", "<f8"), ("dt_min", "<f8"), ("dt_max", "<f8"),
                             ("CFL", "<f4"), ("lmhc", "<f4"), ("h_min", "<f4"),
                             ("h_max", "<f4"), ("minimal_u", "<f4"), ("pad2", "<f4")])
    hdr["magic"] = b"SPHINT01"
    hdr["n"], hdr["op"], hdr["ti_old"], hdr["ti_current"] = n, OPS[op], ti_old, ti_current
    hdr["mab"] = max_active_bin
    hdr["time_base"], hdr["dt_min"], hdr["dt_max"] = ip.time_base, ip.dt_min, ip.dt_max
    hdr["CFL"], hdr["lmhc"] = ip.CFL, ip.log_max_h_change
    hdr["h_min"], hdr["h_max"], hdr["minimal_u"] = ip.h_min, ip.h_max, ip.minimal_u
    order = [("x", np.float64), ("v_full", np.float32), ("v", np.float32), ("a", np.float32),
             ("u_full", np.float32), ("u", np.float32), ("u_dt", np.float32),
             ("h", np.float32), ("h_dt", np.float32), ("rho", np.float32), ("P", np.float32),
             ("c", np.float32), ("v_sig", np.float32), ("time_bin", np.int8),
             ("min_ngb_bin", np.int8)]
    inp = os.path.join(workdir, "integ_in.bin")
    out = os.path.join(workdir, "integ_out.bin")
    with open(inp, "wb") as f:
        f.write(hdr.tobytes())
        for k, t in order:
            f.write(np.ascontiguousarray(st[k], t).tobytes())
    subprocess.run([exe, inp, out], check=True, capture_output=True)
    buf = open(out, "rb").read()
    assert buf[:8] == b"SPHINT02"
    off, res = 8, {}
    for k, t in order:
        shape = st[k].shape
        cnt = int(np.prod(shape))
        res[k] = np.frombuffer(buf, t, cnt, off).reshape(shape).copy()
        off += cnt * np.dtype(t).itemsize
    return res
