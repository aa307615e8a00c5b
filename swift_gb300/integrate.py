"""Time integration of a box of gas particles on the GPU: the reference's
engine sequence (engine_init_particles, engine.c:2245; engine_step) with the
drift-everything policy (the reference's --drift-all, engine_policy_drift_all)
and a cell rebuild whenever the drifted particles need one.

Per step, as the reference's task graph runs it:
    ti_old = ti_current; ti_current = ti_end_min
    max_active_bin = get_max_active_bin(ti_current)        (timeline.h:146)
    drift every particle to ti_current (drift_part + hydro_predict_extra,
        cell_drift.c:253-332)
    the space takes the drifted positions and h without a rebuild while
        cell_need_rebuild_for_hydro_pair (cell.h:1237) holds for no pair of
        neighbouring top-level cells (sphgpu_space_drift); otherwise the
        positions get the rebuild's periodic wrap (space_cell_index.c:
        113-123) and a new space is built from them: its cell assignment on
        the device (sphgpu_cell_assign), adopted by the host planner
    density -> ghost for the active particles (time_bin <= max_active_bin)
    force for the active particles; inactive ones lend their predicted state
    kick2, timestep, kick1 for the active particles
        (runner_time_integration.c:360, :639, :87)

The particle state stays in device memory (torch tensors, the caller's
order): the kicks, the drift and the time steps are CUDA kernels of the
library (sphgpu_integ_*), and between rebuilds the space takes the drifted
state, runs the loops and hands its results back in device memory (the
gather lists of sparse steps planned on the device).  Only a rebuild copies
the particle state to the host, for the planner of the new space.
"""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import api, snapshot

NUM_TIME_BINS = 56
MAX_NR_TIMESTEPS = 1 << (NUM_TIME_BINS + 1)


def default_log_max_h_change():
    """hydro_props_init's log of the largest h change per step from the
    default volume change of 1.4 (hydro_properties.c): log(1.4^(1/3))."""
    return float(np.log(np.power(np.float32(1.4), np.float32(1.0) / np.float32(3.0),
                                 dtype=np.float32), dtype=np.float32))


class Integrator:
    """Integrates ``box`` (positions, velocities, masses, h, u) forward in
    time on ``cuda:0``.  ``time_end`` fixes the integer time line
    (time_base = time_end / 2^57); dt_min / dt_max / cfl are the engine's
    and hydro scheme's parameters.  Space parameters (eta, h_tolerance,
    max_iter, periodic ...) pass through to every rebuild."""

    def __init__(self, box, *, time_end=1.0, cfl=0.1, dt_min=1e-12, dt_max=1e-2,
                 log_max_h_change=None, minimal_u=0.0, device="cuda", device_rebuild=True,
                 **space_params):
        self.device_rebuild = bool(device_rebuild)
        self._settings = dict(time_end=float(time_end), cfl=float(cfl), dt_min=float(dt_min),
                              dt_max=float(dt_max), minimal_u=float(minimal_u))
        if not torch.cuda.is_available():
            raise RuntimeError("Integrator needs a CUDA device")
        self.dev = torch.device(device)
        self.n = int(box["x"].shape[0])
        d = box["dim"]
        self.dim = tuple(float(v) for v in (d if np.ndim(d) else (d, d, d)))
        self.space_params = dict(space_params)
        self.box_meta = {k: box[k] for k in ("eta",) if k in box}
        prm = api.make_params(box, **space_params)
        self.ip = api.IntegParams()
        self.ip.time_base = float(time_end) / MAX_NR_TIMESTEPS
        self.ip.dt_min = float(dt_min)
        self.ip.dt_max = float(dt_max)
        self.ip.CFL = float(cfl)
        self.ip.log_max_h_change = (default_log_max_h_change() if log_max_h_change is None
                                    else float(log_max_h_change))
        self.ip.h_min = prm.h_min
        self.ip.h_max = prm.h_max
        self.ip.minimal_u = float(minimal_u)
        self.ip.dim[:] = list(self.dim)
        self.ip.periodic = prm.periodic
        n, dev = self.n, self.dev
        f32 = dict(dtype=torch.float32, device=dev)
        self.m = np.ascontiguousarray(box["m"], np.float32)
        v = torch.as_tensor(np.ascontiguousarray(box["v"], np.float32), device=dev)
        u = torch.as_tensor(np.ascontiguousarray(box["u"], np.float32), device=dev)
        self.t = {
            "x": torch.as_tensor(np.ascontiguousarray(box["x"], np.float64), device=dev),
            "v_full": v.clone(), "v": v.clone(), "a": torch.zeros((n, 3), **f32),
            "u_full": u.clone(), "u": u.clone(), "u_dt": torch.zeros(n, **f32),
            "h": torch.as_tensor(np.ascontiguousarray(box["h"], np.float32), device=dev),
            "h_dt": torch.zeros(n, **f32), "rho": torch.zeros(n, **f32),
            "P": torch.zeros(n, **f32), "c": torch.zeros(n, **f32),
            "v_sig": torch.zeros(n, **f32),
            "time_bin": torch.zeros(n, dtype=torch.int8, device=dev),
            "min_ngb_bin": torch.full((n,), NUM_TIME_BINS + 1, dtype=torch.int8, device=dev),
        }
        # grad-h term and Balsara switch: the force state an inactive
        # particle keeps from its last ghost
        self.f = torch.zeros(n, **f32)
        self.balsara = torch.zeros(n, **f32)
        # the space's results of a step (sphgpu_download's columns)
        self.fields = torch.zeros((n, 24), **f32)
        self.ti_current = 0
        self.ti_end_min = 0
        self.steps = 0
        self.last_active = 0
        self.rebuilds = 0
        self._space = None  # the space of the last rebuild, drifted since

    # -- device state ------------------------------------------------------
    def _state(self):
        st = api.IntegState()
        for k in api.INTEG_FIELDS:
            setattr(st, k, ctypes.c_void_p(self.t[k].data_ptr()))
        return st

    def _stream(self):
        return ctypes.c_void_p(torch.cuda.current_stream(self.dev).cuda_stream)

    def state(self):
        """The particle state as numpy arrays (the caller's order).  Between
        rebuilds positions are not wrapped into the periodic box (the
        reference wraps them at its rebuilds only)."""
        torch.cuda.synchronize(self.dev)
        out = {k: v.cpu().numpy() for k, v in self.t.items()}
        out["f"] = self.f.cpu().numpy()
        out["balsara"] = self.balsara.cpu().numpy()
        return out

    def close(self):
        """Frees the space (the device state stays)."""
        if self._space is not None:
            self._space.close()
            self._space = None

    @property
    def time(self):
        return self.ti_current * self.ip.time_base

    # -- snapshots and restarts ---------------------------------------------
    def save(self, path):
        """Write a snapshot (swift_gb300.snapshot: the PartType0 output
        fields) with the state a restart needs.  The positions get the
        rebuild's periodic wrap first and the next step rebuilds the space,
        as an integrator restarted from the snapshot does: both continue
        from the same cell tree."""
        self._wrap()
        self.close()
        st = self.state()
        fields = {k: st[k] for k in ("x", "v", "h", "u", "rho", "P")}
        fields["m"] = self.m
        restart = {k: st[k] for k in snapshot.RESTART_FIELDS}
        restart.update(ti_current=np.int64(self.ti_current),
                       ti_end_min=np.int64(self.ti_end_min), steps=np.int64(self.steps),
                       log_max_h_change=np.float32(self.ip.log_max_h_change),
                       settings=np.array([self._settings[k] for k in
                                          ("time_end", "cfl", "dt_min", "dt_max", "minimal_u")]))
        if "eta" in self.box_meta:
            restart["eta"] = np.float64(self.box_meta["eta"])
        snapshot.write(path, fields, self.dim, self.time, restart)

    @classmethod
    def restart(cls, path, device="cuda", **space_params):
        """An integrator that continues from a snapshot written by
        :meth:`save`, bit for bit where the original would have gone on."""
        box = snapshot.read(path)
        r = box.pop("restart")
        if "ti_current" not in r:
            raise ValueError(f"{path} is a plain snapshot without restart data")
        if "eta" in r:
            box["eta"] = float(r["eta"])
        time_end, cfl, dt_min, dt_max, minimal_u = (float(v) for v in r["settings"])
        it = cls(box, time_end=time_end, cfl=cfl, dt_min=dt_min, dt_max=dt_max,
                 log_max_h_change=float(r["log_max_h_change"]), minimal_u=minimal_u,
                 device=device, **space_params)
        for k in ("rho", "P"):
            it.t[k].copy_(torch.as_tensor(np.ascontiguousarray(box[k]), device=it.dev))
        for k in snapshot.RESTART_FIELDS:
            if k in ("f", "balsara"):
                continue
            it.t[k].copy_(torch.as_tensor(np.ascontiguousarray(r[k]), device=it.dev))
        it.f.copy_(torch.as_tensor(np.array(r["f"], np.float32), device=it.dev))
        it.balsara.copy_(torch.as_tensor(np.array(r["balsara"], np.float32), device=it.dev))
        it.ti_current = int(r["ti_current"])
        it.ti_end_min = int(r["ti_end_min"])
        it.steps = int(r["steps"])
        return it

    # -- the operations ----------------------------------------------------
    def _kick(self, which, mab):
        L = api.lib()
        api._check(L.sphgpu_integ_kick(ctypes.byref(self.ip), ctypes.byref(self._state()),
                                       self.n, which, self.ti_current, mab, self._stream()))

    def _drift(self, ti_old, ti_new):
        # no wrap: the space keeps every particle in its cell until a rebuild
        L = api.lib()
        api._check(L.sphgpu_integ_drift(ctypes.byref(self.ip), ctypes.byref(self._state()),
                                        self.n, ti_old, ti_new, 0, self._stream()))

    def _wrap(self):
        """The rebuild's periodic wrap of the positions (space_cell_index.c:
        113-123: one box length added or taken off, the far edge to 0)."""
        if not self.ip.periodic:
            return
        x = self.t["x"]
        D = torch.tensor(self.dim, dtype=torch.float64, device=self.dev)[None, :]
        y = torch.where(x < 0.0, x + D, torch.where(x >= D, x - D, x))
        x.copy_(torch.where(y == D, torch.zeros_like(y), y))

    def _timestep(self, mab):
        L = api.lib()
        tmin, bad = ctypes.c_int64(), ctypes.c_int64()
        api._check(L.sphgpu_integ_timestep(ctypes.byref(self.ip), ctypes.byref(self._state()),
                                           self.n, self.ti_current, mab, ctypes.byref(tmin),
                                           ctypes.byref(bad), self._stream()))
        if bad.value:
            raise api.SphGpuError(api.EINVAL, f"{bad.value} particles want a time step "
                                  f"below dt_min ({self.ip.dt_min})")
        self.ti_end_min = tmin.value

    def _rebuild(self, mab):
        """A new space from the current state: the periodic wrap, the cell
        assignment on the device from the positions in HBM, the host
        planner on the adopted tree (the one host copy of the state)."""
        self.close()
        self._wrap()
        torch.cuda.synchronize(self.dev)
        host = {k: self.t[k].cpu().numpy() for k in ("x", "v", "h", "u", "time_bin")}
        box = dict(x=host["x"], v=host["v"], m=self.m, h=host["h"], u=host["u"],
                   time_bin=host["time_bin"], dim=self.dim, **self.box_meta)
        assigned = None
        if self.device_rebuild:
            order, _, cells, _ = api.cell_assign(self.t["x"], self.t["h"], self.dim,
                                                 **self.space_params)
            assigned = (order, cells)
        self._space = api.Space(box, assigned=assigned, max_active_bin=mab,
                                **self.space_params)
        self.rebuilds += 1

    def _hydro(self, mab, stages=api.STAGE_ALL):
        """density -> ghost (-> force) for the particles with time_bin <= mab,
        on the space of the last rebuild when the drifted state allows it
        (sphgpu_space_drift), else on a new one.  Results stay on the
        device."""
        t = self.t
        # the space works on its own stream: the drift's state must be there
        torch.cuda.current_stream(self.dev).synchronize()
        if self._space is not None:
            try:
                self._space.drift(t["x"], t["h"])
            except api.SphGpuError as e:
                if e.code != api.EREBUILD:
                    raise
                self.close()
        if self._space is None:
            self._rebuild(mab)
        sp = self._space
        # the caller's state for this step: what the kicks and the drift
        # made of v and u, and the force inputs the inactive particles lend
        sp.set_state(v=t["v"], u=t["u"], rho=t["rho"], f=self.f, pressure=t["P"],
                     soundspeed=t["c"], balsara=self.balsara, time_bin=t["time_bin"])
        sp.set_active(mab)
        sp.step(stages)
        F = sp.download_into(self.fields)  # complete on return
        act = t["time_bin"] <= mab
        self.last_active = int(act.sum())
        for k, col in (("h", "h"), ("rho", "rho"), ("P", "pressure"), ("c", "soundspeed")):
            t[k].copy_(torch.where(act, F[:, api.FIELD_COLS[col]], t[k]))
        self.f.copy_(torch.where(act, F[:, api.FIELD_COLS["f"]], self.f))
        self.balsara.copy_(torch.where(act, F[:, api.FIELD_COLS["balsara"]], self.balsara))
        if not stages & api.STAGE_FORCE:
            return
        c0 = api.FIELD_COLS["ax"]
        t["a"].copy_(torch.where(act[:, None], F[:, c0:c0 + 3], t["a"]))
        for k in ("u_dt", "h_dt", "v_sig"):
            t[k].copy_(torch.where(act, F[:, api.FIELD_COLS[k]], t[k]))
        nb = F[:, api.FIELD_COLS["min_ngb_bin"]].to(torch.int8)
        t["min_ngb_bin"].copy_(torch.where(act, nb, t["min_ngb_bin"]))

    # -- the engine sequence -----------------------------------------------
    def init(self):
        """engine_init_particles: a density / ghost pass to settle h, then
        the initial step at ti = 0 with every particle active (force, kick2
        over a zero interval, time steps, kick1)."""
        mab = NUM_TIME_BINS
        self._hydro(mab, api.STAGE_DENSITY | api.STAGE_GHOST)
        self._hydro(mab)
        self._kick(2, mab)
        self._timestep(mab)
        self._kick(1, mab)
        return self

    def step(self):
        """engine_step: advance to the next synchronisation point."""
        ti_old = self.ti_current
        self.ti_current = self.ti_end_min
        mab = api.lib().sphgpu_integ_max_active_bin(self.ti_current)
        self._drift(ti_old, self.ti_current)
        self._hydro(mab)
        self._kick(2, mab)
        self._timestep(mab)
        self._kick(1, mab)
        self.steps += 1
        return mab
