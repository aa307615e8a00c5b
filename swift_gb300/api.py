"""Python host mirror of the C ABI (include/swift_gb300.h).

The reference's host for this path is C (runner_main.c dispatching
runner_dosub_*_density/force and runner_do_ghost); this module is the thin
Python face of the same C-ABI library, used by the tests, the benchmark and
the serving loop.  Arrays are NumPy; nothing here computes physics.  If the
compiled library is missing the import fails loudly: there is no CPU
fallback.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from . import build as _build

STAGE_DENSITY, STAGE_GHOST, STAGE_FORCE, STAGE_ALL = 1, 2, 4, 7
ALL_ACTIVE = 127  # max_active_bin that activates every time bin
STAGE_PRIME = 8  # oracle/run flag: a full all-active step runs first
OK, EINVAL, ECUDA, ENOMEM, ENOCONV, ESTATE, ENODEV, EREBUILD = 0, -1, -2, -3, -4, -5, -6, -7

FIELD_COLS = {
    "d_rho": 0, "d_rho_dh": 1, "d_wcount": 2, "d_wcount_dh": 3, "d_div_v": 4,
    "d_rot_vx": 5, "d_rot_vy": 6, "d_rot_vz": 7,
    "h": 8, "rho": 9, "f": 10, "pressure": 11, "soundspeed": 12,
    "balsara": 13, "v_sig_ghost": 14,
    "ax": 15, "ay": 16, "az": 17, "u_dt": 18, "h_dt": 19, "v_sig": 20,
    "min_ngb_bin": 21,
}
INT_COLS = {"ngb_first": 0, "ngb_final": 1, "ngb_force": 2, "ghost_iters": 3}
CELL_COLS = {"leaf_first": 0, "leaf_count": 1, "leaf_depth": 2, "depth_h": 3,
             "position": 4, "top": 5}


class SphGpuError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"sphgpu error {code}: {msg}")
        self.code = code


class Params(ctypes.Structure):
    _fields_ = [("dim", ctypes.c_double * 3), ("periodic", ctypes.c_int32),
                ("eta", ctypes.c_float), ("h_tolerance", ctypes.c_float),
                ("h_max", ctypes.c_float), ("h_min", ctypes.c_float),
                ("alpha", ctypes.c_float), ("max_iter", ctypes.c_int32),
                ("max_active_bin", ctypes.c_int32),
                ("max_top_level_cells", ctypes.c_int32)]


class Tuning(ctypes.Structure):
    _fields_ = [("threads_per_particle", ctypes.c_int32),
                ("jtile", ctypes.c_int32), ("rerun_lists", ctypes.c_int32),
                ("block_warps", ctypes.c_int32), ("bulk_stage", ctypes.c_int32),
                ("row_widen", ctypes.c_float), ("row_cap", ctypes.c_int32),
                ("tc_filter", ctypes.c_int32)]


class IntegParams(ctypes.Structure):
    _fields_ = [("time_base", ctypes.c_double), ("dt_min", ctypes.c_double),
                ("dt_max", ctypes.c_double), ("CFL", ctypes.c_float),
                ("log_max_h_change", ctypes.c_float), ("h_min", ctypes.c_float),
                ("h_max", ctypes.c_float), ("minimal_u", ctypes.c_float),
                ("dim", ctypes.c_double * 3), ("periodic", ctypes.c_int32)]


INTEG_FIELDS = ("x", "v_full", "v", "a", "u_full", "u", "u_dt", "h", "h_dt", "rho",
                "P", "c", "v_sig", "time_bin", "min_ngb_bin")


class IntegState(ctypes.Structure):
    _fields_ = [(k, ctypes.c_void_p) for k in INTEG_FIELDS]


# Every symbol the header declares, with its ctypes signature.
_P = ctypes.c_void_p
_I32 = ctypes.c_int32
SIGNATURES = {
    "sphgpu_abi_version": (ctypes.c_int, []),
    "sphgpu_last_error": (ctypes.c_char_p, []),
    "sphgpu_default_params": (None, [ctypes.POINTER(Params)]),
    "sphgpu_space_create": (ctypes.c_int, [ctypes.POINTER(Params), ctypes.c_int64,
                                           _P, _P, _P, _P, _P, _P,
                                           ctypes.POINTER(_P)]),
    "sphgpu_space_destroy": (ctypes.c_int, [_P]),
    "sphgpu_space_info": (ctypes.c_int, [_P, _P]),
    "sphgpu_space_cells": (ctypes.c_int, [_P, _P]),
    "sphgpu_space_leaves": (ctypes.c_int, [_P, _P, _P]),
    "sphgpu_set_active": (ctypes.c_int, [_P, _I32]),
    "sphgpu_set_tuning": (ctypes.c_int, [_P, ctypes.POINTER(Tuning)]),
    "sphgpu_get_tuning": (ctypes.c_int, [_P, ctypes.POINTER(Tuning)]),
    "sphgpu_step": (ctypes.c_int, [_P, _I32, _P]),
    "sphgpu_step_host": (ctypes.c_int, [_P, _P, _P, _P, _P, _P, _P, _P]),
    "sphgpu_space_update": (ctypes.c_int, [_P, _P, _P, _P, _P]),
    "sphgpu_step_stats": (ctypes.c_int, [_P, _P, _I32]),
    "sphgpu_step_plain": (ctypes.c_int, [_P, _P]),
    "sphgpu_step_host_async": (ctypes.c_int, [_P, _P, _P, _P, _P, _P, _P]),
    "sphgpu_step_host_wait": (ctypes.c_int, [_P]),
    "sphgpu_download": (ctypes.c_int, [_P, _P, _P]),
    "sphgpu_force_from_state": (ctypes.c_int, [_P, _P, _P, _P, _P, _P, _P, _P]),
    "sphgpu_download_min_ngb_bin": (ctypes.c_int, [_P, _P]),
    "sphgpu_integ_kick": (ctypes.c_int, [ctypes.POINTER(IntegParams), ctypes.POINTER(IntegState),
                                         ctypes.c_int64, _I32, ctypes.c_int64, _I32, _P]),
    "sphgpu_integ_drift": (ctypes.c_int, [ctypes.POINTER(IntegParams), ctypes.POINTER(IntegState),
                                          ctypes.c_int64, ctypes.c_int64, ctypes.c_int64, _I32,
                                          _P]),
    "sphgpu_integ_timestep": (ctypes.c_int, [ctypes.POINTER(IntegParams),
                                             ctypes.POINTER(IntegState), ctypes.c_int64,
                                             ctypes.c_int64, _I32, _P, _P, _P]),
    "sphgpu_integ_max_active_bin": (ctypes.c_int, [ctypes.c_int64]),
    "sphgpu_begin_loops": (ctypes.c_int, [_P, _P]),
    "sphgpu_dosub_self1_density": (ctypes.c_int, [_P, _I32, _P]),
    "sphgpu_dosub_pair1_density": (ctypes.c_int, [_P, _I32, _I32, _P]),
    "sphgpu_do_ghost": (ctypes.c_int, [_P, _I32, _P]),
    "sphgpu_dosub_self2_force": (ctypes.c_int, [_P, _I32, _P]),
    "sphgpu_dosub_pair2_force": (ctypes.c_int, [_P, _I32, _I32, _P]),
    "sphgpu_do_end_hydro_force": (ctypes.c_int, [_P, _P]),
    "sphgpu_phase_times": (ctypes.c_int, [_P, _P, _P, _I32]),
    "sphgpu_host_times": (ctypes.c_int, [_P, _P, _I32]),
    "sphgpu_set_device_planning": (ctypes.c_int, [_P, _I32]),
    "sphgpu_space_drift": (ctypes.c_int, [_P, _P, _P, _P]),
    "sphgpu_space_set_state": (ctypes.c_int, [_P, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P]),
    "sphgpu_plan_times": (ctypes.c_int, [_P, _P, _P, _I32]),
    "sphgpu_check_device_plans": (ctypes.c_int, [_P, _P]),
    "sphgpu_count_hits": (ctypes.c_int, [_P, _P]),
    "sphgpu_density_noalloc": (ctypes.c_int, [_P, _P, _P, _P]),
    "sphgpu_autotune": (ctypes.c_int, [_P, _I32, _P, _P, _P]),
    "sphgpu_hydro_sort": (ctypes.c_int, [_P, _I32, _P]),
    "sphgpu_space_tree": (ctypes.c_int, [_P, _P, _P]),
    "sphgpu_cell_sort": (ctypes.c_int, [_P, _I32, _I32, _P, _P]),
    "sphgpu_cell_assign": (ctypes.c_int, [ctypes.POINTER(Params), _P, _P, ctypes.c_int64, _P,
                                          _P, _P, _P, _P, _I32, _P]),
    "sphgpu_cell_assign_times": (ctypes.c_int, [_P]),
    "sphgpu_space_create_assigned": (ctypes.c_int, [ctypes.POINTER(Params), ctypes.c_int64,
                                                    _P, _P, _P, _P, _P, _P, _P, _P, _I32,
                                                    ctypes.POINTER(_P)]),
    "sphgpu_server_create": (ctypes.c_int, [ctypes.POINTER(Params), ctypes.c_int64, _I32,
                                            ctypes.POINTER(_P)]),
    "sphgpu_server_destroy": (ctypes.c_int, [_P]),
    "sphgpu_server_submit": (ctypes.c_int, [_P, ctypes.c_int64, ctypes.POINTER(Params),
                                            ctypes.c_int64, _P, _P, _P, _P, _P, _I32]),
    "sphgpu_server_pump": (ctypes.c_int, [_P, ctypes.c_double, _P]),
    "sphgpu_server_poll": (ctypes.c_int, [_P, _P, _I32, _P]),
    "sphgpu_server_fetch": (ctypes.c_int, [_P, ctypes.c_int64, _P, _P, _P]),
    "sphgpu_server_stats": (ctypes.c_int, [_P, _P]),
    "sphgpu_server_times": (ctypes.c_int, [_P, _P]),
}

_lib = None


def lib(build_if_missing=True):
    """Load the in-tree library (building it first if allowed)."""
    global _lib
    if _lib is not None:
        return _lib
    path = _build.LIB
    if build_if_missing:
        path = _build.build()
    if not os.path.exists(path):
        raise ImportError(f"swift_gb300: compiled library missing at {path}; "
                          "run swift_gb300.build.build()")
    L = ctypes.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return L


def _check(rc):
    if rc != OK:
        msg = lib().sphgpu_last_error()
        raise SphGpuError(rc, msg.decode() if msg else "")


def _ptr(a):
    return ctypes.c_void_p(a.ctypes.data) if a is not None else None


def make_params(box, **kw):
    L = lib()
    p = Params()
    L.sphgpu_default_params(ctypes.byref(p))
    d = box["dim"]
    p.dim[:] = list(d) if np.ndim(d) else [d, d, d]
    p.eta = kw.get("eta", box.get("eta", p.eta))
    for k in ("periodic", "h_tolerance", "h_max", "h_min", "alpha", "max_iter",
              "max_top_level_cells"):
        if k in kw:
            setattr(p, k, kw[k])
    p.max_active_bin = kw.get("max_active_bin", box.get("max_active_bin",
                                                        p.max_active_bin))
    return p


def cell_assign(x, h, dim, **params):
    """The rebuild's cell assignment on the device (sphgpu_cell_assign).

    ``x`` [n, 3] float64 and ``h`` [n] float32 are CUDA tensors (the caller's
    order; numpy arrays are copied to the current CUDA device).  Returns
    ``(order, depth_h, cells, cdim)``: ``order`` (int32) gives the caller's
    index of every particle in cell order and ``depth_h`` (int8) its h-depth,
    both CUDA tensors; ``cells`` is the int32 [ncells, 5] tree (first, count,
    depth, parent, top; the numbering of :meth:`Space.tree`); ``cdim`` the
    top-level grid."""
    import torch
    dev = torch.device("cuda", torch.cuda.current_device())
    x = torch.as_tensor(x, dtype=torch.float64, device=dev).contiguous()
    h = torch.as_tensor(h, dtype=torch.float32, device=dev).contiguous()
    n = int(h.shape[0])
    if x.shape != (n, 3):
        raise ValueError("x must be [n, 3] with n = len(h)")
    prm = make_params({"dim": dim}, **params)
    order = torch.empty(n, dtype=torch.int32, device=dev)
    depth_h = torch.empty(n, dtype=torch.int8, device=dev)
    cdim = np.zeros(3, np.int32)
    ncells = ctypes.c_int32()
    # top cells + 8 children for each split cell (> 400 particles), with
    # room for four levels of splits; a deeper tree is fetched again
    cap = (prm.max_top_level_cells + 2) ** 3 + 32 * (n // 401) + 64
    stream = ctypes.c_void_p(torch.cuda.current_stream(dev).cuda_stream)
    for _ in range(2):
        cells = np.zeros((cap, 5), np.int32)
        rc = lib().sphgpu_cell_assign(ctypes.byref(prm), ctypes.c_void_p(x.data_ptr()),
                                      ctypes.c_void_p(h.data_ptr()), n,
                                      ctypes.c_void_p(order.data_ptr()),
                                      ctypes.c_void_p(depth_h.data_ptr()), _ptr(cdim),
                                      ctypes.byref(ncells), _ptr(cells), cap, stream)
        if rc == OK or ncells.value <= cap:
            break
        cap = ncells.value
    _check(rc)
    return order, depth_h, cells[:ncells.value].copy(), tuple(int(v) for v in cdim)


def cell_assign_times():
    """Host-clock phases (ms) of this thread's last :func:`cell_assign`: h scan
    and grid, keys and sort, tree levels, numbering and records, depth_h; and
    the number of kernels it launched."""
    ms = np.zeros(6, np.float64)
    _check(lib().sphgpu_cell_assign_times(_ptr(ms)))
    return dict(zip(("grid", "keys_sort", "tree_levels", "numbering", "depth_h", "launches"),
                    (float(v) for v in ms)))


def tuning_key(jtile, tpp, block_warps):
    """Name of an autotuner candidate."""
    return f"jtile={jtile},tpp={tpp},block_warps={block_warps}"


class Space:
    """A box of SPH particles with its cell tree, resident on the GPU once a
    GPU call is made.  Mirrors the reference's space + runner entry points."""

    def __init__(self, box, assigned=None, **params):
        """``assigned``: optionally ``(order, cells)`` from :func:`cell_assign`
        (order as a host or CUDA int32 array), adopted instead of the host's
        own cell assignment."""
        L = lib()
        self.n = int(box["x"].shape[0])
        self._keep = {
            "x": np.ascontiguousarray(box["x"], np.float64),
            "v": np.ascontiguousarray(box["v"], np.float32),
            "m": np.ascontiguousarray(box["m"], np.float32),
            "h": np.ascontiguousarray(box["h"], np.float32),
            "u": np.ascontiguousarray(box["u"], np.float32),
            "tb": np.ascontiguousarray(box["time_bin"], np.int8),
        }
        k = self._keep
        self.params = make_params(box, **params)
        h = ctypes.c_void_p()
        if assigned is None:
            _check(L.sphgpu_space_create(ctypes.byref(self.params), self.n,
                                         _ptr(k["x"]), _ptr(k["v"]), _ptr(k["m"]),
                                         _ptr(k["h"]), _ptr(k["u"]), _ptr(k["tb"]),
                                         ctypes.byref(h)))
        else:
            order, cells = assigned
            if hasattr(order, "cpu"):
                order = order.cpu().numpy()
            order = np.ascontiguousarray(order, np.int32)
            cells = np.ascontiguousarray(cells, np.int32)
            _check(L.sphgpu_space_create_assigned(
                ctypes.byref(self.params), self.n, _ptr(k["x"]), _ptr(k["v"]), _ptr(k["m"]),
                _ptr(k["h"]), _ptr(k["u"]), _ptr(k["tb"]), _ptr(order), _ptr(cells),
                int(cells.shape[0]), ctypes.byref(h)))
        self._h = h

    # -- lifecycle ---------------------------------------------------------
    def close(self):
        if getattr(self, "_h", None):
            lib().sphgpu_space_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # -- tree --------------------------------------------------------------
    def info(self):
        out = np.zeros(8, np.int64)
        _check(lib().sphgpu_space_info(self._h, _ptr(out)))
        keys = ("n", "cdim0", "cdim1", "cdim2", "cells", "leaves", "tasks",
                "entries")
        return dict(zip(keys, (int(v) for v in out)))

    def cells(self):
        out = np.zeros((self.n, 6), np.int32)
        _check(lib().sphgpu_space_cells(self._h, _ptr(out)))
        return {name: out[:, col] for name, col in CELL_COLS.items()}

    def leaves(self):
        nl = self.info()["leaves"]
        geom = np.zeros((nl, 6), np.float64)
        ints = np.zeros((nl, 3), np.int32)
        _check(lib().sphgpu_space_leaves(self._h, _ptr(geom), _ptr(ints)))
        return geom, ints

    # -- configuration -----------------------------------------------------
    def set_tuning(self, tpp=1, jtile=16, rerun_lists=1, block_warps=8, bulk_stage=0,
                   row_widen=0.0, row_cap=0, tc_filter=0):
        t = Tuning(tpp, jtile, rerun_lists, block_warps, bulk_stage, row_widen, row_cap,
                   tc_filter)
        _check(lib().sphgpu_set_tuning(self._h, ctypes.byref(t)))

    def bulk_stage(self):
        """1 when the gathers stage j-blocks by bulk copies."""
        t = Tuning()
        _check(lib().sphgpu_get_tuning(self._h, ctypes.byref(t)))
        return t.bulk_stage

    def tuning(self):
        t = Tuning()
        _check(lib().sphgpu_get_tuning(self._h, ctypes.byref(t)))
        return (t.threads_per_particle, t.jtile, t.rerun_lists, t.block_warps)

    def tree(self):
        """Cell records: first, count, depth, parent, top (one row per cell)."""
        n = ctypes.c_int32()
        _check(lib().sphgpu_space_tree(self._h, ctypes.byref(n), None))
        rec = np.zeros((n.value, 5), np.int32)
        _check(lib().sphgpu_space_tree(self._h, ctypes.byref(n), _ptr(rec)))
        return rec

    def hydro_sort(self, flags=0x1FFF):
        _check(lib().sphgpu_hydro_sort(self._h, int(flags), None))

    def cell_sort(self, cell, axis, count):
        d = np.zeros(count + 1, np.float32)
        i = np.zeros(count + 1, np.int32)
        _check(lib().sphgpu_cell_sort(self._h, int(cell), int(axis), _ptr(d), _ptr(i)))
        return d, i

    def autotune(self, reps=3):
        """Pick the fastest gather configuration for this box (native
        autotuner); returns ({jtile, block_warps, ...}, {config: ms})."""
        best = Tuning()
        ms = np.zeros(24, np.float32)
        n = ctypes.c_int32()
        _check(lib().sphgpu_autotune(self._h, int(reps), ctypes.byref(best),
                                     _ptr(ms), ctypes.byref(n)))
        shapes = [(jt, tpp, bw) for jt in (32, 16, 8) for tpp in (1, 2) for bw in (8, 4)]
        cands = [tuning_key(*sh) for sh in shapes]
        # the fastest shape of each lane count (the first of equal times)
        for lanes in (1, 2):
            ks = [k for k, sh in enumerate(shapes) if sh[1] == lanes]
            kb = min(ks, key=lambda k: (ms[k], k))
            cands += [f"{cands[kb]},row_widen={w}" for w in (1.32, 1.44, 1.56, 1.69)]
        table = {name: float(ms[k]) for k, name in enumerate(cands[:n.value])}
        return ({"threads_per_particle": best.threads_per_particle,
                 "jtile": best.jtile, "rerun_lists": best.rerun_lists,
                 "block_warps": best.block_warps,
                 "row_widen": round(float(best.row_widen), 4)}, table)

    def set_active(self, max_active_bin):
        _check(lib().sphgpu_set_active(self._h, int(max_active_bin)))

    # -- GPU passes --------------------------------------------------------
    def step(self, stages=STAGE_ALL, stream=None):
        _check(lib().sphgpu_step(self._h, stages, stream))

    def step_plain(self, stream=None):
        _check(lib().sphgpu_step_plain(self._h, stream))

    def primed_step(self, max_active_bin, stages=STAGE_ALL, plain=False):
        """Two steps: every particle active, then ``stages`` at
        ``max_active_bin`` on the state the first leaves (active particles
        restart from the input h; inactive ones keep h, density and force
        state, which their active neighbours' loops read)."""
        self.set_active(ALL_ACTIVE)
        self.step()
        self.set_active(max_active_bin)
        if plain:
            self.step_plain()
        else:
            self.step(stages)

    def set_state(self, v=None, m=None, u=None, rho=None, f=None, pressure=None,
                  soundspeed=None, balsara=None, time_bin=None, stream=None):
        """A caller's particle state (input order; numpy arrays or CUDA
        tensors; None keeps the space's): see sphgpu_space_set_state."""
        keep = []

        def ptr(a, dtype, shape):
            if a is None:
                return None
            if hasattr(a, "data_ptr"):
                assert a.is_contiguous() and tuple(a.shape) == shape
                assert a.element_size() == np.dtype(dtype).itemsize
                keep.append(a)
                return ctypes.c_void_p(a.data_ptr())
            a = np.ascontiguousarray(a, dtype)
            assert a.shape == shape
            keep.append(a)
            return _ptr(a)
        n = self.n
        _check(lib().sphgpu_space_set_state(
            self._h, ptr(v, np.float32, (n, 3)), ptr(m, np.float32, (n,)),
            ptr(u, np.float32, (n,)), ptr(rho, np.float32, (n,)), ptr(f, np.float32, (n,)),
            ptr(pressure, np.float32, (n,)), ptr(soundspeed, np.float32, (n,)),
            ptr(balsara, np.float32, (n,)), ptr(time_bin, np.int8, (n,)), stream))

    def download_into(self, fields):
        """Results into a caller's float32 [n][24] array (a CUDA tensor or
        a numpy array), sphgpu_download's column layout."""
        assert tuple(fields.shape) == (self.n, 24)
        if hasattr(fields, "data_ptr"):
            assert fields.is_contiguous() and fields.element_size() == 4
            p = ctypes.c_void_p(fields.data_ptr())
        else:
            assert fields.flags["C_CONTIGUOUS"] and fields.dtype == np.float32
            p = _ptr(fields)
        _check(lib().sphgpu_download(self._h, p, None))
        return fields

    def drift(self, x, h, stream=None):
        """New positions and h (input order; numpy arrays or CUDA tensors)
        without a rebuild; raises SphGpuError(EREBUILD) when the particles
        moved too far for the cell tree (the space is then unchanged)."""
        def ptr(a, dtype, shape):
            if hasattr(a, "data_ptr"):
                assert a.is_contiguous() and tuple(a.shape) == shape
                assert a.element_size() == np.dtype(dtype).itemsize and a.is_floating_point()
                return ctypes.c_void_p(a.data_ptr()), a
            a = np.ascontiguousarray(a, dtype)
            assert a.shape == shape
            return _ptr(a), a
        px, kx = ptr(x, np.float64, (self.n, 3))
        ph, kh = ptr(h, np.float32, (self.n,))
        _check(lib().sphgpu_space_drift(self._h, px, ph, stream))
        del kx, kh

    def set_device_planning(self, on=True):
        """Device planning of sparse steps' gather lists (on by default)."""
        _check(lib().sphgpu_set_device_planning(self._h, int(bool(on))))

    def plan_times(self, reset=False):
        """(ms of device planning summed over device-planned steps, steps)."""
        ms = ctypes.c_double()
        steps = ctypes.c_int64()
        _check(lib().sphgpu_plan_times(self._h, ctypes.byref(ms), ctypes.byref(steps),
                                       int(bool(reset))))
        return ms.value, steps.value

    def check_device_plans(self):
        """Device plans of the last step against the host planner's for the
        same state: {density, rerun, force}: (differing pairs, pairs)."""
        out = np.zeros(6, np.int64)
        _check(lib().sphgpu_check_device_plans(self._h, _ptr(out)))
        return {k: (int(out[i]), int(out[3 + i]))
                for i, k in enumerate(("density", "rerun", "force"))}

    def step_stats(self, reset=False):
        """{graph_steps, force_replans, late_rounds, captures} since the last
        reset (force_replans: steps run a second time outside the graph)."""
        out = np.zeros(4, np.int64)
        _check(lib().sphgpu_step_stats(self._h, _ptr(out), int(bool(reset))))
        return dict(zip(("graph_steps", "force_replans", "late_rounds", "captures"),
                        (int(v) for v in out)))

    def update(self, v, m, u, stream=None):
        """New velocities, masses and internal energies (input order), e.g.
        after a kick; positions and h stay the space's."""
        arrs = [np.ascontiguousarray(v, np.float32), np.ascontiguousarray(m, np.float32),
                np.ascontiguousarray(u, np.float32)]
        _check(lib().sphgpu_space_update(self._h, *[_ptr(a) for a in arrs], stream))

    def step_host(self, box=None, fields=None, stream=None):
        b = self._keep if box is None else {
            "x": np.ascontiguousarray(box["x"], np.float64),
            "v": np.ascontiguousarray(box["v"], np.float32),
            "m": np.ascontiguousarray(box["m"], np.float32),
            "h": np.ascontiguousarray(box["h"], np.float32),
            "u": np.ascontiguousarray(box["u"], np.float32)}
        _check(lib().sphgpu_step_host(self._h, _ptr(b["x"]), _ptr(b["v"]),
                                      _ptr(b["m"]), _ptr(b["h"]), _ptr(b["u"]),
                                      _ptr(fields), stream))
        return fields

    def step_host_async(self, box, fields):
        """Pipelined step through host buffers (sphgpu_step_host_async):
        ``box`` arrays and ``fields`` must stay alive until step_host_wait
        (or two calls later); pinned buffers make the copies overlap."""
        b = {k: box[k] for k in ("x", "v", "m", "h", "u")}
        _check(lib().sphgpu_step_host_async(self._h, _ptr(b["x"]), _ptr(b["v"]),
                                            _ptr(b["m"]), _ptr(b["h"]), _ptr(b["u"]),
                                            _ptr(fields)))
        return fields

    def step_host_wait(self):
        _check(lib().sphgpu_step_host_wait(self._h))

    def host_times(self, reset=False):
        """Host planning in ms: activation lists, activation uploads, force
        lists planned inside steps."""
        ms = np.zeros(3, np.float64)
        _check(lib().sphgpu_host_times(self._h, _ptr(ms), int(bool(reset))))
        return {"activation_planning": ms[0], "activation_upload": ms[1],
                "force_planning": ms[2]}

    def phase_times(self, reset=False):
        """(ms summed per loop [density, ghost, force], steps timed)."""
        ms = np.zeros(3, np.float64)
        steps = ctypes.c_int64()
        _check(lib().sphgpu_phase_times(self._h, _ptr(ms), ctypes.byref(steps),
                                        1 if reset else 0))
        return ms, steps.value

    def count_hits(self):
        """Neighbour interactions of one pass: density first pass, ghost
        re-runs, force, density at the converged h."""
        out = np.zeros(4, np.int64)
        _check(lib().sphgpu_count_hits(self._h, _ptr(out)))
        return out

    def download(self):
        fields = np.zeros((self.n, 24), np.float32)
        ints = np.zeros((self.n, 4), np.int32)
        _check(lib().sphgpu_download(self._h, _ptr(fields), _ptr(ints)))
        out = {"fields": fields, "ints": ints}
        for name, col in FIELD_COLS.items():
            out[name] = fields[:, col]
        for name, col in INT_COLS.items():
            out[name] = ints[:, col]
        return out

    def min_ngb_bin(self):
        """Smallest time bin > 0 among each particle's force neighbours (last
        force pass; 57 when it has none)."""
        out = np.zeros(self.n, np.int8)
        _check(lib().sphgpu_download_min_ngb_bin(self._h, _ptr(out)))
        return out

    def force_from_state(self, h, rho, f, pressure, soundspeed, balsara):
        arrs = [np.ascontiguousarray(a, np.float32)
                for a in (h, rho, f, pressure, soundspeed, balsara)]
        _check(lib().sphgpu_force_from_state(self._h, *[_ptr(a) for a in arrs],
                                             None))

    # -- drop-in per-task entry points --------------------------------------
    def begin_loops(self):
        _check(lib().sphgpu_begin_loops(self._h, None))

    def dosub_self1_density(self, cell):
        _check(lib().sphgpu_dosub_self1_density(self._h, int(cell), None))

    def dosub_pair1_density(self, ci, cj):
        _check(lib().sphgpu_dosub_pair1_density(self._h, int(ci), int(cj), None))

    def do_ghost(self, cell):
        _check(lib().sphgpu_do_ghost(self._h, int(cell), None))

    def dosub_self2_force(self, cell):
        _check(lib().sphgpu_dosub_self2_force(self._h, int(cell), None))

    def dosub_pair2_force(self, ci, cj):
        _check(lib().sphgpu_dosub_pair2_force(self._h, int(ci), int(cj), None))

    def do_end_hydro_force(self):
        _check(lib().sphgpu_do_end_hydro_force(self._h, None))


class Server:
    """Continuous-batching serving loop: independent boxes resident in one
    device arena, every resident box advanced one step per ``pump()`` by the
    same persistent launches (include/swift_gb300.h, sphgpu_server_*)."""

    def __init__(self, max_particles=0, planner_threads=0, **params):
        L = lib()
        self.params = make_params({"dim": 1.0}, **params)
        h = ctypes.c_void_p()
        _check(L.sphgpu_server_create(ctypes.byref(self.params), int(max_particles),
                                      int(planner_threads), ctypes.byref(h)))
        self._h = h
        self._n = {}

    def close(self):
        if self._h:
            lib().sphgpu_server_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def submit(self, rid, box, nsteps=10, **params):
        n = int(box["x"].shape[0])
        bp = make_params(box, **params)
        arrs = [np.ascontiguousarray(box["x"], np.float64),
                np.ascontiguousarray(box["v"], np.float32),
                np.ascontiguousarray(box["m"], np.float32),
                np.ascontiguousarray(box["h"], np.float32),
                np.ascontiguousarray(box["u"], np.float32)]
        _check(lib().sphgpu_server_submit(self._h, int(rid), ctypes.byref(bp), n,
                                          *[_ptr(a) for a in arrs], int(nsteps)))
        self._n[int(rid)] = n

    def pump(self, wait_s=0.0):
        """Admit what fits, advance every resident box one step, retire the
        finished ones; returns the number of resident boxes."""
        r = ctypes.c_int32()
        _check(lib().sphgpu_server_pump(self._h, float(wait_s), ctypes.byref(r)))
        return r.value

    def poll(self, max_ids=4096):
        ids = np.zeros(max_ids, np.int64)
        c = ctypes.c_int32()
        _check(lib().sphgpu_server_poll(self._h, _ptr(ids), int(max_ids), ctypes.byref(c)))
        return [int(i) for i in ids[:c.value]]

    def fetch(self, rid):
        n = self._n.pop(int(rid))
        fields = np.zeros((n, 24), np.float32)
        ints = np.zeros((n, 4), np.int32)
        t = np.zeros(3, np.float64)
        _check(lib().sphgpu_server_fetch(self._h, int(rid), _ptr(fields), _ptr(ints), _ptr(t)))
        out = {"fields": fields, "ints": ints, "t_submit": t[0], "t_admit": t[1],
               "t_done": t[2]}
        for name, col in FIELD_COLS.items():
            out[name] = fields[:, col]
        for name, col in INT_COLS.items():
            out[name] = ints[:, col]
        return out

    def stats(self):
        st = np.zeros(8, np.int64)
        _check(lib().sphgpu_server_stats(self._h, _ptr(st)))
        keys = ("resident", "arena_particles_used", "arena_particles", "waiting",
                "pumps", "retired", "arena_bytes", "free_hbm_at_start")
        out = dict(zip(keys, (int(v) for v in st)))
        t = np.zeros(4, np.float64)
        _check(lib().sphgpu_server_times(self._h, _ptr(t)))
        out.update(zip(("gpu_s", "force_plan_s", "admit_s", "retire_s"),
                       (float(v) for v in t)))
        return out
