"""ctypes front end of the oracle's C restatement (oracle/sph_oracle.c).

Test infrastructure only: tests, the smoke check and bench.py's CPU-baseline
leg use it as the checker; the GPU library never imports it.  ``build()``
compiles the restatement with the same floating-point flags as the parity
build of the reference (no fast-math, no FMA contraction), so that its sums
can be compared bit for bit with the reference's own loops.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

from .io import COLS, INT_COLS

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libsphoracle.so")
# The timed CPU baseline: the same restatement built with the reference's own
# optimisation flags (m4/ax_cc_maxopt.m4 for gcc: -O3 -ffast-math
# -funroll-loops -fomit-frame-pointer and the host's own CPU tuning).  Its
# sums are not bit-identical to the parity build's; it is never used to check.
LIB_STOCK = os.path.join(BUILD, "libsphoracle_stock.so")


def stock_flags():
    import platform
    native = "-march=native" if platform.machine() in ("x86_64", "AMD64") else "-mcpu=native"
    return ["-O3", "-ffast-math", "-funroll-loops", "-fomit-frame-pointer", native]


NFIELDS, NINTS = 24, 11
STAGE_DENSITY, STAGE_GHOST, STAGE_FORCE = 1, 2, 4
ALL = 7


class Params(ctypes.Structure):
    _fields_ = [("dim", ctypes.c_double * 3), ("periodic", ctypes.c_int32),
                ("eta", ctypes.c_float), ("h_tolerance", ctypes.c_float),
                ("h_max", ctypes.c_float), ("h_min", ctypes.c_float),
                ("alpha", ctypes.c_float), ("max_iter", ctypes.c_int32),
                ("max_active_bin", ctypes.c_int32),
                ("max_top_level_cells", ctypes.c_int32),
                ("subsize_self", ctypes.c_int32), ("subsize_pair", ctypes.c_int32),
                ("reverse_tasks", ctypes.c_int32)]


class Result(ctypes.Structure):
    _fields_ = [("fields", ctypes.POINTER(ctypes.c_float)),
                ("ints", ctypes.POINTER(ctypes.c_int32)),
                ("cdim", ctypes.c_int32 * 3), ("ncells", ctypes.c_int32),
                ("status", ctypes.c_int32), ("ntasks", ctypes.c_int32)]


def build(force=False, stock=False):
    """Compile the restatement: the parity build (no fast-math, no FMA
    contraction; the checker) or, with stock=True, the timed baseline."""
    srcs = [os.path.join(HERE, f) for f in ("sph_oracle.c", "sph_integrate.c")]
    out = LIB_STOCK if stock else LIB
    newest = max(os.path.getmtime(f) for f in srcs + [os.path.join(HERE, "sph_oracle.h")])
    if (not force and os.path.exists(out) and os.path.getmtime(out) >= newest):
        return out
    os.makedirs(BUILD, exist_ok=True)
    tmp = out + ".tmp%d" % os.getpid()
    flags = stock_flags() if stock else ["-O2", "-fno-fast-math", "-ffp-contract=off"]
    subprocess.run(["gcc", "-std=gnu11"] + flags + ["-fPIC", "-shared"] + srcs +
                   ["-o", tmp, "-lm"], check=True)
    os.replace(tmp, out)
    return out


_libs = {}


def lib(stock=False):
    if stock not in _libs:
        path = build(stock=stock)
        L = ctypes.CDLL(path)
        L.sph_oracle_run.restype = ctypes.c_int
        L.sph_oracle_exact64.restype = None
        _libs[stock] = L
    return _libs[stock]


def make_params(box, **kw):
    p = Params()
    d = box["dim"]
    p.dim[:] = list(d) if np.ndim(d) else [d, d, d]
    p.periodic = kw.get("periodic", 1)
    p.eta = kw.get("eta", box.get("eta", 1.2348))
    p.h_tolerance = kw.get("h_tolerance", 1e-4)
    p.h_max = kw.get("h_max", float(np.finfo(np.float32).max))
    p.h_min = kw.get("h_min", 0.0)
    p.alpha = kw.get("alpha", 0.8)
    p.max_iter = kw.get("max_iter", 30)
    p.max_active_bin = kw.get("max_active_bin", box.get("max_active_bin", 56))
    p.max_top_level_cells = kw.get("max_top_level_cells", 12)
    # 0, 0: one task per top cell / top-cell pair; else the reference's
    # Scheduler:cell_sub_size_self_hydro / cell_sub_size_pair_hydro split
    p.subsize_self = kw.get("subsize_self", 0)
    p.subsize_pair = kw.get("subsize_pair", 0)
    # 1: the same tasks in reverse order (a second legal task order)
    p.reverse_tasks = kw.get("reverse_tasks", 0)
    return p


def _ptr(a, t):
    return a.ctypes.data_as(ctypes.POINTER(t))


def run(box, stages=ALL, stock=False, **kw):
    """One density -> ghost -> force pass of the restated reference loops
    (stock=True: the build with the reference's optimisation flags, for
    timing only)."""
    L = lib(stock)
    n = box["x"].shape[0]
    x = np.ascontiguousarray(box["x"], np.float64)
    v = np.ascontiguousarray(box["v"], np.float32)
    m = np.ascontiguousarray(box["m"], np.float32)
    h = np.ascontiguousarray(box["h"], np.float32)
    u = np.ascontiguousarray(box["u"], np.float32)
    tb = np.ascontiguousarray(box["time_bin"], np.int8)
    fields = np.zeros((n, NFIELDS), np.float32)
    ints = np.zeros((n, NINTS), np.int32)
    res = Result()
    res.fields = _ptr(fields, ctypes.c_float)
    res.ints = _ptr(ints, ctypes.c_int32)
    prm = make_params(box, **kw)
    L.sph_oracle_run(ctypes.byref(prm), ctypes.c_int(n), _ptr(x, ctypes.c_double),
                     _ptr(v, ctypes.c_float), _ptr(m, ctypes.c_float),
                     _ptr(h, ctypes.c_float), _ptr(u, ctypes.c_float),
                     _ptr(tb, ctypes.c_byte), ctypes.c_int(stages),
                     ctypes.byref(res))
    out = {"res": fields, "ints": ints, "cdim": tuple(res.cdim),
           "ncells": res.ncells, "status": res.status, "ntasks": res.ntasks}
    for name, col in COLS.items():
        out[name] = fields[:, col]
    for name, col in INT_COLS.items():
        out[name] = ints[:, col]
    return out


def first_pass_tops(box, tops, **kw):
    """The first density pass of the tasks that touch the given top cells:
    the particles of those cells get their complete sums and neighbour
    counts (the bits of run()'s first pass); ``out["in_tops"]`` marks them."""
    L = lib()
    n = box["x"].shape[0]
    x = np.ascontiguousarray(box["x"], np.float64)
    v = np.ascontiguousarray(box["v"], np.float32)
    m = np.ascontiguousarray(box["m"], np.float32)
    h = np.ascontiguousarray(box["h"], np.float32)
    u = np.ascontiguousarray(box["u"], np.float32)
    tb = np.ascontiguousarray(box["time_bin"], np.int8)
    t = np.ascontiguousarray(tops, np.int32)
    fields = np.zeros((n, NFIELDS), np.float32)
    ints = np.zeros((n, NINTS), np.int32)
    res = Result()
    res.fields = _ptr(fields, ctypes.c_float)
    res.ints = _ptr(ints, ctypes.c_int32)
    prm = make_params(box, **kw)
    L.sph_oracle_first_pass_tops(ctypes.byref(prm), ctypes.c_int(n), _ptr(x, ctypes.c_double),
                                 _ptr(v, ctypes.c_float), _ptr(m, ctypes.c_float),
                                 _ptr(h, ctypes.c_float), _ptr(u, ctypes.c_float),
                                 _ptr(tb, ctypes.c_byte), ctypes.c_int(len(t)),
                                 _ptr(t, ctypes.c_int32), ctypes.byref(res))
    out = {"res": fields, "ints": ints, "cdim": tuple(res.cdim)}
    for name, col in COLS.items():
        out[name] = fields[:, col]
    for name, col in INT_COLS.items():
        out[name] = ints[:, col]
    out["in_tops"] = np.isin(out["top"], t)
    return out


def exact64(box, out, which=None):
    """FP64 sums (rho, wcount, div_v, a[3], u_dt) at the oracle's final h;
    with ``which`` (bool per particle) only for those particles (zeros
    elsewhere)."""
    L = lib()
    n = box["x"].shape[0]
    x = np.ascontiguousarray(box["x"], np.float64)
    v = np.ascontiguousarray(box["v"], np.float32)
    m = np.ascontiguousarray(box["m"], np.float32)
    arrs = [np.ascontiguousarray(out[k], np.float32)
            for k in ("h", "rho", "f", "pressure", "soundspeed", "balsara")]
    res = np.zeros((n, 7), np.float64)
    prm = make_params(box)
    if which is None:
        L.sph_oracle_exact64(ctypes.byref(prm), ctypes.c_int(n),
                             _ptr(x, ctypes.c_double), _ptr(v, ctypes.c_float),
                             _ptr(m, ctypes.c_float),
                             *[_ptr(a, ctypes.c_float) for a in arrs],
                             _ptr(res, ctypes.c_double))
    else:
        w = np.ascontiguousarray(which, np.uint8)
        L.sph_oracle_exact64_some(ctypes.byref(prm), ctypes.c_int(n),
                                  _ptr(x, ctypes.c_double), _ptr(v, ctypes.c_float),
                                  _ptr(m, ctypes.c_float),
                                  *[_ptr(a, ctypes.c_float) for a in arrs],
                                  _ptr(w, ctypes.c_ubyte), _ptr(res, ctypes.c_double))
    return res


def tree_sorts(box, **kw):
    """The restated reference sort arrays of every non-empty cell, depth
    first, as (first, count, depth, d[13][count+1], i[13][count+1])."""
    L = lib()
    n = box["x"].shape[0]
    arrs = [np.ascontiguousarray(box["x"], np.float64),
            np.ascontiguousarray(box["v"], np.float32),
            np.ascontiguousarray(box["m"], np.float32),
            np.ascontiguousarray(box["h"], np.float32),
            np.ascontiguousarray(box["u"], np.float32)]
    tb = np.ascontiguousarray(box["time_bin"], np.int8)
    types = [ctypes.c_double] + [ctypes.c_float] * 4
    ptrs = [_ptr(a, t) for a, t in zip(arrs, types)]
    prm = make_params(box, **kw)
    nc = ctypes.c_int32()
    ne = ctypes.c_int64()
    L.sph_oracle_tree_sorts(ctypes.byref(prm), ctypes.c_int(n), *ptrs, _ptr(tb, ctypes.c_byte),
                            ctypes.byref(nc), ctypes.byref(ne), None, None, None)
    rec = np.zeros((nc.value, 3), np.int32)
    d = np.zeros(ne.value, np.float32)
    idx = np.zeros(ne.value, np.int32)
    L.sph_oracle_tree_sorts(ctypes.byref(prm), ctypes.c_int(n), *ptrs, _ptr(tb, ctypes.c_byte),
                            ctypes.byref(nc), ctypes.byref(ne), _ptr(rec, ctypes.c_int32),
                            _ptr(d, ctypes.c_float), _ptr(idx, ctypes.c_int32))
    out, off = [], 0
    for first, count, depth in rec:
        k = 13 * (int(count) + 1)
        out.append((int(first), int(count), int(depth),
                    d[off:off + k].reshape(13, -1), idx[off:off + k].reshape(13, -1)))
        off += k
    return out
