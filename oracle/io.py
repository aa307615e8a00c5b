"""Binary I/O between the oracle's Python side and its C programs.

Test infrastructure only.  ``write_input`` produces the "SPHIN002" file read by
oracle/ref_harness.c (the driver of the reference's own loops) and by the C
restatement in oracle/sph_oracle.c; ``read_output`` parses "SPHOUT01".
"""
from __future__ import annotations

import os
import subprocess

import numpy as np

STAGE_DENSITY, STAGE_GHOST, STAGE_FORCE = 1, 2, 4
ALL_STAGES = STAGE_DENSITY | STAGE_GHOST | STAGE_FORCE

# Field columns of the per-particle result block (24 floats per particle).
COLS = {
    "d_rho": 0, "d_rho_dh": 1, "d_wcount": 2, "d_wcount_dh": 3, "d_div_v": 4,
    "d_rot_vx": 5, "d_rot_vy": 6, "d_rot_vz": 7,
    "h": 8, "rho": 9, "f": 10, "pressure": 11, "soundspeed": 12,
    "balsara": 13, "v_sig_ghost": 14,
    "ax": 15, "ay": 16, "az": 17, "u_dt": 18, "h_dt": 19, "v_sig": 20,
}

CELL_DTYPE = np.dtype([
    ("loc", "<f8", 3), ("width", "<f8", 3), ("h_max", "<f4"),
    ("h_max_active", "<f4"), ("dmin", "<f4"), ("depth", "<i4"),
    ("split", "<i4"), ("count", "<i4"), ("first", "<i4"), ("parent", "<i4"),
    ("top", "<i4"), ("_pad", "<i4"),
])
assert CELL_DTYPE.itemsize == 88

HEADER_DTYPE = np.dtype([
    ("magic", "S8"), ("n", "<i8"), ("dim", "<f8", 3), ("eta", "<f4"),
    ("h_tolerance", "<f4"), ("h_max", "<f4"), ("h_min", "<f4"),
    ("alpha", "<f4"), ("max_iter", "<i4"), ("max_active_bin", "<i4"),
    ("periodic", "<i4"), ("stages", "<i4"), ("max_top_level_cells", "<i4"),
    ("subsize_self", "<i4"), ("subsize_pair", "<i4"),
])
assert HEADER_DTYPE.itemsize == 88


def default_params(box):
    return dict(eta=box.get("eta", 1.2348), h_tolerance=1e-4,
                h_max=np.finfo(np.float32).max, h_min=0.0, alpha=0.8,
                max_iter=30, max_active_bin=box.get("max_active_bin", 56),
                periodic=1, max_top_level_cells=12, subsize_self=0, subsize_pair=0)


def write_input(path, box, stages=ALL_STAGES, **overrides):
    p = default_params(box)
    p.update(overrides)
    n = box["x"].shape[0]
    hdr = np.zeros(1, HEADER_DTYPE)
    hdr["magic"] = b"SPHIN002"
    hdr["n"] = n
    hdr["dim"] = list(box["dim"]) if np.ndim(box["dim"]) else [box["dim"]] * 3
    for k in ("eta", "h_tolerance", "h_max", "h_min", "alpha", "max_iter",
              "max_active_bin", "periodic", "max_top_level_cells", "subsize_self",
              "subsize_pair"):
        hdr[k] = p[k]
    hdr["stages"] = stages
    with open(path, "wb") as f:
        f.write(hdr.tobytes())
        f.write(np.ascontiguousarray(box["x"], np.float64).tobytes())
        f.write(np.ascontiguousarray(box["v"], np.float32).tobytes())
        for k in ("m", "h", "u"):
            f.write(np.ascontiguousarray(box[k], np.float32).tobytes())
        f.write(np.ascontiguousarray(box["time_bin"], np.int8).tobytes())


INT_COLS = {"leaf_first": 0, "leaf_count": 1, "leaf_depth": 2, "depth_h": 3,
            "position": 4, "top": 5, "ngb_first": 6, "ngb_final": 7,
            "ngb_force": 8, "ghost_iters": 9, "min_ngb_bin": 10}


def read_output(path):
    with open(path, "rb") as f:
        buf = f.read()
    assert buf[:8] == b"SPHOUT01", "bad oracle output magic"
    off = 8
    n, nf, ncell, c0, c1, c2, ni = np.frombuffer(buf, "<i8", 7, off)
    off += 56
    width = np.frombuffer(buf, "<f8", 3, off)
    off += 24
    res = np.frombuffer(buf, "<f4", n * nf, off).reshape(n, nf)
    off += 4 * n * nf
    ints = np.frombuffer(buf, "<i4", ni * n, off).reshape(n, ni)
    off += 4 * ni * n
    cells = np.frombuffer(buf, CELL_DTYPE, ncell, off)
    out = {"res": res, "ints": ints, "cells": cells,
           "cdim": (int(c0), int(c1), int(c2)), "width": width.copy()}
    for name, col in COLS.items():
        out[name] = res[:, col]
    for name, col in INT_COLS.items():
        if col < ni and not np.all(ints[:, col] == -1):  # -1: not kept
            out[name] = ints[:, col]
    return out


def ref_harness_path(mode="parity"):
    here = os.path.dirname(os.path.abspath(__file__))
    return os.path.join(here, "_ref", mode, "bin", "ref_harness")


def read_sorts(path):
    """Sort arrays written by the harness: a list of (first, count, depth,
    d[13][count+1] float32, i[13][count+1] int32), cells depth first."""
    out = []
    with open(path, "rb") as f:
        if f.read(8) != b"SPHSRT01":
            raise ValueError("not a sort dump")
        while True:
            rec = f.read(12)
            if len(rec) < 12:
                break
            first, count, depth = np.frombuffer(rec, np.int32)
            ent = np.frombuffer(f.read(13 * (int(count) + 1) * 8), dtype=[("d", "<f4"), ("i", "<i4")])
            ent = ent.reshape(13, int(count) + 1)
            out.append((int(first), int(count), int(depth),
                        np.ascontiguousarray(ent["d"]), np.ascontiguousarray(ent["i"])))
    return out


def run_reference(box, workdir, stages=ALL_STAGES, mode="parity", sorts=False,
                  **overrides):
    """Run the reference's own loops (oracle/_ref) on ``box``; with
    ``sorts`` also return the reference's sort arrays (key "sorts")."""
    exe = ref_harness_path(mode)
    for k in ("max_active_bin",):
        if k in box and k not in overrides:
            overrides[k] = box[k]
    if not os.path.exists(exe):
        raise FileNotFoundError(f"reference harness not built: {exe}")
    inp = os.path.join(workdir, "ref_in.bin")
    out = os.path.join(workdir, "ref_out.bin")
    write_input(inp, box, stages, **overrides)
    args = [exe, inp, out]
    if sorts:
        args.append(os.path.join(workdir, "ref_sorts.bin"))
    subprocess.run(args, check=True, capture_output=True)
    res = read_output(out)
    if sorts:
        res["sorts"] = read_sorts(args[3])
    return res
