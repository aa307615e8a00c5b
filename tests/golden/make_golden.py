"""Generate the golden fixtures of this directory from the reference's own
loops (oracle/_ref/parity/bin/ref_harness: the reference's space build, sorts,
density loops, ghost and force loops, compiled from the reference tree by
oracle/build_ref.sh with -O2 -fno-fast-math -ffp-contract=off).

Each fixture stores the generator recipe (kind, size, seed, parameters), the
full-box sums of every output field (float64 sums of the float32 values) and
the complete outputs of a seeded sample of particles.  Inputs are
regenerated by swift_gb300.ics from the recipe, so the fixtures stay small.

Run on a machine that has the reference tree (oracle/build_ref.sh builds it):
    python tests/golden/make_golden.py
"""
import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import io  # noqa: E402
from swift_gb300 import ics  # noqa: E402

CASES = [
    # name, generator kind, n, generator kwargs, run parameters, sample size
    ("lattice12", "lattice", 12, {"seed": 3}, {}, 0),
    ("plain32", "lattice", 32, {"seed": 1}, {}, 1024),
    ("clustered24_split", "clustered", 24, {"seed": 4}, {"max_top_level_cells": 3}, 1024),
    ("clustered32_deep", "clustered", 32, {"seed": 9, "rms": 1.5},
     {"max_top_level_cells": 3}, 1024),
    # sparse activity: density and ghost only -- the force loop reads the
    # force state of inactive neighbours, which a single pass from initial
    # conditions does not have
    ("sedov24_sparse", "sedov", 24, {"seed": 2}, {"max_active_bin": 21, "stages": 3},
     1024),
    # an open (non-periodic) box, as the reference's cell tests use
    ("lattice16_open", "lattice", 16, {"seed": 24}, {"periodic": 0}, 1024),
    # two steps: every particle active, then the 2% in bins 20-22 on the
    # state the first step leaves (inactive neighbours carry their density
    # and force state into the second step's loops)
    ("sedov24_primed", "sedov", 24, {"seed": 2}, {"max_active_bin": 22, "stages": 15},
     1024),
]

INT_NAMES = ["leaf_first", "leaf_count", "leaf_depth", "depth_h", "position", "top"]

# sort arrays of runner_do_hydro_sort, as per-(cell, axis) digests
# (the clustered generator's FFT is not bit-reproducible across numpy builds
# and CPUs, so only the lattice boxes are regenerated bit for bit on another
# host; the clustered fixture pins the oracle where it was made)
SORT_CASES = [
    # name, generator kind, n, generator kwargs, run parameters
    ("sorts_clustered32_deep", "clustered", 32, {"seed": 9, "rms": 1.5},
     {"max_top_level_cells": 3}),
    ("sorts_lattice20", "lattice", 20, {"seed": 5}, {}),
    ("sorts_lattice48_deep", "lattice", 48, {"seed": 6}, {"max_top_level_cells": 3}),
]


def sort_digest(d, i):
    """8-byte digest of one cell's 13 sort arrays (key bits and indices)."""
    import hashlib
    h = hashlib.blake2b(digest_size=8)
    h.update(np.ascontiguousarray(d, np.float32).tobytes())
    h.update(np.ascontiguousarray(i, np.int32).tobytes())
    return np.frombuffer(h.digest(), np.uint64)[0]


def sort_table(sorts):
    """(records [cells][3] = first, count, depth; digests [cells])."""
    rec = np.array([s[:3] for s in sorts], np.int32).reshape(-1, 3)
    dig = np.array([sort_digest(s[3], s[4]) for s in sorts], np.uint64)
    return rec, dig


def mask_fields(fields, box, run):
    """Zero the first-pass density columns (0-7) of the particles that the
    second step of a primed run leaves inactive: the reference keeps the
    density accumulators in a union with the force state
    (hydro/Minimal/hydro_part.h:135-192), so after a step those columns of an
    inactive particle hold force values, not density sums."""
    if run.get("stages", 7) & 8:
        inactive = box["time_bin"] > run["max_active_bin"]
        fields = fields.copy()
        fields[inactive, :8] = 0.0
    return fields


def make_box(kind, n, kw):
    return getattr(ics, kind)(n, **kw)


def main(only=None):
    for name, kind, n, kw, run, nsample in CASES:
        if only and name not in only:
            continue
        box = make_box(kind, n, kw)
        ref = io.run_reference(box, tempfile.mkdtemp(), **run)
        N = box["x"].shape[0]
        fields = mask_fields(ref["res"][:, :21].astype(np.float32), box, run)
        ints = np.stack([ref[k] for k in INT_NAMES], axis=1).astype(np.int32)
        if nsample and nsample < N:
            idx = np.sort(np.random.default_rng(12345).choice(N, nsample, replace=False))
        else:
            idx = np.arange(N)
        np.savez_compressed(
            os.path.join(HERE, name + ".npz"),
            kind=kind, n=n, gen_kwargs=repr(kw), run_kwargs=repr(run),
            cdim=np.array(ref["cdim"]), sample=idx.astype(np.int32),
            fields=fields[idx], ints=ints[idx],
            field_sums=fields.astype(np.float64).sum(axis=0),
            int_sums=ints.astype(np.int64).sum(axis=0))
        print(name, N, "particles, cdim", ref["cdim"], "->", name + ".npz")
    for name, kind, n, kw, run in SORT_CASES:
        if only and name not in only:
            continue
        box = make_box(kind, n, kw)
        ref = io.run_reference(box, tempfile.mkdtemp(), stages=1, sorts=True, **run)
        rec, dig = sort_table(ref["sorts"])
        np.savez_compressed(os.path.join(HERE, name + ".npz"), kind=kind, n=n,
                            gen_kwargs=repr(kw), run_kwargs=repr(run), records=rec,
                            digests=dig)
        print(name, len(rec), "cells ->", name + ".npz")


if __name__ == "__main__":
    main(sys.argv[1:])
