"""Oracle vs the reference's own loops run here (oracle/_ref), on fresh
seeds: cell assignment, particle order and every density / ghost / force
output must be bit-identical.  Skipped where the reference build is absent
(machines without the reference tree)."""
import os
import tempfile

import numpy as np
import pytest

from swift_gb300 import ics

pytest.importorskip("numpy")
from oracle import io  # noqa: E402

HAVE_REF = os.path.exists(io.ref_harness_path("parity"))
pytestmark = pytest.mark.skipif(not HAVE_REF, reason="reference build (oracle/_ref) absent")

CASES = [
    ("lattice", 16, {"seed": 21}, {}),
    ("clustered", 20, {"seed": 22, "rms": 0.8}, {"max_top_level_cells": 3}),
    ("sedov", 20, {"seed": 23}, {"max_active_bin": 22}),
    # open (non-periodic) boxes, as the reference's test27cells / test125cells
    ("lattice", 16, {"seed": 24}, {"periodic": 0}),
    ("clustered", 20, {"seed": 25}, {"periodic": 0, "max_top_level_cells": 3}),
]


def special_box(kind):
    """Boxes that exercise the grid: a rectangular periodic box, particles
    exactly on the box faces (x == 0 and x == dim, which wraps), h clamped at
    h_min."""
    if kind == "rectangular":
        box = ics.lattice(16, seed=41)
        box["x"][:, 2] *= 0.5
        box["dim"] = (1.0, 1.0, 0.5)
        return box, {}
    if kind == "faces":
        box = ics.lattice(16, seed=42)
        box["x"][::97, 0] = 0.0
        box["x"][5::101, 1] = 1.0
        return box, {}
    if kind == "h_min":
        box = ics.clustered(20, seed=43, rms=0.8)
        return box, {"h_min": 0.07}
    raise ValueError(kind)


@pytest.mark.parametrize("kind", ["rectangular", "faces", "h_min"])
def test_special_boxes_bitwise(kind, oracle_lib):
    box, run = special_box(kind)
    ref = io.run_reference(box, tempfile.mkdtemp(), **run)
    orc = oracle_lib.run(box, **run)
    assert orc["status"] == 0
    for k in ("leaf_first", "leaf_count", "leaf_depth", "depth_h", "position", "top"):
        assert np.array_equal(ref[k], orc[k]), k
    for k in io.COLS:
        assert np.array_equal(ref[k].view(np.uint32), orc[k].view(np.uint32)), k
    if kind == "h_min":
        assert np.any(orc["h"] == np.float32(0.07))


def tiny(n, seed):
    """The first n particles of a 4^3 lattice: one top cell, few or no
    neighbours (h reaches h_max)."""
    box = ics.lattice(4, seed=seed)
    for k in ("x", "v", "m", "h", "u", "time_bin"):
        box[k] = box[k][:n].copy()
    return box


@pytest.mark.parametrize("n", [1, 2, 5, 17])
def test_tiny_open_boxes_bitwise(n, oracle_lib):
    box = tiny(n, seed=n)
    run = {"periodic": 0, "h_max": 0.6}
    ref = io.run_reference(box, tempfile.mkdtemp(), **run)
    orc = oracle_lib.run(box, **run)
    assert orc["status"] == 0
    for k in io.COLS:
        assert np.array_equal(ref[k].view(np.uint32), orc[k].view(np.uint32)), k
    if n == 1:
        assert orc["h"][0] == np.float32(0.6)  # no neighbour: h climbs to h_max


def test_lonely_particle_without_h_max_fails_like_the_reference(oracle_lib):
    """No neighbours and no h_max: the reference aborts after max_iter
    rounds (runner_ghost.c:1592); the oracle reports non-convergence."""
    import subprocess
    box = tiny(1, seed=1)
    with pytest.raises(subprocess.CalledProcessError):
        io.run_reference(box, tempfile.mkdtemp(), periodic=0)
    assert oracle_lib.run(box, periodic=0)["status"] == 1


@pytest.mark.parametrize("kind,n,gen,run", CASES)
def test_bitwise(kind, n, gen, run, oracle_lib):
    box = getattr(ics, kind)(n, **gen)
    ref = io.run_reference(box, tempfile.mkdtemp(), **run)
    orc = oracle_lib.run(box, **run)
    for k in ("leaf_first", "leaf_count", "leaf_depth", "depth_h", "position", "top"):
        assert np.array_equal(ref[k], orc[k]), k
    for k in io.COLS:
        assert np.array_equal(ref[k].view(np.uint32), orc[k].view(np.uint32)), k
