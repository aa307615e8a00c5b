"""Task splitting: the reference's scheduler splits the self and pair tasks
of big cells before a step (scheduler_splittask_hydro,
scheduler_splittasks.c:45-265) and links each piece to the cells it holds,
which the ghost's re-runs walk (runner_ghost.c:1548-1579).  The planner keeps
one task per top cell and top-cell pair instead.

A split happens only where the cell can split with the 1.10 leeway
(cell_can_split_*_hydro_task, cell.h:1152-1186), so the loops' own
recursion (cell_can_recurse_in_*_hydro_task, without the leeway) descends
there too: the same final cell pairs are evaluated in the same frames, and
only the order of the tasks -- the summation order of the sums -- changes.
These tests pin the oracle's restatement of the split against the reference
run with its own splitter, then show that splitting leaves every neighbour
count and cell assignment as it was and moves the sums by rounding only."""
import os
import tempfile

import numpy as np
import pytest

from swift_gb300 import ics

from oracle import io  # noqa: E402

HAVE_REF = os.path.exists(io.ref_harness_path("parity"))

# subsize_self 500 splits the self task of every splittable cell of >= 500
# particles; subsize_pair 256000000 is the reference's default (corner pairs
# split, others stay whole); 40000 also splits the face and edge pairs of
# the 512-particle top cells of a 24^3 lattice.
SPLIT = {"max_top_level_cells": 3, "subsize_self": 500, "subsize_pair": 256000000}
CASES = [("clustered:24", SPLIT),
         ("lattice:24", dict(SPLIT, subsize_pair=40000)),
         ("sedov:24", dict(SPLIT, max_active_bin=22))]

TREE = ("leaf_first", "leaf_count", "leaf_depth", "depth_h", "position", "top")


@pytest.mark.skipif(not HAVE_REF, reason="reference build (oracle/_ref) absent")
@pytest.mark.parametrize("cfg,run", CASES)
def test_split_tasks_bitwise_against_reference(cfg, run, oracle_lib):
    box = ics.make(cfg, seed=3)
    ref = io.run_reference(box, tempfile.mkdtemp(), **run)
    orc = oracle_lib.run(box, **run)
    assert orc["status"] == 0
    for k in TREE + ("ngb_first", "ngb_final", "ngb_force"):
        if k in ref:
            assert np.array_equal(ref[k], orc[k]), k
    for k in io.COLS:
        assert np.array_equal(ref[k].view(np.uint32), orc[k].view(np.uint32)), k


@pytest.mark.parametrize("cfg,run", CASES)
def test_split_changes_only_the_summation_order(cfg, run, oracle_lib):
    box = ics.make(cfg, seed=3)
    whole = {k: v for k, v in run.items() if not k.startswith("subsize")}
    a = oracle_lib.run(box, **whole)
    b = oracle_lib.run(box, **run)
    assert b["ntasks"] > a["ntasks"], (a["ntasks"], b["ntasks"])
    for k in TREE + ("ngb_first", "ngb_force", "min_ngb_bin"):
        assert np.array_equal(a[k], b[k]), k
    # first density pass: the same terms in another order
    for k in ("d_rho", "d_wcount"):
        assert np.max(np.abs(a[k] - b[k]) / np.abs(a[k]).max()) < 1e-5, k
    # the ghost stops anywhere inside its 1e-4 window around the root, so a
    # last-bit change of a sum can move h (and what follows it) by up to that
    # much on the few particles that end near the window's edge
    moved = a["ghost_iters"] != b["ghost_iters"]
    assert moved.mean() < 0.01
    assert np.max(np.abs(a["h"] - b["h"]) / a["h"]) < 2e-4
    same = ~moved
    assert np.max(np.abs(a["h"][same] - b["h"][same]) / a["h"][same]) < 1e-5
    assert np.mean(a["ngb_final"] == b["ngb_final"]) > 0.99
