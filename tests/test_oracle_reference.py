"""Oracle vs the reference's own loops run here (oracle/_ref), on fresh
seeds: cell assignment, particle order and every density / ghost / force
output must be bit-identical.  Skipped where the reference build is absent
(the GPU hosts carry no reference tree)."""
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
]


@pytest.mark.parametrize("kind,n,gen,run", CASES)
def test_bitwise(kind, n, gen, run, oracle_lib):
    box = getattr(ics, kind)(n, **gen)
    ref = io.run_reference(box, tempfile.mkdtemp(), **run)
    orc = oracle_lib.run(box, **run)
    for k in ("leaf_first", "leaf_count", "leaf_depth", "depth_h", "position", "top"):
        assert np.array_equal(ref[k], orc[k]), k
    for k in io.COLS:
        assert np.array_equal(ref[k].view(np.uint32), orc[k].view(np.uint32)), k
