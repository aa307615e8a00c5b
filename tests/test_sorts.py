"""Per-cell sort arrays (runner_do_hydro_sort, runner_sort.c:203): the
oracle's against the reference's own arrays (golden digests and, where the
reference is built here, directly), and the device sort against both, bit
for bit -- keys, indices and the order of ties."""
import ast
import glob
import os
import sys

import numpy as np
import pytest

from swift_gb300 import ics

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
sys.path.insert(0, GOLDEN)
from make_golden import sort_table  # noqa: E402

SORT_FIXTURES = sorted(glob.glob(os.path.join(GOLDEN, "sorts_*.npz")))
# boxes that every host regenerates bit for bit (seeded lattices; the
# clustered generator's FFT differs in the last bits between numpy builds)
PORTABLE = [p for p in SORT_FIXTURES if "lattice" in os.path.basename(p)]


def load(path):
    g = np.load(path)
    box = getattr(ics, str(g["kind"]))(int(g["n"]), **ast.literal_eval(str(g["gen_kwargs"])))
    return g, box, ast.literal_eval(str(g["run_kwargs"]))


@pytest.mark.parametrize("path", SORT_FIXTURES, ids=[os.path.basename(p)[:-4] for p in SORT_FIXTURES])
def test_oracle_sorts_match_reference_golden(path, oracle_lib):
    g, box, run = load(path)
    rec, dig = sort_table(oracle_lib.tree_sorts(box, **run))
    assert np.array_equal(rec, g["records"])
    assert np.array_equal(dig, g["digests"])


def test_sort_fixtures_present():
    names = {os.path.basename(p) for p in SORT_FIXTURES}
    assert {"sorts_clustered32_deep.npz", "sorts_lattice20.npz",
            "sorts_lattice48_deep.npz"} <= names
    deep = np.load(os.path.join(GOLDEN, "sorts_lattice48_deep.npz"))["records"]
    assert deep[:, 2].max() >= 2  # merges over two levels


def test_oracle_sorts_match_reference_directly(oracle_lib, tmp_path):
    from oracle import io
    if not os.path.exists(io.ref_harness_path("parity")):
        pytest.skip("reference harness not built here")
    box = ics.clustered(24, seed=4)
    ref = io.run_reference(box, str(tmp_path), stages=1, sorts=True, max_top_level_cells=3)
    ours = oracle_lib.tree_sorts(box, max_top_level_cells=3)
    assert len(ours) == len(ref["sorts"])
    for a, b in zip(ours, ref["sorts"]):
        assert a[:3] == b[:3]
        assert np.array_equal(a[3].view(np.uint32), b[3].view(np.uint32))
        assert np.array_equal(a[4], b[4])


def _gpu_sorts(box, run):
    from swift_gb300 import api
    with api.Space(box, **run) as sp:
        sp.hydro_sort(0x1FFF)
        tree = sp.tree()
        out = {}
        for c, (first, count, depth, _, _) in enumerate(tree):
            if count == 0:
                continue
            ds, ids = [], []
            for j in range(13):
                d, i = sp.cell_sort(c, j, int(count))
                ds.append(d)
                ids.append(i)
            out[(int(first), int(depth))] = (int(first), int(count), int(depth),
                                             np.stack(ds), np.stack(ids))
    return out


@pytest.mark.gpu
@pytest.mark.parametrize("path", PORTABLE, ids=[os.path.basename(p)[:-4] for p in PORTABLE])
def test_gpu_sorts_match_reference_golden(path):
    g, box, run = load(path)
    gpu = _gpu_sorts(box, run)
    order = [gpu[(int(f), int(d))] for f, _, d in g["records"]]
    rec, dig = sort_table(order)
    assert np.array_equal(rec, g["records"])
    assert np.array_equal(dig, g["digests"])


@pytest.mark.gpu
@pytest.mark.parametrize("cfg,run", [("lattice:16", {}),
                                     ("clustered:24", {"max_top_level_cells": 3}),
                                     ("clustered:40", {}),
                                     # top cells of ~9,700 particles: arrays longer
                                     # than a block's shared memory
                                     ("clustered:64", {"max_top_level_cells": 3})])
def test_gpu_sorts_match_oracle(cfg, run, oracle_lib):
    box = ics.make(cfg, seed=12)
    ours = oracle_lib.tree_sorts(box, **run)
    gpu = _gpu_sorts(box, run)
    assert len(gpu) == len(ours)
    for first, count, depth, d, i in ours:
        g = gpu[(first, depth)]
        assert g[1] == count
        assert np.array_equal(g[3].view(np.uint32), d.view(np.uint32)), (first, depth)
        assert np.array_equal(g[4], i), (first, depth)
