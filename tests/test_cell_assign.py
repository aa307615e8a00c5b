"""Device-resident cell assignment (sphgpu_cell_assign): the rebuild's grid,
top cells, octree split and depth_h computed on the GPU from positions in
device memory, against the host build (sphgpu_space_create, bit-exact
against the reference's space_rebuild) -- the same cell records in the same
numbering, and for every particle the same leaf, depth_h and top cell."""
import ctypes

import numpy as np
import pytest

from swift_gb300 import api, ics

CASES = [("lattice:16", {}),
         ("clustered:24", {"max_top_level_cells": 3}),
         ("sedov:20", {}),
         ("clustered:20", {"max_top_level_cells": 3, "periodic": 0})]


def per_particle(order, depth_h, cells, n):
    """Leaf first / count / depth and depth_h per particle (caller's order)
    from the device outputs."""
    parent = cells[:, 3]
    split = np.zeros(len(cells), bool)
    split[parent[parent >= 0]] = True
    out = {k: np.full(n, -1, np.int64) for k in ("leaf_first", "leaf_count", "leaf_depth", "top")}
    for c in np.nonzero(~split & (cells[:, 1] > 0))[0]:
        first, count, depth, _, top = cells[c]
        idx = order[first:first + count]
        out["leaf_first"][idx] = first
        out["leaf_count"][idx] = count
        out["leaf_depth"][idx] = depth
        out["top"][idx] = top
    out["depth_h"] = np.empty(n, np.int64)
    out["depth_h"][order] = depth_h
    return out


def check_against_host(box, run):
    with api.Space(box, **run) as sp:
        tree = sp.tree()
        host = sp.cells()
        info = sp.info()
    order, dh, cells, cdim = api.cell_assign(box["x"], box["h"], box["dim"], **run)
    order = order.cpu().numpy()
    n = box["x"].shape[0]
    assert cdim == (info["cdim0"], info["cdim1"], info["cdim2"])
    assert np.array_equal(np.sort(order), np.arange(n))
    assert np.array_equal(cells, tree)
    dev = per_particle(order, dh.cpu().numpy(), cells, n)
    for k in ("leaf_first", "leaf_count", "leaf_depth", "depth_h", "top"):
        assert np.array_equal(dev[k], host[k]), k
    return cells


@pytest.mark.gpu
@pytest.mark.parametrize("cfg,run", CASES)
def test_device_tree_equals_host_tree(cfg, run):
    box = ics.make(cfg, seed=7)
    cells = check_against_host(box, run)
    if "clustered:24" in cfg:
        assert cells[:, 2].max() >= 1  # the split ran


@pytest.mark.gpu
def test_device_tree_deep_and_large():
    """A deeper tree (three top cells per side, clustered) and a 2.1M
    particle box."""
    box = ics.clustered(40, seed=9, rms=0.8)
    cells = check_against_host(box, {"max_top_level_cells": 3})
    assert cells[:, 2].max() >= 2
    check_against_host(ics.clustered(128, seed=1), {})


@pytest.mark.gpu
def test_device_tree_deeper_than_the_short_keys():
    """600 particles packed in a cube of side 1e-5 split down to depth ~15,
    below the levels the first (32-bit) keys hold: the call sorts again
    with 64-bit keys and still gives the host build's tree."""
    box = ics.lattice(12, seed=5)
    rng = np.random.default_rng(5)
    extra = 0.5 + 1e-5 * rng.random((600, 3))
    for k, v in (("x", extra), ("v", np.zeros((600, 3), np.float32)),
                 ("m", np.full(600, box["m"][0], np.float32)),
                 ("h", np.full(600, box["h"][0], np.float32)),
                 ("u", np.ones(600, np.float32)), ("time_bin", np.zeros(600, np.int8))):
        box[k] = np.concatenate([box[k], v.astype(box[k].dtype)])
    cells = check_against_host(box, {"max_top_level_cells": 3})
    assert cells[:, 2].max() >= 12


@pytest.mark.gpu
def test_device_tree_wraps_one_period():
    """Positions one box length outside a periodic box are wrapped back as
    the rebuild does; x itself is left alone."""
    import torch
    box = ics.clustered(24, seed=11)
    shifted = dict(box)
    x = box["x"].copy()
    x[::3, 0] += 1.0
    x[1::3, 1] -= 1.0
    shifted["x"] = x
    xd = torch.as_tensor(x, device="cuda")
    a = api.cell_assign(xd, box["h"], box["dim"])
    b = api.cell_assign(box["x"], box["h"], box["dim"])
    assert np.array_equal(a[2], b[2])
    assert np.array_equal(a[0].cpu().numpy(), b[0].cpu().numpy())
    assert np.array_equal(xd.cpu().numpy(), x)


@pytest.mark.gpu
@pytest.mark.parametrize("kind", ["nan", "outside_open", "h_zero", "two_periods"])
def test_device_tree_rejects_bad_input(kind):
    box = ics.lattice(12, seed=3)
    x, h, run = box["x"].copy(), box["h"].copy(), {}
    if kind == "nan":
        x[5, 1] = np.nan
    elif kind == "outside_open":
        x[7, 2] = 1.25
        run = {"periodic": 0}
    elif kind == "h_zero":
        h[9] = 0.0
    else:
        x[2, 0] = 2.5
    with pytest.raises(api.SphGpuError) as e:
        api.cell_assign(x, h, box["dim"], **run)
    assert e.value.code == api.EINVAL


def test_cell_assign_rejects_null_arguments():
    L = api.lib()
    p = api.Params()
    L.sphgpu_default_params(ctypes.byref(p))
    n = ctypes.c_int32()
    cdim = (ctypes.c_int32 * 3)()
    rc = L.sphgpu_cell_assign(ctypes.byref(p), None, None, 10, None, None, cdim,
                              ctypes.byref(n), None, 0, None)
    assert rc == api.EINVAL


def host_assignment(box, run):
    with api.Space(box, **run) as sp:
        cells = sp.cells()
        tree = sp.tree()
        info = sp.info()
    order = np.argsort(cells["position"]).astype(np.int32)
    return order, tree, cells, info


@pytest.mark.parametrize("cfg,run", CASES)
def test_space_adopts_an_assigned_tree(cfg, run):
    """sphgpu_space_create_assigned with the host build's own order and tree,
    and with the particles of every leaf reordered (as the device's
    assignment orders them): the same tree, leaves and plans."""
    box = ics.make(cfg, seed=7)
    order, tree, cells, info = host_assignment(box, run)
    rng = np.random.default_rng(1)
    shuffled = order.copy()
    parent = tree[:, 3]
    split = np.zeros(len(tree), bool)
    split[parent[parent >= 0]] = True
    for first, count in tree[~split & (tree[:, 1] > 0), :2]:
        shuffled[first:first + count] = rng.permutation(shuffled[first:first + count])
    for o in (order, shuffled):
        with api.Space(box, assigned=(o, tree), **run) as sp:
            assert np.array_equal(sp.tree(), tree)
            got = sp.cells()
            inf = sp.info()
        for k in ("leaf_first", "leaf_count", "leaf_depth", "depth_h", "top"):
            assert np.array_equal(got[k], cells[k]), k
        for k in ("cells", "leaves", "tasks", "entries"):
            assert inf[k] == info[k], k


def test_space_rejects_an_inconsistent_tree():
    box = ics.clustered(24, seed=7)
    run = {"max_top_level_cells": 3}
    order, tree, _, _ = host_assignment(box, run)
    bad = order.copy()
    bad[0] = bad[1]
    with pytest.raises(api.SphGpuError):
        api.Space(box, assigned=(bad, tree), **run)
    t2 = tree.copy()
    t2[-1, 0] = -5  # a child outside its parent
    with pytest.raises(api.SphGpuError):
        api.Space(box, assigned=(order, t2), **run)


def _leaves(tree):
    parent = tree[:, 3]
    split = np.zeros(len(tree), bool)
    split[parent[parent >= 0]] = True
    return np.nonzero(~split & (tree[:, 1] > 0))[0]


def test_space_rejects_bad_top_counts():
    """Top-cell counts that are negative, or that do not add up to the
    particle count, are refused before any cell is filled."""
    box = ics.clustered(24, seed=7)
    run = {"max_top_level_cells": 3}
    order, tree, _, _ = host_assignment(box, run)
    ntop = int(np.sum(tree[:, 3] < 0))
    for delta in (+1, -1):
        t2 = tree.copy()
        t2[0, 1] += delta                 # one top count too large / too small
        with pytest.raises(api.SphGpuError, match="top-cell count"):
            api.Space(box, assigned=(order, t2), **run)
    t2 = tree.copy()
    t2[0, 1] = -t2[0, 1]                  # negative
    with pytest.raises(api.SphGpuError, match="top-cell count"):
        api.Space(box, assigned=(order, t2), **run)
    assert ntop == 27


def test_space_rejects_a_particle_in_the_wrong_leaf():
    """Swapping two particles of different leaves (same top cell, so the
    order stays a permutation and the counts stay right) puts each outside
    its octant: refused.  Swapping across top cells is refused too."""
    box = ics.clustered(24, seed=7)
    run = {"max_top_level_cells": 3}
    order, tree, _, _ = host_assignment(box, run)
    leaves = _leaves(tree)
    # two leaves of the same top cell with different parents' octants
    by_top = {}
    for c in leaves:
        by_top.setdefault(int(tree[c, 4]), []).append(int(c))
    top, ls = next((t, v) for t, v in by_top.items() if len(v) >= 2)
    a, b = ls[0], ls[-1]
    bad = order.copy()
    i, j = int(tree[a, 0]), int(tree[b, 0])
    bad[i], bad[j] = bad[j], bad[i]
    with pytest.raises(api.SphGpuError, match="octant|top cell"):
        api.Space(box, assigned=(bad, tree), **run)
    # across top cells
    tops = np.nonzero((tree[:, 3] < 0) & (tree[:, 1] > 0))[0]
    bad = order.copy()
    i, j = int(tree[tops[0], 0]), int(tree[tops[1], 0])
    bad[i], bad[j] = bad[j], bad[i]
    with pytest.raises(api.SphGpuError, match="top cell"):
        api.Space(box, assigned=(bad, tree), **run)


def test_space_rejects_children_that_do_not_tile_their_parent():
    """A child range shortened by one particle leaves a gap in its parent."""
    box = ics.clustered(24, seed=7)
    run = {"max_top_level_cells": 3}
    order, tree, _, _ = host_assignment(box, run)
    kids = np.nonzero((tree[:, 3] >= 0) & (tree[:, 1] > 1))[0]
    t2 = tree.copy()
    t2[kids[0], 1] -= 1
    with pytest.raises(api.SphGpuError, match="tile"):
        api.Space(box, assigned=(order, t2), **run)


@pytest.mark.gpu
def test_space_from_device_assignment_matches_host_space():
    """The whole pass on a space built from the device's cell assignment:
    the same neighbour counts as the host-built space, sums within rounding
    (only the order inside leaves differs)."""
    box = ics.clustered(32, seed=3)
    order, dh, cells, cdim = api.cell_assign(box["x"], box["h"], box["dim"])
    with api.Space(box) as sp:
        sp.step(api.STAGE_DENSITY)
        a = sp.download()
    with api.Space(box, assigned=(order, cells)) as sp:
        sp.step(api.STAGE_DENSITY)
        b = sp.download()
    assert np.array_equal(a["ngb_first"], b["ngb_first"])
    for k in ("d_rho", "d_wcount"):
        assert np.max(np.abs(a[k] - b[k]) / np.abs(a[k])) < 1e-5, k
