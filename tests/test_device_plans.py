"""Device planning of sparse steps (swift_gb300/csrc/devplan.cu).

After a sparse activation of a resident space, every batched step plans its
own gather lists on the device: the flags from the time bins, each cell's
h_max / h_max_active / activity from its particles, the density and re-run
lists through the reference's recursions (runner_doiact_functions_hydro.h
DOSUB_SELF1/PAIR1 and the ghost's DOSUB_SUBSET), and after the ghost the
force lists from the post-ghost h_max (DOSUB_SELF2/PAIR2,
runner_ghost.c:1617-1632).  The lists must equal the host planner's for the
same state, leaf by leaf and entry by entry, so that steps planned either way
give bit-identical results; the host planner takes over from the device's
state for the plain form.
"""
import numpy as np
import pytest

from swift_gb300 import api, ics

pytestmark = pytest.mark.gpu


def _box(cfg, seed):
    box = ics.make(cfg, seed=seed)
    if not cfg.startswith("sedov"):
        n = box["x"].shape[0]
        box["time_bin"][:] = 20 + (np.arange(n) * 7919) % 4
    return box


def _sparse_bins(box, seq):
    top = int(box["time_bin"].max())
    return [b for b in seq if b < top]


@pytest.mark.parametrize("cfg", ["sedov:24", "sedov:32", "clustered:24", "lattice:16"])
def test_device_plans_equal_host_plans(cfg):
    box = _box(cfg, 5)
    with api.Space(box) as sp:
        sp.set_active(api.ALL_ACTIVE)
        sp.step()
        for b in _sparse_bins(box, (22, 20, 23, 21, 22, 20)):
            sp.set_active(b)
            sp.step()
            chk = sp.check_device_plans()
            assert all(bad == 0 for bad, _ in chk.values()), (cfg, b, chk)
            assert chk["density"][1] > 0 and chk["force"][1] > 0, (cfg, b, chk)
        ms, steps = sp.plan_times()
        assert steps > 0 and ms > 0


def _run(box, device, seq, plain_last=None):
    with api.Space(box) as sp:
        sp.set_device_planning(device)
        sp.set_active(api.ALL_ACTIVE)
        sp.step()
        sp.step_stats(reset=True)
        for b in seq:
            sp.set_active(b)
            sp.step()
        if plain_last is not None:
            sp.set_active(plain_last)
            sp.step_plain()
        return sp.download(), sp.step_stats()


@pytest.mark.parametrize("cfg", ["sedov:32", "clustered:24"])
def test_device_planned_steps_equal_host_planned_steps(cfg):
    box = _box(cfg, 7)
    seq = _sparse_bins(box, (22, 20, 23, 21, 22))
    a, sa = _run(box, True, seq)
    b, sb = _run(box, False, seq)
    # device planning: every sparse step one graph, one capture
    assert sa["graph_steps"] == len(seq) and sa["captures"] == 1, sa
    for k in a:
        assert np.array_equal(a[k], b[k], equal_nan=True), (cfg, k)


def test_plain_step_after_device_planned_steps():
    """The host planner takes over from the device's state: a plain step
    after device-planned steps equals the same plain step after
    host-planned ones."""
    box = _box("sedov:24", 9)
    seq = (22, 20, 21)
    a, _ = _run(box, True, seq, plain_last=22)
    b, _ = _run(box, False, seq, plain_last=22)
    for k in a:
        assert np.array_equal(a[k], b[k], equal_nan=True), k


def test_plan_buffers_grow_when_a_step_needs_more():
    """Device planning entered after a small activation sizes its buffers
    from that activation's lists; a step whose active region (the Sedov
    box's inner 7% instead of its 1% core) is several times larger outgrows
    them, grows them and runs again outside the graph, with the results of a
    host-planned step."""
    box = _box("sedov:48", 11)

    def run(device):
        with api.Space(box) as sp:
            # host-planned (the space is not resident yet): small lists and
            # plan buffers; the particles outside the core have no density
            # yet, so some forces read zero densities (NaN h_dt in both runs)
            sp.set_device_planning(device)
            sp.set_active(20)
            sp.step()
            sp.step_stats(reset=True)
            sp.set_active(26)
            sp.step()
            chk = sp.check_device_plans() if device else None
            return sp.download(), sp.step_stats(), chk

    a, st, chk = run(True)
    b, _, _ = run(False)
    assert st["force_replans"] == 1, st
    assert all(bad == 0 for bad, _ in chk.values()), chk
    for k in a:
        assert np.array_equal(a[k], b[k], equal_nan=True), k
