"""The density gathers' tensor-core candidate filter (tuning tc_filter):
TF32 r^2 for 16 particles x 8 candidates per mma.sync, with a margin that
drops no candidate the FP32 test would keep, then the exact classification
of the candidates that pass.  The neighbour sets must be those of the FP32
test of every candidate, and the oracle's."""
import numpy as np
import pytest

from swift_gb300 import api, ics

pytestmark = pytest.mark.gpu


def rel_err(a, b, floor_frac=1e-3):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    scale = np.maximum(np.abs(b), floor_frac * np.max(np.abs(b)) + 1e-30)
    return np.abs(a - b) / scale


def scaled_err(a, b):
    """|a - b| relative to the field's scale (max |b|)."""
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return np.abs(a - b) / (np.max(np.abs(b)) + 1e-30)


def run(box, tc, stages=api.STAGE_ALL, **tun):
    with api.Space(box) as sp:
        sp.set_tuning(tc_filter=tc, **tun)
        sp.step(stages)
        sp.step(stages)    # graph replay
        return sp.download()


@pytest.mark.parametrize("tpp,jtile", [(1, 32), (2, 32), (1, 16), (2, 8)])
@pytest.mark.parametrize("spec", ["clustered:40", "lattice:32"])
def test_filter_keeps_the_neighbour_sets(spec, tpp, jtile):
    """Identical first-pass counts and rows' effect; the rest of the step
    within FP32 summation-order noise (a band hit may trade places with a
    plain hit inside an 8-candidate batch)."""
    box = ics.make(spec, seed=9)
    tun = dict(tpp=tpp, jtile=jtile, rerun_lists=1, block_warps=8)
    # the first density pass alone: the same neighbours, the same terms (in
    # the same order but for band hits; the frame offset of a hit is its
    # entry's, bit-close to the table's the FP32 path uses)
    a, b = (run(box, tc, api.STAGE_DENSITY, **tun) for tc in (1, 0))
    assert np.array_equal(a["ngb_first"], b["ngb_first"])
    for k in ("d_rho", "d_wcount"):
        assert rel_err(a[k], b[k]).max() < 1e-5, k
    # sums whose terms cancel: against the field's scale
    for k in ("d_rho_dh", "d_wcount_dh", "d_div_v", "d_rot_vx", "d_rot_vy", "d_rot_vz"):
        assert scaled_err(a[k], b[k]).max() < 1e-5, k
    # the whole step: Newton may stop a round earlier or later inside the
    # ghost's tolerance window
    a, b = run(box, 1, **tun), run(box, 0, **tun)
    assert np.array_equal(a["ngb_first"], b["ngb_first"])
    assert np.mean(a["ngb_final"] == b["ngb_final"]) > 0.999
    assert np.mean(a["ngb_force"] == b["ngb_force"]) > 0.999
    assert rel_err(a["h"], b["h"]).max() < 2e-4
    for k in ("rho", "pressure", "soundspeed"):
        assert rel_err(a[k], b[k]).max() < 3e-4, k


def test_filter_matches_the_oracle(oracle_lib):
    """First-pass neighbour counts equal the oracle's (the reference's loops
    restated), with one and two lanes per particle, without rows too."""
    box = ics.make("clustered:32", seed=21)
    ref = oracle_lib.run(box)
    for tpp, lists in ((1, 1), (2, 1), (1, 0), (2, 0)):
        g = run(box, 1, tpp=tpp, jtile=32, rerun_lists=lists, block_warps=8)
        assert np.array_equal(g["ngb_first"], ref["ngb_first"]), (tpp, lists)
        assert np.mean(g["ngb_final"] == ref["ngb_final"]) > 0.999, (tpp, lists)
        assert rel_err(g["h"], ref["h"]).max() < 2e-4, (tpp, lists)


def test_filter_with_strongly_uneven_h():
    """h set 40 % too small on a third of the particles and 60 % too large on
    another third: wide and narrow thresholds in one group (the margin is
    the group's), the catch-up gathers filtered too."""
    box = ics.make("clustered:24", seed=17)
    h = box["h"].copy()
    h[::3] *= np.float32(0.6)
    h[1::3] *= np.float32(1.6)
    box["h"] = h
    tun = dict(tpp=1, jtile=32, rerun_lists=1, block_warps=8)
    a, b = run(box, 1, **tun), run(box, 0, **tun)
    assert np.array_equal(a["ngb_first"], b["ngb_first"])
    assert np.mean(a["ngb_final"] == b["ngb_final"]) > 0.999
    assert rel_err(a["h"], b["h"]).max() < 2e-4
    assert rel_err(a["rho"], b["rho"]).max() < 3e-4
