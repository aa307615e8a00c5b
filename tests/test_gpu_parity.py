"""GPU parity: the sm_103a path against the oracle (oracle/sph_oracle.c,
itself bit-identical to the reference's loops), through the C ABI.

Tolerances: neighbour counts and cell assignment are compared exactly.
Positive sums (rho, wcount, P, c, v_sig) are compared at 1e-4 relative per
particle.  Signed sums whose terms cancel (rho_dh, wcount_dh, div_v, rot_v,
a, du/dt, dh/dt) are compared at 1e-4 of the field's scale (its largest
magnitude in the box): their per-particle value is a residual of cancelling
terms, so only an absolute tolerance is meaningful -- the same convention as
the absolute-tolerance row of the reference's tests/difffloat.py.
h is compared within the ghost's own tolerance: two runs that converge
independently may each stop anywhere inside the 1e-4 window around the root
(runner_ghost.c:1388), so they differ by up to 2e-4; quantities downstream
of h in a full pass are then compared at 1e-3 of their scale, while the
force loop fed with the oracle's own post-ghost state is held to 1e-4.
"""
import numpy as np
import pytest

from swift_gb300 import api, ics

pytestmark = pytest.mark.gpu

REL = 1e-4


def scaled_err(a, b):
    """|a - b| relative to the field's scale (max |b|)."""
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return np.abs(a - b) / (np.max(np.abs(b)) + 1e-30)


def rel_err(a, b, floor_frac=1e-3):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    scale = np.maximum(np.abs(b), floor_frac * np.max(np.abs(b)) + 1e-30)
    return np.abs(a - b) / scale


@pytest.fixture(scope="module", params=["lattice:16", "lattice:32", "clustered:40"])
def case(request, oracle_lib):
    box = ics.make(request.param, seed=5)
    ref = oracle_lib.run(box)
    return request.param, box, ref


def test_first_density_pass_counts_exact(case):
    name, box, ref = case
    with api.Space(box) as sp:
        sp.step(api.STAGE_DENSITY)
        out = sp.download()
    assert np.array_equal(out["ngb_first"], ref["ngb_first"]), name
    for k in ("d_rho", "d_wcount"):
        assert rel_err(out[k], ref[k]).max() < REL, (name, k)
    for k in ("d_rho_dh", "d_wcount_dh", "d_div_v", "d_rot_vx", "d_rot_vy",
              "d_rot_vz"):
        assert scaled_err(out[k], ref[k]).max() < REL, (name, k)


def test_full_pass_matches_oracle(case):
    name, box, ref = case
    with api.Space(box) as sp:
        sp.step(api.STAGE_ALL)
        out = sp.download()
    assert rel_err(out["h"], ref["h"]).max() < 2e-4, name
    for k in ("rho", "pressure", "soundspeed", "v_sig"):
        assert rel_err(out[k], ref[k]).max() < 3e-4, (name, k)
    for k in ("ax", "ay", "az", "u_dt", "h_dt", "f", "balsara"):
        assert scaled_err(out[k], ref[k]).max() < 1e-3, (name, k)
    # neighbour counts after independent ghosts agree except where h differs
    # inside the tolerance window
    assert np.mean(out["ngb_final"] == ref["ngb_final"]) > 0.99, name


def test_force_counts_exact_from_oracle_state(case):
    name, box, ref = case
    with api.Space(box) as sp:
        sp.step(api.STAGE_ALL)
        sp.force_from_state(ref["h"], ref["rho"], ref["f"], ref["pressure"],
                            ref["soundspeed"], ref["balsara"])
        out = sp.download()
    assert np.array_equal(out["ngb_force"], ref["ngb_force"]), name
    for k in ("ax", "ay", "az", "u_dt", "h_dt"):
        assert scaled_err(out[k], ref[k]).max() < REL, (name, k)
    assert rel_err(out["v_sig"], ref["v_sig"]).max() < 1e-6, name


def test_plain_equals_batched(case):
    name, box, ref = case
    with api.Space(box) as sp:
        sp.step(api.STAGE_ALL)
        a = sp.download()
        sp.step_plain()
        b = sp.download()
    assert np.array_equal(a["ngb_first"], b["ngb_first"])
    assert rel_err(b["h"], a["h"]).max() < 2e-4, name
    for k in ("rho", "v_sig"):
        assert rel_err(b[k], a[k]).max() < 3e-4, (name, k)
    for k in ("ax", "ay", "az", "u_dt", "h_dt"):
        assert scaled_err(b[k], a[k]).max() < 1e-3, (name, k)


@pytest.mark.parametrize("jtile,block_warps,tpp", [(32, 4, 1), (16, 8, 1), (16, 4, 1),
                                                   (8, 8, 1), (32, 8, 2), (16, 8, 2),
                                                   (8, 4, 2), (32, 8, 4)])
def test_every_tuning_keeps_parity(case, jtile, block_warps, tpp):
    """Each configuration the autotuner may pick holds the exact-count bar."""
    name, box, ref = case
    with api.Space(box) as sp:
        sp.set_tuning(tpp=tpp, jtile=jtile, block_warps=block_warps)
        assert sp.tuning() == (tpp, jtile, 1, block_warps)  # re-run lists on
        sp.step(api.STAGE_DENSITY)
        first = sp.download()
        sp.step(api.STAGE_ALL)
        sp.force_from_state(ref["h"], ref["rho"], ref["f"], ref["pressure"],
                            ref["soundspeed"], ref["balsara"])
        out = sp.download()
    assert np.array_equal(first["ngb_first"], ref["ngb_first"]), name
    assert rel_err(first["d_rho"], ref["d_rho"]).max() < REL, name
    assert np.array_equal(out["ngb_force"], ref["ngb_force"]), name
    for k in ("ax", "ay", "az", "u_dt", "h_dt"):
        assert scaled_err(out[k], ref[k]).max() < REL, (name, k)


@pytest.mark.parametrize("tpp,widen,cap", [(1, 1.69, 256), (2, 1.0, 64), (2, 2.25, 512)])
def test_row_bound_and_capacity_keep_parity(case, tpp, widen, cap):
    """Rows recorded over another radius or with another capacity (more or
    fewer particles covered by their rows, the rest gathered) keep the
    exact first-pass and force counts and the oracle's sums."""
    name, box, ref = case
    with api.Space(box) as sp:
        sp.set_tuning(tpp=tpp, jtile=32, block_warps=8, row_widen=widen, row_cap=cap)
        sp.step(api.STAGE_DENSITY)
        first = sp.download()
        sp.step()
        sp.step()          # graph replay
        full = sp.download()
        sp.force_from_state(ref["h"], ref["rho"], ref["f"], ref["pressure"],
                            ref["soundspeed"], ref["balsara"])
        out = sp.download()
    assert np.array_equal(first["ngb_first"], ref["ngb_first"]), name
    assert np.array_equal(out["ngb_force"], ref["ngb_force"]), name
    assert rel_err(full["h"], ref["h"]).max() < 2e-4, name
    for k in ("rho", "pressure", "soundspeed"):
        assert rel_err(full[k], ref[k]).max() < 3e-4, (name, k)
    for k in ("ax", "ay", "az", "u_dt", "h_dt"):
        assert scaled_err(out[k], ref[k]).max() < REL, (name, k)


@pytest.mark.parametrize("tpp,jtile", [(1, 32), (2, 32), (1, 16), (2, 8)])
def test_bulk_copy_staging_matches_loads(tpp, jtile):
    """j-blocks fetched by bulk copies (cp.async.bulk into shared memory on an
    mbarrier) give the same step, bit for bit, as j-blocks loaded lane by
    lane: the same records reach the same tests."""
    box = ics.make("clustered:32", seed=12)
    outs = []
    for bulk in (0, 1):
        with api.Space(box) as sp:
            sp.set_tuning(tpp=tpp, jtile=jtile, block_warps=8, bulk_stage=bulk)
            assert sp.bulk_stage() == bulk
            sp.step()
            sp.step()          # graph replay
            outs.append(sp.download())
    a, b = outs
    assert np.array_equal(a["fields"].view(np.uint32), b["fields"].view(np.uint32))
    assert np.array_equal(a["ints"], b["ints"])


@pytest.mark.parametrize("tpp", [1, 2])
def test_rerun_lists_match_rerun_gathers(tpp):
    """Re-runs from the neighbour lists (recorded by one or two lanes per
    particle) give the neighbour sets of re-runs that gather (same counts),
    sums within FP32 summation-order noise."""
    box = ics.make("clustered:40", seed=9)
    outs = []
    for lists in (1, 0):
        with api.Space(box) as sp:
            sp.set_tuning(tpp=tpp, jtile=16, rerun_lists=lists, block_warps=8)
            sp.step()
            sp.step()          # graph replay
            outs.append(sp.download())
    a, b = outs
    assert np.array_equal(a["ngb_first"], b["ngb_first"])
    # summation order differs, so a particle may stop one Newton round
    # earlier or later inside the ghost's tolerance window
    assert np.mean(a["ghost_iters"] == b["ghost_iters"]) > 0.999
    assert np.mean(a["ngb_final"] == b["ngb_final"]) > 0.999
    assert rel_err(a["h"], b["h"]).max() < 2e-4
    for k in ("rho", "pressure", "soundspeed"):
        assert rel_err(a[k], b[k]).max() < 3e-4, k


def test_solver_hands_outgrown_particles_to_catchup_rounds(oracle_lib):
    """Particles whose h grows by far more than the lists' widening (h0 set
    40 % too small on a third of a clustered box) leave the per-particle
    solver for the catch-up gathers: the step still matches the oracle
    (exact first-pass counts, h and densities within tolerance) and the
    re-runs without lists."""
    box = ics.make("clustered:24", seed=17)
    box["h"] = box["h"].copy()
    box["h"][::3] *= np.float32(0.6)
    ref = oracle_lib.run(box)
    outs = []
    for lists in (1, 0):
        with api.Space(box) as sp:
            sp.set_tuning(tpp=2, jtile=32, rerun_lists=lists, block_warps=8)
            sp.step()
            sp.step()          # graph replay
            outs.append(sp.download())
    a, b = outs
    assert np.array_equal(a["ngb_first"], ref["ngb_first"])
    assert np.array_equal(a["ngb_first"], b["ngb_first"])
    assert np.mean(a["ghost_iters"] == ref["ghost_iters"]) > 0.999
    assert np.mean(a["ngb_final"] == ref["ngb_final"]) > 0.999
    assert rel_err(a["h"], ref["h"]).max() < 2e-4
    for k in ("rho", "pressure", "soundspeed"):
        assert rel_err(a[k], ref[k]).max() < 3e-4, k
        assert rel_err(a[k], b[k]).max() < 3e-4, k
    for k in ("ax", "ay", "az", "u_dt"):
        assert scaled_err(a[k], ref[k]).max() < 1e-3, k


def test_autotune_picks_a_candidate():
    box = ics.make("clustered:24", seed=2)
    with api.Space(box) as sp:
        sp.step()
        best, table = sp.autotune(reps=1)
        # 12 tile shapes, then 4 row radii for the fastest shape of each
        # lane count
        assert len(table) == 20 and all(v > 0 for v in table.values())
        key = api.tuning_key(best["jtile"], best["threads_per_particle"],
                             best["block_warps"])
        if best["row_widen"] > 0:
            key += f",row_widen={best['row_widen']:g}"
        assert table[key] == min(table.values())
        assert sp.tuning()[1] == best["jtile"]
        sp.step()
        assert np.all(np.isfinite(sp.download()["ax"]))


def test_step_host_matches_resident_step_and_checks_inputs():
    box = ics.make("clustered:20", seed=3)
    with api.Space(box) as sp:
        sp.step()
        ref = sp.download()
        fields = np.zeros((box["x"].shape[0], 24), np.float32)
        sp.step_host(None, fields)
        assert np.array_equal(fields[:, api.FIELD_COLS["ax"]], ref["ax"])
        faster = dict(box)
        faster["v"] = box["v"] * 2.0      # velocities may change
        sp.step_host(faster, fields)
        assert not np.array_equal(fields[:, api.FIELD_COLS["ax"]], ref["ax"])
        # positions and h may move within the tree (a drift without a
        # rebuild, tests/test_drift.py), not beyond it
        moved = dict(box)
        moved["x"] = box["x"].copy()
        moved["x"][7, 0] += 1e-3
        sp.step_host(moved, fields)
        far = dict(box)
        far["x"] = box["x"].copy()
        far["x"][7, 0] += 0.3
        with pytest.raises(api.SphGpuError) as e:
            sp.step_host(far, fields)
        assert e.value.code == api.EREBUILD
        grown = dict(box)
        grown["h"] = box["h"] * 40.0
        with pytest.raises(api.SphGpuError) as e:
            sp.step_host(grown, fields)
        assert e.value.code == api.EREBUILD


def test_space_update_gives_the_step_of_the_new_state():
    """sphgpu_space_update (new v, m, u after a kick) followed by a resident
    step gives the results, bit for bit, of the host-buffer step on the same
    new state; bad values are refused."""
    box = ics.make("clustered:20", seed=4)
    n = box["x"].shape[0]
    rng = np.random.default_rng(2)
    v2 = (box["v"] + rng.normal(0, 0.05, box["v"].shape)).astype(np.float32)
    m2 = (box["m"] * (1 + 0.1 * rng.random(n))).astype(np.float32)
    u2 = (box["u"] * (1 + 0.5 * rng.random(n))).astype(np.float32)
    new = dict(box, v=v2, m=m2, u=u2)
    with api.Space(box) as sp:
        sp.step()
        fields = np.zeros((n, 24), np.float32)
        sp.step_host(new, fields)
    with api.Space(box) as sp:
        sp.step()
        sp.update(v2, m2, u2)
        sp.step()
        out = sp.download()
        bad = m2.copy()
        bad[3] = 0.0
        with pytest.raises(api.SphGpuError):
            sp.update(v2, bad, u2)
    assert np.array_equal(out["fields"].view(np.uint32), fields.view(np.uint32))


def test_step_host_async_pipeline_matches_step_host():
    """The pipelined host-buffer step: three steps in flight two at a time
    give, bit for bit, the results of the synchronous call on the same
    inputs; a position change is reported when its step is waited for."""
    box = ics.make("clustered:20", seed=3)
    n = box["x"].shape[0]
    boxes = []
    for k in range(3):
        b = {key: np.ascontiguousarray(box[key]) for key in ("x", "v", "m", "h", "u")}
        b["v"] = (box["v"] * (1.0 + 0.5 * k)).astype(np.float32)
        boxes.append(b)
    with api.Space(box) as sp:
        sp.step()
        sync = []
        for b in boxes:
            f = np.zeros((n, 24), np.float32)
            sp.step_host(b, f)
            sync.append(f)
        outs = [np.zeros((n, 24), np.float32) for _ in boxes]
        for b, f in zip(boxes, outs):
            sp.step_host_async(b, f)
        sp.step_host_wait()
        for k in range(3):
            assert np.array_equal(outs[k].view(np.uint32), sync[k].view(np.uint32)), k
        moved = dict(boxes[0])
        moved["x"] = boxes[0]["x"].copy()
        moved["x"][5, 1] += 1e-3
        f = np.zeros((n, 24), np.float32)
        sp.step_host_async(moved, f)
        with pytest.raises(api.SphGpuError):
            sp.step_host_wait()


def test_step_host_async_pipeline_with_late_rounds():
    """A step that needs more ghost rounds than its graph holds (h set fifty
    times too small on a third of the particles): in the pipelined form the
    host reads the step's status during the next call and runs the late
    rounds and the force then; its results, copied down again, equal the
    synchronous call's bit for bit."""
    box = ics.make("clustered:20", seed=5)
    box["h"] = box["h"].copy()
    box["h"][::3] *= np.float32(0.02)
    n = box["x"].shape[0]
    boxes = []
    for k in range(3):
        b = {key: np.ascontiguousarray(box[key]) for key in ("x", "v", "m", "h", "u")}
        b["v"] = (box["v"] * (1.0 + 0.5 * k)).astype(np.float32)
        boxes.append(b)
    with api.Space(box) as sp:
        sp.step()
        sync = []
        for b in boxes:
            f = np.zeros((n, 24), np.float32)
            sp.step_host(b, f)
            sync.append(f)
        sp.step_stats(reset=True)
        outs = [np.zeros((n, 24), np.float32) for _ in boxes]
        for b, f in zip(boxes, outs):
            sp.step_host_async(b, f)
        sp.step_host_wait()
        assert sp.step_stats()["late_rounds"] > 0
        for k in range(3):
            assert np.array_equal(outs[k].view(np.uint32), sync[k].view(np.uint32)), k


# --- open boxes and tiny inputs --------------------------------------------

@pytest.mark.parametrize("cfg,run", [("lattice:16", {"periodic": 0}),
                                     ("clustered:20", {"periodic": 0,
                                                       "max_top_level_cells": 3})])
def test_open_box_parity(cfg, run, oracle_lib):
    box = ics.make(cfg, seed=31)
    ref = oracle_lib.run(box, **run)
    with api.Space(box, **run) as sp:
        sp.step(api.STAGE_DENSITY)
        first = sp.download()
        sp.step()
        full = sp.download()
        sp.force_from_state(ref["h"], ref["rho"], ref["f"], ref["pressure"],
                            ref["soundspeed"], ref["balsara"])
        force = sp.download()
    assert np.array_equal(first["ngb_first"], ref["ngb_first"]), cfg
    assert np.array_equal(force["ngb_force"], ref["ngb_force"]), cfg
    assert rel_err(full["h"], ref["h"]).max() < 2e-4
    for k in ("rho", "pressure", "soundspeed"):
        assert rel_err(full[k], ref[k]).max() < 3e-4, k
    for k in ("ax", "ay", "az", "u_dt", "h_dt"):
        assert scaled_err(force[k], ref[k]).max() < REL, k


def test_parity_with_the_reference_task_split(oracle_lib):
    """Against the oracle with the reference scheduler's task split
    (scheduler_splittask_hydro; bit-identical to the reference run with its
    own splitter): the planner's one task per top cell and top-cell pair
    reaches the same cell pairs, so counts stay exact and the sums agree at
    the usual tolerances."""
    box = ics.make("clustered:24", seed=3)
    run = {"max_top_level_cells": 3}
    ref = oracle_lib.run(box, subsize_self=500, subsize_pair=256000000, **run)
    assert ref["ntasks"] > oracle_lib.run(box, **run)["ntasks"]
    with api.Space(box, **run) as sp:
        sp.step(api.STAGE_DENSITY)
        first = sp.download()
        sp.step()
        full = sp.download()
        sp.force_from_state(ref["h"], ref["rho"], ref["f"], ref["pressure"],
                            ref["soundspeed"], ref["balsara"])
        force = sp.download()
    assert np.array_equal(first["ngb_first"], ref["ngb_first"])
    assert np.array_equal(force["ngb_force"], ref["ngb_force"])
    assert rel_err(full["h"], ref["h"]).max() < 2e-4
    for k in ("rho", "pressure", "soundspeed"):
        assert rel_err(full[k], ref[k]).max() < 3e-4, k
    for k in ("ax", "ay", "az", "u_dt", "h_dt"):
        assert scaled_err(force[k], ref[k]).max() < REL, k


@pytest.mark.parametrize("kind", ["rectangular", "faces", "h_min"])
def test_special_boxes(kind, oracle_lib):
    import sys
    sys.path.insert(0, __import__("os").path.dirname(__file__))
    from test_oracle_reference import special_box
    box, run = special_box(kind)
    ref = oracle_lib.run(box, **run)
    with api.Space(box, **run) as sp:
        sp.step(api.STAGE_DENSITY)
        first = sp.download()
        sp.step()
        full = sp.download()
        sp.force_from_state(ref["h"], ref["rho"], ref["f"], ref["pressure"],
                            ref["soundspeed"], ref["balsara"])
        force = sp.download()
    assert np.array_equal(first["ngb_first"], ref["ngb_first"]), kind
    assert np.array_equal(force["ngb_force"], ref["ngb_force"]), kind
    assert rel_err(full["h"], ref["h"]).max() < 2e-4
    for k in ("rho", "pressure", "soundspeed"):
        assert rel_err(full[k], ref[k]).max() < 3e-4, k
    for k in ("ax", "ay", "az", "u_dt"):
        assert scaled_err(force[k], ref[k]).max() < REL, k


def _tiny(n, seed):
    box = ics.lattice(4, seed=seed)
    for k in ("x", "v", "m", "h", "u", "time_bin"):
        box[k] = box[k][:n].copy()
    return box


@pytest.mark.parametrize("n", [1, 2, 5, 17])
def test_tiny_open_boxes(n, oracle_lib):
    box = _tiny(n, seed=n)
    run = {"periodic": 0, "h_max": 0.6}
    ref = oracle_lib.run(box, **run)
    with api.Space(box, **run) as sp:
        sp.step()
        out = sp.download()
    assert np.array_equal(out["ngb_first"], ref["ngb_first"])
    assert rel_err(out["h"], ref["h"]).max() < 2e-4
    assert rel_err(out["rho"], ref["rho"]).max() < 3e-4
    if n == 1:
        assert out["h"][0] == np.float32(0.6)


def test_lonely_particle_without_h_max_reports_nonconvergence():
    with api.Space(_tiny(1, seed=1), periodic=0) as sp:
        with pytest.raises(api.SphGpuError) as e:
            sp.step()
    assert e.value.code == api.ENOCONV


# --- sparse activity on carried state --------------------------------------

@pytest.mark.parametrize("cfg,mab", [("sedov:24", 22), ("sedov:32", 21),
                                     ("clustered:24", 21)])
def test_primed_sparse_step(cfg, mab, oracle_lib):
    """An all-active step, then a step at max_active_bin on the state it
    leaves, against the oracle's same two steps; inactive particles keep
    their state bit for bit on the GPU."""
    box = ics.make(cfg, seed=6)
    if cfg.startswith("clustered"):
        box["time_bin"][:] = 20 + (np.arange(box["x"].shape[0]) * 7919) % 4
    ref = oracle_lib.run(box, api.STAGE_PRIME | api.STAGE_ALL, max_active_bin=mab)
    act = box["time_bin"] <= mab
    assert 0 < act.sum() < act.size
    with api.Space(box) as sp:
        sp.set_active(api.ALL_ACTIVE)
        sp.step()
        first = sp.download()
        sp.set_active(mab)
        sp.step(api.STAGE_DENSITY)
        dens = sp.download()
        sp.step()
        out = sp.download()
    # first density pass of the active particles: counts exact
    assert np.array_equal(dens["ngb_first"][act], ref["ngb_first"][act]), cfg
    assert rel_err(dens["d_rho"][act], ref["d_rho"][act]).max() < REL
    # inactive particles: untouched by the second step
    for k in ("h", "rho", "f", "pressure", "soundspeed", "balsara", "ax", "ay",
              "az", "u_dt", "h_dt", "v_sig"):
        assert np.array_equal(out[k][~act], first[k][~act]), k
    # every particle against the oracle's two steps
    assert rel_err(out["h"], ref["h"]).max() < 2e-4, cfg
    for k in ("rho", "pressure", "soundspeed", "v_sig"):
        assert rel_err(out[k], ref[k]).max() < 3e-4, (cfg, k)
    for k in ("ax", "ay", "az", "u_dt", "h_dt"):
        assert scaled_err(out[k][act], ref[k][act]).max() < 1e-3, (cfg, k)
    assert np.mean(out["ngb_final"][act] == ref["ngb_final"][act]) > 0.99


def test_sparse_steps_replay_one_graph(oracle_lib):
    """After the all-active step, every sparse step is one CUDA graph: the
    force lists are planned when the active set is set, from each active
    particle's last converged h, and checked on the device against the
    post-ghost h (on a static box the check always passes, so no step
    re-plans and the graph captured for the first sparse step serves them
    all).  The last step matches the oracle's primed sparse step."""
    box = ics.make("sedov:32", seed=6)
    mab = 21
    ref = oracle_lib.run(box, api.STAGE_PRIME | api.STAGE_ALL, max_active_bin=mab)
    act = box["time_bin"] <= mab
    with api.Space(box) as sp:
        sp.set_active(api.ALL_ACTIVE)
        sp.step()
        sp.step_stats(reset=True)
        for b in (22, 20, 23, 21, 22, mab):
            sp.set_active(b)
            sp.step()
        st = sp.step_stats()
        out = sp.download()
    assert st["graph_steps"] == 6 and st["captures"] == 1, st
    assert st["force_replans"] == 0 and st["late_rounds"] == 0, st
    assert np.array_equal(out["ngb_first"][act], ref["ngb_first"][act])
    assert rel_err(out["h"], ref["h"]).max() < 2e-4
    for k in ("rho", "pressure", "soundspeed", "v_sig"):
        assert rel_err(out[k], ref[k]).max() < 3e-4, k
    for k in ("ax", "ay", "az", "u_dt", "h_dt"):
        assert scaled_err(out[k][act], ref[k][act]).max() < 1e-3, k
    assert np.mean(out["ngb_force"][act] == ref["ngb_force"][act]) > 0.99


def test_all_active_steps_replay_one_graph():
    """All-active steps after the first: one graph each, the force plan of
    the first step verified on the device every step."""
    box = ics.make("clustered:24", seed=3)
    with api.Space(box) as sp:
        sp.step()
        a = sp.download()
        sp.step_stats(reset=True)
        for _ in range(3):
            sp.step()
        st = sp.step_stats()
        b = sp.download()
    assert st == {"graph_steps": 3, "force_replans": 0, "late_rounds": 0, "captures": 1}, st
    assert np.array_equal(a["ngb_force"], b["ngb_force"])
    assert np.array_equal(a["ngb_first"], b["ngb_first"])


def test_primed_sparse_plain_equals_batched():
    box = ics.make("sedov:24", seed=8)
    with api.Space(box) as sp:
        sp.primed_step(22)
        a = sp.download()
    with api.Space(box) as sp:
        sp.primed_step(22, plain=True)
        b = sp.download()
    act = box["time_bin"] <= 22
    assert np.array_equal(a["ngb_first"][act], b["ngb_first"][act])
    assert rel_err(b["h"], a["h"]).max() < 2e-4
    for k in ("ax", "ay", "az", "u_dt"):
        assert scaled_err(b[k][act], a[k][act]).max() < 1e-3, k


# --- directly against the reference's own outputs (golden fixtures) ---------

import ast  # noqa: E402
import glob  # noqa: E402
import os  # noqa: E402

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


@pytest.mark.parametrize("path", sorted(p for p in glob.glob(os.path.join(GOLDEN, "*.npz"))
       if not os.path.basename(p).startswith("sorts_")),
                         ids=lambda p: os.path.basename(p)[:-4])
def test_gpu_against_reference_golden(path):
    g = np.load(path)
    box = getattr(ics, str(g["kind"]))(int(g["n"]), **ast.literal_eval(str(g["gen_kwargs"])))
    run = ast.literal_eval(str(g["run_kwargs"]))
    stages = run.pop("stages", api.STAGE_ALL)
    with api.Space(box, **run) as sp:
        if stages & api.STAGE_PRIME:
            sp.primed_step(run["max_active_bin"], stages & api.STAGE_ALL)
        else:
            sp.step(stages)
        out = sp.download()
    idx = g["sample"]
    ref = g["fields"]
    active = box["time_bin"][idx] <= run.get("max_active_bin", 56)
    assert active.sum() > 0
    col = api.FIELD_COLS
    h = out["fields"][idx][active]
    r = ref[active]
    assert np.max(np.abs(h[:, col["h"]] - r[:, 8]) / r[:, 8]) < 2e-4
    for name, c in (("rho", 9), ("pressure", 11), ("soundspeed", 12)):
        assert np.max(np.abs(h[:, col[name]] - r[:, c]) / np.abs(r[:, c])) < 3e-4, name
    if stages & api.STAGE_FORCE:
        for name, c in (("ax", 15), ("ay", 16), ("az", 17), ("u_dt", 18), ("h_dt", 19)):
            scale = np.max(np.abs(ref[:, c])) + 1e-30
            assert np.max(np.abs(h[:, col[name]] - r[:, c])) / scale < 1e-3, name
        assert np.max(np.abs(h[:, col["v_sig"]] - r[:, 20]) / r[:, 20]) < 3e-4
