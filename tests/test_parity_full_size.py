"""GPU parity at the benchmark sizes, against the oracle (oracle/sph_oracle.c,
bit-identical to the reference's own loops in the same task order).

Boxes: the batched form's clustered 128^3 box (2,097,152 particles); the
sparse-activity 256^3 Sedov box (16,777,216 particles) on its primed second
step; the serving mix with boxes up to the stream's largest (64^3 = 262,144);
and the first density pass of chosen top cells of the strongly clustered
384^3 box (56,623,104 particles), where h moves by more than 10 % and the
catch-up gathers carry the ghost.

Tolerances (the reference's tests/difffloat.py conventions: a relative
tolerance per particle, and a stated limit below which a value counts as
near zero):

* neighbour counts: exact, given the same h (the first pass from the input
  h; the density at the oracle's converged h; the force from the oracle's
  post-ghost state);
* given the same h or state, every field per particle: positive sums (rho,
  wcount, v_sig) within 1e-4 relative; signed sums whose terms cancel
  (rho_dh, wcount_dh, div_v, rot_v, a, du/dt, dh/dt) within 1e-4 relative to
  max(|value|, FLOOR x the field's rms), FLOOR = 1: the near-zero limit is
  the field's rms.  Below it a value is a residual of terms that cancel, and
  FP32 arithmetic itself does not hold it to 1e-4: the reference's own
  accelerations differ from the FP64 brute force by up to 2.2e-4 relative
  at 0.1 x rms, 8.4e-5 at 0.3 x rms and 2.5e-5 at 1 x rms (clustered 48^3
  box); the test prints both codes' errors against the FP64 brute force
  (sph_oracle_exact64) at these floors for the 128^3 box, and holds the GPU
  to twice the reference's; where the reference's own FP64 error at the
  floor exceeds 5e-5 (the hot particles of the Sedov blast, whose
  accelerations cancel much larger pressure terms), the GPU is held to twice
  that error instead of 1e-4;
* after the independent ghosts (the full pass): the reference's own spread
  between two task orders on the same box, measured in the test (the oracle
  with and without the reference scheduler's task split, or in reversed
  task order): each field's largest deviation from the oracle, in units of
  the field's rms, is held to three times the spread's (1e-4 at least, and
  never above 1e-3 for the positive fields) -- the largest deviation is set
  by the few particles whose Newton iteration stops one step earlier or
  later, a rare-event statistic; the h window itself is the ghost's 1e-4
  tolerance (runner_ghost.c:1385-1392), so two convergences may sit 2e-4
  apart.

The oracle runs in threads (its C calls release the GIL) beside the GPU.
"""
import concurrent.futures as cf

import numpy as np
import pytest

from swift_gb300 import api, ics

pytestmark = pytest.mark.gpu

REL = 1e-4
FLOOR = 1.0
FLOORS = (0.1, 0.3, 1.0)
SPLIT = {"subsize_self": 500, "subsize_pair": 256000000}
POS_D = ("d_rho", "d_wcount")
SIGNED_D = ("d_rho_dh", "d_wcount_dh", "d_div_v", "d_rot_vx", "d_rot_vy", "d_rot_vz")
SIGNED_F = ("ax", "ay", "az", "u_dt", "h_dt")
STATE = ("h", "rho", "f", "pressure", "soundspeed", "balsara")


def pp_err(a, b, floor=None):
    """Per-particle |a - b| / max(|b|, floor x rms(b))."""
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    scale = np.abs(b)
    if floor is not None:
        scale = np.maximum(scale, floor * np.sqrt(np.mean(b * b)))
    return np.abs(a - b) / np.maximum(scale, 1e-37)


def rms_err(a, b):
    """Largest |a - b| in units of the field's rms."""
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return np.max(np.abs(a - b)) / (np.sqrt(np.mean(b * b)) + 1e-37)


def floors(a, b):
    return " ".join(f"{pp_err(a, b, F).max():.1e}" for F in FLOORS)


def check_same_h_density(out, ref, mask=None, what=""):
    m = slice(None) if mask is None else mask
    assert np.array_equal(out["ngb_first"][m], ref["ngb_first"][m]), what
    report = {}
    for k in POS_D:
        report[k] = pp_err(out[k][m], ref[k][m]).max()
    for k in SIGNED_D:
        report[k] = pp_err(out[k][m], ref[k][m], FLOOR).max()
    print(what, {k: f"{v:.2e}" for k, v in report.items()})
    print("  signed sums at floors", FLOORS, {k: floors(out[k][m], ref[k][m]) for k in SIGNED_D})
    for k, v in report.items():
        assert v < REL, (what, k, v)


EXACT_COLS = {"ax": 3, "ay": 4, "az": 5, "u_dt": 6}


def check_same_state_force(out, ref, mask=None, what="", exact=None):
    """Force given the same post-ghost state.  With ``exact`` (the FP64
    brute force on that state) a field whose reference value is itself
    further than REL/2 from FP64 at the floor is held to twice the
    reference's own FP64 error instead of REL: FP32 cannot do better."""
    m = slice(None) if mask is None else mask
    assert np.array_equal(out["ngb_force"][m], ref["ngb_force"][m]), what
    report = {"v_sig": pp_err(out["v_sig"][m], ref["v_sig"][m]).max()}
    bound = {"v_sig": REL}
    for k in SIGNED_F:
        report[k] = pp_err(out[k][m], ref[k][m], FLOOR).max()
        bound[k] = REL
        if exact is not None and k in EXACT_COLS:
            e_ref = pp_err(ref[k][m], exact[m, EXACT_COLS[k]], FLOOR).max()
            e_gpu = pp_err(out[k][m], exact[m, EXACT_COLS[k]], FLOOR).max()
            print(f"  {k} vs FP64 at floor {FLOOR:g} x rms: reference {e_ref:.2e}, GPU {e_gpu:.2e}")
            bound[k] = max(REL, 2.0 * e_ref)
    print(what, {k: f"{v:.2e}" for k, v in report.items()})
    print("  signed sums at floors", FLOORS, {k: floors(out[k][m], ref[k][m]) for k in SIGNED_F})
    for k, v in report.items():
        assert v < bound[k], (what, k, v, bound[k])


FULL_POS = ("h", "rho", "pressure", "soundspeed", "v_sig")
FULL_SIGNED = ("f", "balsara", "ax", "ay", "az", "u_dt", "h_dt")


def check_full_pass(out, ref, spread_ref, mask=None, what="", same_state=None):
    """GPU vs oracle after independent ghosts, against the oracle's own
    spread between two task orders (spread_ref vs ref) and, where given, the
    GPU's deviation from the oracle on the same post-ghost state (the part
    of the difference that comes from FP32 arithmetic, not from the ghost)."""
    m = slice(None) if mask is None else mask
    same_state = same_state or {}
    rows = {}
    for k in FULL_POS + FULL_SIGNED:
        got = rms_err(out[k][m], ref[k][m])
        own = rms_err(spread_ref[k][m], ref[k][m])
        rows[k] = (got, max(own, same_state.get(k, 0.0)))
    print(what, {k: f"{g:.2e} (own {o:.2e})" for k, (g, o) in rows.items()})
    # the ghost's window: both stop within 1e-4 of the root
    assert pp_err(out["h"][m], ref["h"][m]).max() < 2e-4, what
    for k, (got, own) in rows.items():
        bound = max(3.0 * own, REL)
        if k in FULL_POS:
            bound = min(bound, 1e-3)
        assert got <= bound, (what, k, got, own)
    # neighbour counts agree wherever both converged to the same iterate
    same = out["ghost_iters"][m] == ref["ghost_iters"][m]
    assert np.mean(same) > 0.99, what


@pytest.fixture(scope="module")
def pool():
    with cf.ThreadPoolExecutor(4) as ex:
        yield ex


# --- clustered 128^3 (the batched form's box) -------------------------------

@pytest.fixture(scope="module")
def c128(pool, oracle_lib):
    from oracle import integrate as oi
    box = ics.make("clustered:128", seed=5)
    fa = pool.submit(oracle_lib.run, box)
    fb = pool.submit(oracle_lib.run, box, **SPLIT)
    with api.Space(box) as sp:
        sp.step(api.STAGE_DENSITY)
        first = sp.download()
        sp.step()
        full = sp.download()
        ref = fa.result()
        # density at the oracle's converged h; force from its post-ghost state
        st6 = np.stack([ref[k] for k in STATE], 1)
        boxh = dict(box)
        boxh["h"] = ref["h"].copy()
        fc = pool.submit(oracle_lib.run, boxh, oracle_lib.STAGE_DENSITY)
        fd = pool.submit(oi.run_state_force, box, st6)
        fe = pool.submit(oracle_lib.exact64, box, ref)
        sp.force_from_state(*[ref[k] for k in STATE])
        force = sp.download()
    with api.Space(boxh) as sp:
        sp.step(api.STAGE_DENSITY)
        dens_h = sp.download()
    return dict(box=box, first=first, full=full, force=force, dens_h=dens_h, ref=ref,
                split=fb.result(), ref_h=fc.result(), ref_force=fd.result(),
                exact=fe.result())


def test_c128_first_pass_exact(c128):
    check_same_h_density(c128["first"], c128["ref"], what="128^3 first pass")


def test_c128_density_at_converged_h_exact(c128):
    check_same_h_density(c128["dens_h"], c128["ref_h"], what="128^3 density at the oracle's h")


def test_c128_force_from_oracle_state_exact(c128):
    rf = _force_rows(c128["ref_force"])
    check_same_state_force(c128["force"], rf, what="128^3 force from the oracle's state")


def test_c128_errors_against_the_fp64_brute_force(c128):
    """Both codes' FP32 accelerations and du/dt against the FP64 brute force
    on the oracle's post-ghost state, at the floors of the module's
    docstring: the GPU's error is at most twice the reference's."""
    ex = c128["exact"]
    rf = c128["ref_force"]
    g = c128["force"]
    for k, col, refv in (("ax", 3, rf["a"][:, 0]), ("ay", 4, rf["a"][:, 1]),
                         ("az", 5, rf["a"][:, 2]), ("u_dt", 6, rf["u_dt"])):
        e_ref = [pp_err(refv, ex[:, col], F).max() for F in FLOORS]
        e_gpu = [pp_err(g[k], ex[:, col], F).max() for F in FLOORS]
        print(f"{k}: vs FP64 at floors {FLOORS}: reference "
              + " ".join(f"{v:.1e}" for v in e_ref) + " | GPU " + " ".join(f"{v:.1e}" for v in e_gpu))
        assert e_gpu[-1] <= 2.0 * e_ref[-1] + 1e-6, (k, e_gpu, e_ref)


def _force_rows(force):
    out = dict(force)
    if "a" in out:
        for j, k in enumerate(("ax", "ay", "az")):
            out[k] = out["a"][:, j]
    return out


def _same_state(gpu, ref, mask=None):
    m = slice(None) if mask is None else mask
    return {k: rms_err(gpu[k][m], ref[k][m]) for k in SIGNED_F}


def test_c128_full_pass_within_the_references_own_spread(c128):
    assert c128["split"]["ntasks"] > c128["ref"]["ntasks"]
    same = _same_state(c128["force"], _force_rows(c128["ref_force"]))
    check_full_pass(c128["full"], c128["ref"], c128["split"], what="128^3 full pass",
                    same_state=same)
    assert np.array_equal(c128["full"]["ngb_first"], c128["ref"]["ngb_first"])


# --- Sedov 256^3, primed sparse step -----------------------------------------

SEDOV_MAB = 21


@pytest.fixture(scope="module")
def sedov256(pool, oracle_lib):
    box = ics.make("sedov:256", seed=6)
    act = box["time_bin"] <= SEDOV_MAB
    stages = api.STAGE_PRIME | api.STAGE_ALL
    fa = pool.submit(oracle_lib.run, box, stages, max_active_bin=SEDOV_MAB)
    fb = pool.submit(oracle_lib.run, box, stages, max_active_bin=SEDOV_MAB, **SPLIT)
    from oracle import integrate as oi
    with api.Space(box) as sp:
        sp.set_active(api.ALL_ACTIVE)
        sp.step()
        prime = sp.download()
        sp.set_active(SEDOV_MAB)
        sp.step(api.STAGE_DENSITY)
        dens = sp.download()
        sp.step()
        out = sp.download()
        ref = fa.result()
        # the force of the active particles on the oracle's state
        st6 = np.stack([ref[k] for k in STATE], 1)
        fc = pool.submit(oi.run_state_force, box, st6, max_active_bin=SEDOV_MAB)
        fe = pool.submit(oracle_lib.exact64, box, ref, act)
        sp.force_from_state(*[ref[k] for k in STATE])
        force = sp.download()
    return dict(box=box, act=act, prime=prime, dens=dens, out=out, ref=ref,
                split=fb.result(), force=force, ref_force=_force_rows(fc.result()),
                exact=fe.result())


def test_sedov256_sparse_step(sedov256):
    d = sedov256
    act = d["act"]
    frac = act.mean()
    assert 0.005 < frac < 0.15, frac
    check_same_h_density(d["dens"], d["ref"], mask=act, what="sedov 256^3 sparse first pass")
    for k in STATE + ("ax", "ay", "az", "u_dt", "h_dt", "v_sig"):
        assert np.array_equal(d["out"][k][~act], d["prime"][k][~act]), k
    check_same_state_force(d["force"], d["ref_force"], mask=act,
                           what="sedov 256^3 force from the oracle's state", exact=d["exact"])
    same = _same_state(d["force"], d["ref_force"], mask=act)
    check_full_pass(d["out"], d["ref"], d["split"], mask=act, what="sedov 256^3 sparse step",
                    same_state=same)


# --- serving mix up to the stream's largest box --------------------------------

def test_serving_mix_at_full_box_sizes(pool, oracle_lib):
    """Five boxes, from the stream's largest (64^3) to its smallest (16^3),
    two of them joining a pump later: each against the oracle, and each
    box's full pass within the oracle's own spread between two task orders
    (the reference driver's order and its reverse; the trees of these boxes
    are too shallow for the scheduler's task split)."""
    from swift_gb300 import serve
    specs = [serve.RequestSpec(0, "clustered", 64, 31, 1.2),   # 262,144: the largest
             serve.RequestSpec(1, "lattice", 64, 32, 0.8),
             serve.RequestSpec(2, "clustered", 40, 33, 1.9),
             serve.RequestSpec(3, "lattice", 24, 34, 0.6),
             serve.RequestSpec(4, "clustered", 16, 35, 1.4)]   # 4,096: the smallest
    boxes = [serve.make_box(s) for s in specs]
    futs = [pool.submit(oracle_lib.run, b) for b in boxes]
    revs = [pool.submit(oracle_lib.run, b, reverse_tasks=1) for b in boxes]
    with api.Server(max_particles=1 << 21) as srv:
        for i in (0, 2):
            srv.submit(i, boxes[i], nsteps=2)
        srv.pump(wait_s=10.0)
        for i in (1, 3, 4):
            srv.submit(i, boxes[i], nsteps=2)
        out = {}
        for _ in range(10000):
            srv.pump(wait_s=0.01)
            for rid in srv.poll():
                out[rid] = srv.fetch(rid)
            if len(out) == len(boxes):
                break
    assert len(out) == len(boxes)
    for i in range(len(boxes)):
        ref = futs[i].result()
        assert np.array_equal(out[i]["ngb_first"], ref["ngb_first"]), i
        check_full_pass(out[i], ref, revs[i].result(), what=f"serving box {i}")


# --- 384^3, rms 1.0: first pass of chosen top cells ------------------------------

def test_large384_first_pass_of_chosen_top_cells(oracle_lib):
    box = ics.clustered(384, seed=1, rms=1.0)
    with api.Space(box) as sp:
        sp.step(api.STAGE_DENSITY)
        out = sp.download()
        cells = sp.cells()
    top = cells["top"]
    counts = np.bincount(top)
    # the densest and the emptiest top cells, and two in between
    order = np.argsort(counts)
    tops = [int(order[-1]), int(order[0]), int(order[len(order) // 2]), int(order[len(order) // 3])]
    ref = oracle_lib.first_pass_tops(box, tops)
    m = ref["in_tops"]
    assert np.array_equal(ref["top"], top)
    assert m.sum() == counts[tops].sum() > 0
    check_same_h_density(out, ref, mask=m, what="384^3 first pass, 4 top cells")
