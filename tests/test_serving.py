"""Serving loop: request stream generator (CPU) and the continuous-batching
server on the GPU -- each box's result is the same alone and in the mix, and
the same as the single-box batched form and the oracle's loops."""
import numpy as np
import pytest

from swift_gb300 import serve

FIELDS = ("h", "rho", "f", "pressure", "soundspeed", "balsara", "ax", "ay",
          "az", "u_dt", "h_dt", "v_sig")


def test_request_stream_is_seeded_and_in_range():
    a = serve.request_stream(400, seed=3)
    b = serve.request_stream(400, seed=3)
    assert a == b
    ns = np.array([s.n ** 3 for s in a])
    assert ns.min() >= 16 ** 3 and ns.max() <= 64 ** 3
    # log-uniform in N: the median sits near sqrt(4096 * 262144) = 32768
    assert 16000 < np.median(ns) < 65000
    kinds = [s.kind for s in a]
    assert 0.4 < kinds.count("lattice") / len(kinds) < 0.6
    us = np.array([s.u for s in a])
    assert us.min() >= 0.5 and us.max() <= 2.0


def test_poisson_arrivals():
    t = serve.poisson_arrivals(20000, 250.0, seed=1)
    assert np.all(np.diff(t) >= 0)
    assert abs(20000 / t[-1] - 250.0) / 250.0 < 0.03
    assert np.all(serve.poisson_arrivals(5, None) == 0)


def test_make_box_applies_u():
    s = serve.RequestSpec(0, "clustered", 16, 5, 1.25)
    box = serve.make_box(s)
    assert box["x"].shape == (4096, 3)
    assert np.all(box["u"] == np.float32(1.25))


# --- GPU ---------------------------------------------------------------------

def _run_until_done(srv, ids):
    out = {}
    for _ in range(10000):
        srv.pump(wait_s=0.01)
        for rid in srv.poll():
            out[rid] = srv.fetch(rid)
        if set(ids) <= set(out):
            return out
    raise AssertionError("server did not finish")


@pytest.mark.gpu
def test_alone_equals_mix():
    """A box run alone and the same box run while five others of other
    sizes and shapes share its launches, joining and leaving at other steps:
    identical results, bit for bit."""
    from swift_gb300 import api
    specs = [serve.RequestSpec(0, "clustered", 20, 11, 1.5),
             serve.RequestSpec(1, "lattice", 16, 12, 0.7),
             serve.RequestSpec(2, "clustered", 24, 13, 1.1),
             serve.RequestSpec(3, "lattice", 28, 14, 1.9),
             serve.RequestSpec(4, "clustered", 16, 15, 0.6),
             serve.RequestSpec(5, "lattice", 22, 16, 1.3)]
    boxes = [serve.make_box(s) for s in specs]
    alone = {}
    with api.Server(max_particles=1 << 20) as srv:
        for i in (0, 3):
            srv.submit(i, boxes[i], nsteps=4)
            alone.update(_run_until_done(srv, [i]))
    with api.Server(max_particles=1 << 20) as srv:
        for i in (1, 2):
            srv.submit(i, boxes[i], nsteps=4)
        srv.pump(wait_s=5.0)
        srv.pump(wait_s=5.0)          # 1 and 2 are two steps in
        srv.submit(0, boxes[0], nsteps=4)
        srv.submit(3, boxes[3], nsteps=4)
        srv.pump(wait_s=5.0)
        srv.submit(4, boxes[4], nsteps=4)
        srv.submit(5, boxes[5], nsteps=4)
        mix = _run_until_done(srv, range(6))
    for i in (0, 3):
        assert np.array_equal(alone[i]["fields"].view(np.uint32),
                              mix[i]["fields"].view(np.uint32)), i
        assert np.array_equal(alone[i]["ints"], mix[i]["ints"]), i
    for i in range(6):
        assert np.all(np.isfinite(mix[i]["fields"][:, :21])), i


@pytest.mark.gpu
def test_server_matches_single_space_and_oracle(oracle_lib):
    from swift_gb300 import api
    from test_gpu_parity import rel_err, scaled_err
    spec = serve.RequestSpec(0, "clustered", 24, 21, 1.7)
    box = serve.make_box(spec)
    with api.Server(max_particles=1 << 20) as srv:
        srv.submit(7, box, nsteps=3)
        out = _run_until_done(srv, [7])[7]
    with api.Space(box) as sp:
        # the arena's configuration: j-blocks of 16, one lane per particle,
        # 8 warps per block, rows of the first pass for the ghost and force
        sp.set_tuning(jtile=16, rerun_lists=1, block_warps=8)
        sp.step()
        one = sp.download()
    # the same lists and kernels as the single-box batched form
    for k in ("ngb_first", "ngb_final", "ngb_force"):
        assert np.array_equal(out[k], one[k]), k
    for k in FIELDS:
        assert np.array_equal(out[k], one[k]), k
    ref = oracle_lib.run(box)
    assert np.array_equal(out["ngb_first"], ref["ngb_first"])
    assert rel_err(out["h"], ref["h"]).max() < 2e-4
    for k in ("rho", "pressure", "soundspeed", "v_sig"):
        assert rel_err(out[k], ref[k]).max() < 3e-4, k
    for k in ("ax", "ay", "az", "u_dt", "h_dt"):
        assert scaled_err(out[k], ref[k]).max() < 1e-3, k


@pytest.mark.gpu
def test_server_stream_small():
    from swift_gb300 import api
    specs = serve.request_stream(40, seed=9, n_max=40000)
    boxes = serve.make_boxes(specs)
    arr = serve.poisson_arrivals(len(specs), 400.0, seed=9)
    with api.Server(max_particles=1 << 21) as srv:
        lat, wall, _ = serve.serve(srv, boxes, arr, nsteps=3)
        st = srv.stats()
    assert len(lat) == 40 and st["resident"] == 0 and st["retired"] == 40
    assert st["arena_particles_used"] == 0
    assert all(v > 0 for v in lat.values())
