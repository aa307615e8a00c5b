"""Serving workload: a seeded stream of independent SPH boxes run through the
continuous-batching server (``api.Server``).

Each request is one box of the two shapes the hot path is measured on -- a
jittered lattice or the clustered Gaussian-random-field box (coin flip) --
with N drawn log-uniform in [4,096, 262,144] and rounded to the nearest cube
n^3 (16 <= n <= 64), a uniform u in [0.5, 2], and 10 density -> ghost ->
force steps kept device-resident.  Arrivals are Poisson at a given rate, or
all at t = 0 to measure capacity.

``serve`` drives the server as a request loop would: it submits every
request whose arrival time has passed, pumps the server (admission by free
arena space, one step of every resident box per pump, retirement of the
finished ones) and records each request's latency from its arrival to the
pump that returned it.
"""
from __future__ import annotations

import math
import time
from collections import deque
from dataclasses import dataclass

import numpy as np

from . import ics

N_MIN, N_MAX = 4096, 262144
STEPS = 10


@dataclass
class RequestSpec:
    rid: int
    kind: str        # "lattice" or "clustered"
    n: int           # particles per side; the box holds n^3
    seed: int
    u: float


def request_stream(count, seed=0, n_min=N_MIN, n_max=N_MAX):
    """``count`` seeded request specifications."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(count):
        N = math.exp(rng.uniform(math.log(n_min), math.log(n_max)))
        n = int(min(64, max(16, round(N ** (1.0 / 3.0)))))
        kind = "lattice" if rng.random() < 0.5 else "clustered"
        out.append(RequestSpec(i, kind, n, int(rng.integers(1 << 30)),
                               float(rng.uniform(0.5, 2.0))))
    return out


def make_box(spec):
    """The box of one request (seeded, so the same spec gives the same box)."""
    if spec.kind == "lattice":
        box = ics.lattice(spec.n, seed=spec.seed)
    else:
        box = ics.clustered(spec.n, seed=spec.seed, rms=0.3)
    box["u"][:] = spec.u
    return box


def _make(spec):
    return make_box(spec)


def make_boxes(specs, processes=0):
    """Boxes of many requests; ``processes`` > 1 generates them in a spawned
    process pool."""
    if processes and processes > 1 and len(specs) > 8:
        import multiprocessing as mp
        with mp.get_context("spawn").Pool(processes) as pool:
            return pool.map(_make, specs, chunksize=8)
    return [make_box(s) for s in specs]


def poisson_arrivals(count, rate, seed=0):
    """Arrival times (s) of a Poisson process of the given rate; all zero
    when ``rate`` is None (a saturating burst)."""
    if rate is None:
        return np.zeros(count)
    rng = np.random.default_rng(seed + 104729)
    return np.cumsum(rng.exponential(1.0 / rate, size=count))


def serve(server, boxes, arrivals, nsteps=STEPS, keep=None):
    """Run a request stream through ``server``.

    Returns per-request latency (s, arrival -> completion), the wall time
    from the first arrival to the last completion, and the results of the
    requests listed in ``keep``."""
    order = np.argsort(arrivals, kind="stable")
    pending = deque(int(i) for i in order)
    arr_of = {}
    lat = {}
    kept = {}
    keep = set(keep or ())
    t0 = time.perf_counter()
    while pending or arr_of:
        now = time.perf_counter() - t0
        while pending and arrivals[pending[0]] <= now:
            i = pending.popleft()
            server.submit(i, boxes[i], nsteps)
            arr_of[i] = float(arrivals[i])
        resident = server.pump(wait_s=0.002)
        done_t = time.perf_counter() - t0
        for rid in server.poll():
            res = server.fetch(rid)
            lat[rid] = done_t - arr_of.pop(rid)
            if rid in keep:
                kept[rid] = res
        if resident == 0 and pending and not arr_of:
            wait = arrivals[pending[0]] - (time.perf_counter() - t0)
            if wait > 0:
                time.sleep(min(wait, 0.01))
    wall = time.perf_counter() - t0 - float(np.min(arrivals))
    return lat, wall, kept


def latency_summary(lat):
    v = np.array(sorted(lat.values()))
    return {"p50_s": float(np.percentile(v, 50)), "p99_s": float(np.percentile(v, 99)),
            "mean_s": float(v.mean()), "max_s": float(v.max())}
