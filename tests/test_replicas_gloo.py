"""Multi-rank aggregation of bench.py on CPU (gloo, world size 2): every rank
runs its own replica box; the job's value is all ranks' interactions over the
slowest rank's time."""
import os
import socket

import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    t_step = [0.010, 0.012][rank]
    inter = [1000.0, 1500.0][rank]
    v = bench.reduce_over_ranks(t_step, 0.02 + rank, inter, device="cpu")
    q.put((rank, v))
    dist.destroy_process_group()


def test_two_rank_reduction():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    res = dict(q.get() for _ in range(2))
    for r in (0, 1):
        t_step, e2e, total = res[r]
        assert t_step == pytest.approx(0.012)
        assert e2e == pytest.approx(1.02)
        assert total == pytest.approx(2500.0)
