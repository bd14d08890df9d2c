"""Replica aggregation of bench.py across ranks, on CPU with gloo (world size 2)."""
import os
import socket

import pytest
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
    # rank 1 is slower: the job time is the slowest replica's
    step_ms, e2e_s = bench.max_over_ranks(10.0 + 5.0 * rank, 0.02 + 0.01 * rank, dist)
    q.put((rank, step_ms, e2e_s, bench.job_value(1000, step_ms, world)))
    dist.destroy_process_group()


def test_replicas_max_over_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
    res = sorted(q.get(timeout=5) for _ in range(2))
    for rank, step_ms, e2e_s, value in res:
        assert step_ms == pytest.approx(15.0) and e2e_s == pytest.approx(0.03)
        assert value == pytest.approx(2 * 1000 / 0.015)
