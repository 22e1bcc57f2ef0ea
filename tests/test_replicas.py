"""The multi-GPU path: independent replicas whose only collective is the
timing reduction (max over ranks).  Two gloo ranks on CPU."""
from __future__ import annotations

import os
import socket

import pytest


def _free_port() -> int:
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank(rank: int, world: int, port: int, out):
    import torch.distributed as dist

    from tmp_gb300 import replicas

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        # each rank stepped 1000 units of its own; rank r took 1 + r seconds
        out.put((rank, replicas.job_rate(1000, 1.0 + rank, world, dist)))
    finally:
        dist.barrier()
        dist.destroy_process_group()


def test_job_rate_two_gloo_ranks():
    import torch.multiprocessing as mp

    world = 2
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    res = dict(q.get(timeout=120) for _ in range(world))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for r in range(world):
        t_max, rate = res[r]
        assert t_max == 2.0  # the slowest rank's time
        assert rate == 1000 * world / 2.0  # all ranks' work over that time


def test_job_rate_single_process():
    from tmp_gb300 import replicas

    assert replicas.job_rate(500, 0.25, 1) == (0.25, 2000.0)
