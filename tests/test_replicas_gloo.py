"""The N-GPU form of bench.py is N independent replicas (no data-path collective): the
whole-job figure is the slowest rank's time and the sum of every rank's rays.  This runs that
reduction with two gloo ranks on the CPU."""
from __future__ import annotations

import os
import socket

import pytest


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank(rank, world, port, q):
    import torch
    import torch.distributed as dist

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench

    ms = [120.0, 150.0][rank]
    rays = [1.0e9, 2.0e9][rank]
    paths = [3.0e8, 4.0e8][rank]
    out = bench.reduce_replicas(ms, rays, paths, world, torch.device("cpu"))
    q.put((rank, out))
    dist.barrier()
    dist.destroy_process_group()


def test_replica_reduction_two_ranks():
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = dict(q.get(timeout=120) for _ in range(2))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for r in range(2):
        assert res[r] == (150.0, 3.0e9, 7.0e8)


def test_single_rank_is_identity():
    import bench

    assert bench.reduce_replicas(5.0, 6.0, 7.0, 1, None) == (5.0, 6.0, 7.0)
