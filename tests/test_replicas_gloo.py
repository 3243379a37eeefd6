"""Replicas-only multi-GPU aggregation (bench.py), exercised with two gloo ranks on
the CPU: the job time is the slowest rank's, the work is the sum over ranks."""
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    import sys
    from pathlib import Path

    sys.path.insert(0, str(Path(__file__).resolve().parents[1]))
    import torch.distributed as dist

    import bench

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    ms, e2e, units = bench.aggregate_replicas(10.0 + rank, 20.0 - rank, 1000.0 * (rank + 1))
    q.put((rank, ms, e2e, units))
    dist.destroy_process_group()


def test_two_rank_aggregation():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    out = sorted(q.get(timeout=10) for _ in range(2))
    for rank, ms, e2e, units in out:
        assert (ms, e2e, units) == (11.0, 20.0, 3000.0)


def test_single_process_passthrough():
    import bench

    assert bench.aggregate_replicas(1.5, 2.5, 7.0) == (1.5, 2.5, 7.0)
