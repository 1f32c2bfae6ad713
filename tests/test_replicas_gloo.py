"""Replica aggregation of bench.py on CPU: two gloo ranks, each with its own step time; the
reported step time is the maximum over ranks and the throughput counts every rank's rays."""
import os
import socket

import pytest
import torch.multiprocessing as mp


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def rank_main(rank, world, port, out):
    import sys
    import torch
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import bench
    dist.init_process_group("gloo", init_method="env://")
    ms, value = bench.replica_throughput(2.0 + rank, 1_000_000, world, torch.device("cpu"))
    out.put((rank, ms, value))
    dist.barrier()
    dist.destroy_process_group()


def test_two_replicas_max_time_and_summed_rays():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = free_port()
    procs = [ctx.Process(target=rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for _, ms, value in res:
        assert ms == pytest.approx(3.0)
        assert value == pytest.approx(2 * 1_000_000 / 3.0e-3 / 1e6)


def test_single_replica_is_plain_ratio():
    import bench
    import torch
    ms, value = bench.replica_throughput(2.5, 5_000_000, 1, torch.device("cpu"))
    assert ms == 2.5 and value == pytest.approx(5_000_000 / 2.5e-3 / 1e6)
