"""The multi-GPU path of bench.py runs independent replicas (the apply and the
solves do not shard across GPUs here): every rank times its own workload and
the reported step time is the maximum over ranks.  This checks that
aggregation with two gloo ranks on the CPU (127.0.0.1 rendezvous)."""
import os
import socket
import sys

import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import torch
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        ms, per_s = bench.replica_throughput(1.0 + rank, 1000, world, torch.device("cpu"))
        out[rank] = (ms, per_s)
    finally:
        dist.destroy_process_group()


@pytest.mark.timeout(120)
def test_two_gloo_ranks_take_the_slowest_step():
    world = 2
    ctx = mp.get_context("spawn")
    out = ctx.Manager().dict()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, world, port, out)) for r in range(world)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(100)
        assert p.exitcode == 0
    for r in range(world):
        ms, per_s = out[r]
        assert ms == 2.0                      # max over ranks
        assert per_s == world * 1000 / 2e-3   # whole-job units per second


def test_single_rank_needs_no_process_group():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.replica_throughput(4.0, 10, 1, None) == (4.0, 10 / 4e-3)
