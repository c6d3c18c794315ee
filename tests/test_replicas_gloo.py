"""Replicas on several ranks (bench.py --gpus N under torchrun): every rank
estimates its own instance, the timed region is the slowest rank's and the
value counts the path steps of all ranks.  Checked here with two gloo ranks
on the CPU through the same helper bench.py calls under NCCL."""
import os
import socket
import sys

import pytest

torch = pytest.importorskip("torch")
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        # rank r: timed region 1.5 + r seconds, 1000 (r + 1) path steps
        t, units = bench.aggregate_ranks(1.5 + rank, 1000 * (rank + 1), dist, "cpu")
        dist.barrier()
        out.put((rank, t, units))
    finally:
        dist.destroy_process_group()


def test_two_replicas_take_the_slowest_time_and_all_units():
    ctx = mp.get_context("spawn")
    out = ctx.Queue()
    world, port = 2, _free_port()
    procs = [ctx.Process(target=_rank, args=(r, world, port, out)) for r in range(world)]
    for p in procs:
        p.start()
    res = sorted(out.get(timeout=120) for _ in range(world))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, t, units in res:
        assert t == 2.5 and units == 3000.0, (rank, t, units)


def test_one_process_passes_through():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.aggregate_ranks(2.0, 7, None, "cpu") == (2.0, 7.0)
