"""The multi-GPU path of bench.py is replicas only (independent reconstructions, no data-path collective): timing is
the maximum over ranks and the value is the whole job's reconstructions over that time. Checked with two gloo ranks
on the CPU."""
import os
import sys

import pytest
import torch.multiprocessing as mp

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _rank(rank, world, port, out):
    import torch
    import torch.distributed as dist

    sys.path.insert(0, REPO)
    import bench

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    ms = bench.max_over_ranks(10.0 + 5.0 * rank, world, torch.device("cpu"))
    value = bench.replica_throughput(64, world, ms * 1e-3)
    cfg = bench.config(type("A", (), {"n": 8, "batch": 64})(), world)
    out.put((rank, ms, value, cfg["global_batch"], cfg["parallelism"]))
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_replica_timing():
    world, port = 2, 29611
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in range(world))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, ms, value, gb, par in res:
        assert ms == pytest.approx(15.0)  # the slower rank's time on every rank
        assert value == pytest.approx(64 * 2 / 15e-3)
        assert gb == 128 and par == "replicas x2"
