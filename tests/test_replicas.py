"""The N > 1 path of bench.py on CPU: world-size-2 gloo ranks, each a
replica with its own step time; the job time is the slowest rank's and the
whole-job value counts every rank's views."""

import os
import sys

import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _rank(rank, world, port, q):
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench

    ms = bench.job_time_ms(1000.0 + 500.0 * rank, world, torch.device("cpu"))
    dist.barrier()
    q.put((rank, ms, world * 20 / (ms / 1000.0)))
    dist.destroy_process_group()


def test_job_time_is_max_over_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29500 + os.getpid() % 1000
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
    assert all(p.exitcode == 0 for p in procs)
    res = sorted(q.get(timeout=5) for _ in range(2))
    assert [r[1] for r in res] == [1500.0, 1500.0]
    assert res[0][2] == pytest.approx(2 * 20 / 1.5)


def test_single_rank_is_local_time():
    import importlib

    sys.path.insert(0, ROOT)
    bench = importlib.import_module("bench")
    assert bench.job_time_ms(12.5, 1, torch.device("cpu")) == 12.5
