"""CPU test of the replica path of bench.py (N > 1): every rank times its own replica, the
job time is the max over ranks and the value counts all ranks' atoms (gloo, 2 ranks)."""
import os
import sys

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _worker(rank, world, port, out):
    sys.path.insert(0, ROOT)
    import bench
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    ms = 100.0 + 50.0 * rank                   # rank 1 is the slow one
    m = bench.reduce_max(ms, dist)
    v = bench.replica_value(1000, 10, m, world)
    out[rank] = (m, v)
    dist.barrier()
    dist.destroy_process_group()


def test_replica_aggregation_two_ranks():
    import random
    port = 29500 + random.randint(0, 2000)
    mgr = mp.get_context("spawn").Manager()          # no fork of a threaded process
    out = mgr.dict()
    mp.spawn(_worker, args=(2, port, out), nprocs=2, join=True)
    for r in range(2):
        m, v = out[r]
        assert m == 150.0
        assert v == pytest.approx(2 * 1000 * 10 / 0.150)


def test_reduce_max_without_group():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.reduce_max(3.5, None) == 3.5
