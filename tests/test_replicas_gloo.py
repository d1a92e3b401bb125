"""Replica aggregation of bench.py under torch.distributed, two gloo ranks on CPU.

Chains are independent (replicas only): every rank sweeps its own chains and
the whole-job throughput is all ranks' chain-sweeps over the slowest rank's
time.  The GPU timing itself needs CUDA; the reduction logic is tested here.
"""
import os
import sys
from pathlib import Path

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

ROOT = Path(__file__).resolve().parent.parent


def _rank(rank, world, port, out):
    sys.path.insert(0, str(ROOT))
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    ms_local = 1000.0 + 500.0 * rank           # rank 1 is the slow one
    units, ms = bench.replica_throughput(dist, ms_local, 256 * 20)
    out[rank] = (units, ms, bench.dist_max(dist, float(rank)))
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_replica_throughput():
    world, port = 2, 29000 + os.getpid() % 1000
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(_rank, args=(world, port, out), nprocs=world, join=True)
        res = dict(out)
    for r in range(world):
        units, ms, mx = res[r]
        assert ms == 1500.0                     # max over ranks
        assert units == pytest.approx(2 * 256 * 20 / 1.5)
        assert mx == 1.0


def test_single_process_is_identity():
    sys.path.insert(0, str(ROOT))
    import bench
    units, ms = bench.replica_throughput(None, 2000.0, 100)
    assert ms == 2000.0 and units == pytest.approx(50.0)
