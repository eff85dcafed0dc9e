"""The multi-GPU form of the bench is replicas only (each rank trains its own copy of
the workload; the ADMM needs no exchange between replicas): two gloo ranks on the CPU
check the host logic -- the slowest rank's time is what every rank reports, and the
whole-job rate counts every replica's iterations."""
import os
import sys

import pytest
import torch.distributed as dist
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _rank(rank, world, port, out):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    sys.path.insert(0, ROOT)
    import bench
    ms_max = bench.max_over_ranks(100.0 + 50.0 * rank, world, "cpu")
    out[rank] = (ms_max, bench.replica_rate(world, 10, ms_max / 1e3))
    dist.barrier()
    dist.destroy_process_group()


def test_two_replicas_report_the_slowest_rank():
    pytest.importorskip("torch")
    port = 29500 + os.getpid() % 1000
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(_rank, args=(2, port, out), nprocs=2, join=True)
        res = dict(out)
    assert res[0] == res[1] == (150.0, pytest.approx(2 * 10 / 0.150))
