"""The multi-rank path of bench.py on CPU: two gloo ranks time different
amounts, both report the slowest, and the job throughput counts both
replicas (weak scaling, no data-path collective)."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _rank(rank, world, port, out):
    import torch
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    ms = bench.max_over_ranks(100.0 + 50.0 * rank, torch.device("cpu"), world)
    out[rank] = (ms, bench.replicas_glups(world, 1000, 10, ms))
    dist.destroy_process_group()


def test_two_gloo_ranks_report_the_slowest():
    import torch.multiprocessing as mp
    port = 29500 + os.getpid() % 1000
    with mp.Manager() as m:
        out = m.dict()
        mp.start_processes(_rank, args=(2, port, out), nprocs=2, start_method="spawn")
        res = dict(out)
    assert res[0] == res[1]
    ms, v = res[0]
    assert ms == 150.0
    assert v == pytest.approx(2 * 1000 * 10 / 0.150 / 1e9)
