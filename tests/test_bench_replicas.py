"""bench.py's N > 1 path (replicas only: one independent sigma per rank, no
data-path collective) on two gloo ranks on the CPU: every rank ends with the
slowest rank's step times, and the whole-job throughput counts both ranks'
work."""
import os
import sys

import pytest
import torch.multiprocessing as mp

from conftest import ROOT


def _rank(rank, world, port, out):
    import torch.distributed as dist

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import bench

    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        # rank r took (1 + r) ms per step and (2 + r) ms end to end
        res = bench.whole_job(1e9, 1e-3 * (1 + rank), 1e-3 * (2 + rank), dist, device="cpu")
        out[rank] = res
    finally:
        dist.destroy_process_group()


def test_replicas_take_the_slowest_rank():
    pytest.importorskip("torch.distributed")
    port = 29500 + os.getpid() % 1000
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(_rank, args=(2, port, out), nprocs=2, join=True)
        res = dict(out)
    for r in (0, 1):
        t_step, t_e2e, value, e2e = res[r]
        assert t_step == pytest.approx(2e-3) and t_e2e == pytest.approx(3e-3)
        assert value == pytest.approx(2 * 1e9 / 2e-3 / 1e12)
        assert e2e == pytest.approx(2 * 1e9 / 3e-3 / 1e12)


def test_single_process_whole_job():
    sys.path.insert(0, ROOT)
    import bench

    assert bench.whole_job(1e9, 1e-3, 2e-3) == (1e-3, 2e-3, 1.0, 0.5)
