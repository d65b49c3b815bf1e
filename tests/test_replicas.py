"""The multi-GPU path of bench.py is replicas only: each rank deconvolves independently and
the job's throughput is all ranks' voxel-updates over the slowest rank's time.  This checks
that host logic with two gloo ranks on the CPU (no GPU, no data-path collective)."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, times, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench

    ms = bench.max_over_ranks(times[rank], world)
    value = bench.replica_value(1000.0, ms, world)
    out[rank] = (ms, value)
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_replicas_take_the_slowest_rank():
    world = 2
    times = [40.0, 50.0]
    with mp.get_context("spawn").Manager() as m:  # no fork from this multi-threaded process
        out = m.dict()
        mp.spawn(_worker, args=(world, _free_port(), times, out), nprocs=world, join=True)
        res = dict(out)
    for r in range(world):
        ms, value = res[r]
        assert ms == 50.0
        assert value == pytest.approx(1000.0 * world / 0.050)


def test_single_rank_needs_no_process_group():
    import bench

    assert bench.max_over_ranks(12.5, 1) == 12.5
    assert bench.replica_value(10.0, 1000.0, 1) == pytest.approx(10.0)
