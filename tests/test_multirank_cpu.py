"""bench.py's multi-GPU bookkeeping with two CPU ranks over gloo.

On N GPUs every rank advances its own replica of the grid (the path does not
shard), the job time is the maximum over ranks and the value counts every
rank's points.  These tests run that logic with world_size 2 on the CPU.
"""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank(rank, world, port, out):
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    w, r, local = bench.dist_setup()
    assert (w, r, local) == (world, rank, rank)
    seconds = 1.0 + rank  # rank 1 is the slow one
    job = bench.max_over_ranks(seconds, True, "cpu")
    out[rank] = (job, bench.job_value(1000000, 10, w, job))
    dist.barrier()
    dist.destroy_process_group()


def test_two_ranks_take_the_slowest_and_count_all_points():
    port = _free_port()
    out = mp.get_context("spawn").Manager().dict()   # no fork of this multi-threaded process
    mp.spawn(_rank, args=(2, port, out), nprocs=2, join=True)
    assert out[0] == out[1]
    job, value = out[0]
    assert job == 2.0
    assert value == pytest.approx(1e6 * 10 * 2 / 2.0 / 1e6)


def test_single_rank_needs_no_process_group():
    import bench
    assert bench.max_over_ranks(3.5, False) == 3.5
    assert bench.job_value(256 ** 3, 10, 1, 1.0) == pytest.approx(167.77216)
