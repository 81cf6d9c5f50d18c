"""Multi-rank logic of the benchmark on CPU (gloo, world size 2): every rank
assembles its own replica, so the only cross-rank step is the reduction of
the timings to the slowest rank."""
import os
import socket
import sys

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as tdist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import bench

    tdist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        out[rank] = bench.reduce_max(1.5 + rank, world, device="cpu")
        tdist.barrier()
    finally:
        tdist.destroy_process_group()


def test_timing_reduction_takes_the_slowest_rank():
    world = 2
    ctx = mp.get_context("spawn")
    with ctx.Manager() as manager:
        out = manager.dict()
        mp.start_processes(_rank_main, args=(world, _free_port(), out), nprocs=world, start_method="spawn", join=True)
        assert dict(out) == {0: 2.5, 1: 2.5}


def test_single_rank_is_identity():
    sys.path.insert(0, ROOT)
    import bench

    assert bench.reduce_max(3.25, 1) == 3.25
