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


def test_reference_arm_under_two_ranks_prints_one_line():
    """`bench.py --impl reference` launched as two ranks (as the scaling runs
    launch it): rank 0 alone runs the CPU oracle and prints the one JSON line,
    rank 1 exits 0 without work."""
    import json
    import subprocess

    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node=2",
           "--master-addr", "127.0.0.1", "--master-port", str(_free_port()),
           os.path.join(ROOT, "bench.py"), "--impl", "reference", "--gpus", "2", "--cells", "6", "--steps", "1",
           "--warmup", "1"]
    out = subprocess.run(cmd, capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [ln for ln in out.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, out.stdout
    line = json.loads(lines[0])
    assert line["impl"] == "reference" and line["n_gpus"] == 2 and line["value"] > 0
    assert line["cpu_baseline"]["kind"] == "port" and line["cpu_baseline"]["one_thread"]["value"] > 0
