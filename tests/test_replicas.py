"""Multi-process host logic of bench.py's replica mode, on CPU with gloo
(world size 2): every rank renders its own frame, the timed value is the
slowest rank's time, and the whole-job rate counts all ranks' paths.  Also:
the CPU reference arm prints only on rank 0 and other ranks exit without
work."""
import os
import socket
import sys

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    sys.path.insert(0, ROOT)
    import bench

    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        ms = [31.5, 33.25][rank]
        m = bench.reduce_max(ms, dist, "cpu")
        out[rank] = (m, bench.whole_job_rate(2048, world, m / 1000.0))
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_replica_max_and_rate():
    world = 2
    mgr = mp.get_context("spawn").Manager()
    out = mgr.dict()
    mp.start_processes(_worker, args=(world, _free_port(), out), nprocs=world, start_method="spawn", join=True)
    assert out[0][0] == out[1][0] == 33.25
    assert abs(out[0][1] - 2048 * 2 / 0.03325) < 1e-6
    assert out[0] == out[1]


def test_reference_arm_rank_nonzero_does_nothing(capsys):
    sys.path.insert(0, ROOT)
    import bench

    class A:
        warmup, steps, size, paths, gpus = 1, 1, 64, 64, 2

    assert bench.run_reference(A, 1) is None
    assert capsys.readouterr().out == ""


def test_single_process_reduce_is_identity():
    sys.path.insert(0, ROOT)
    import bench

    assert bench.reduce_max(12.5, None, "cpu") == 12.5
    assert bench.whole_job_rate(100, 1, 0.5) == 200.0
