"""bench.py with N > 1 ranks: every rank runs its own replica (the path does
not shard) and the job's throughput is all ranks' cell-steps over the
slowest rank's time. The host logic runs here as two gloo ranks on the CPU:
the max over ranks, the whole-job value, and the reference arm, which only
rank 0 runs."""
import io
import os
import socket
import sys
from contextlib import redirect_stdout

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port),
                      RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        import bench
        # rank r took 10 + 5 r ms: the job took the slowest rank's 15 ms
        ms = bench.max_over_ranks(10.0 + 5.0 * rank, dist, "cpu")
        value = bench.job_value(1 << 20, 20000, 5, world, ms * 1e-3)
        # the reference arm: rank 0 alone runs it and prints one line
        class Args:
            gpus, steps, warmup = world, 1, 0
        from yolohtli_gb300 import workloads as W
        wl = W.fk_holes_1024(n=64, nsteps=8, nholes=2, npatch=1)
        buf = io.StringIO()
        if rank != 0:
            with redirect_stdout(buf):
                bench.run_reference(Args, wl)
        out[rank] = (ms, value, buf.getvalue())
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_aggregate_as_one_job():
    world = 2
    out = mp.Manager().dict()
    mp.spawn(_rank_main, args=(world, _free_port(), out), nprocs=world,
             join=True)
    for r in range(world):
        ms, value, printed = out[r]
        assert ms == 15.0
        # 2 replicas x 2^20 cells x 20,000 steps x 5 solves in 15 ms
        assert value == pytest.approx(2 * (1 << 20) * 20000 * 5 / 15e-3 / 1e9)
    assert out[1][2] == ""  # a rank other than 0 prints nothing


def test_one_rank_without_a_process_group():
    import bench
    assert bench.max_over_ranks(7.5, None, "cpu") == 7.5
    assert bench.job_value(100, 10, 2, 1, 2.0) == pytest.approx(1e-6)
