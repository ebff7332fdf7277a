"""bench.py's multi-rank host logic on CPU (gloo, world size 2): each rank
times its own replica; the job's time is the slowest rank's, and the
reported value is the units all ranks processed over that time.  The
reference arm runs on rank 0 alone; the other ranks exit without work."""
import os
import socket
import sys

import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, times, out):
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        t = bench.max_over_ranks(times[rank], dist, device="cpu")
        out.put((rank, t, bench.aggregate_value(1000 * 20, t, world)))
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_slowest_rank_sets_the_job_time():
    ctx = mp.get_context("spawn")
    out = ctx.Queue()
    times = [0.5, 0.75]
    mp.start_processes(_rank, args=(2, _free_port(), times, out), nprocs=2, start_method="spawn")
    got = sorted(out.get(timeout=60) for _ in range(2))
    for rank, t, value in got:
        assert t == 0.75
        assert value == pytest.approx(2 * 1000 * 20 / 0.75 / 1e6)


def test_single_process_is_its_own_maximum():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(1.25, None) == 1.25
    assert bench.aggregate_value(998_400 * 100, 0.0827, 1) == pytest.approx(998_400 * 100 / 0.0827 / 1e6)


def test_reference_arm_other_ranks_exit_without_work(capsys):
    sys.path.insert(0, ROOT)
    import argparse
    import bench
    args = argparse.Namespace(workload="c1_3d_evp", steps=1, warmup=3, gpus=2)
    assert bench.run_reference(args, 1, 2) == 0
    assert capsys.readouterr().out == ""
