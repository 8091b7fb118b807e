"""The N > 1 path of bench.py on CPU: world-size-2 gloo ranks (127.0.0.1).
Every GPU machine has one GPU and the path runs replicas only, so what needs
covering is the host logic: the max-over-ranks time, the whole-job
aggregate, and the reference arm running on rank 0 alone."""
import argparse
import contextlib
import io
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


def _rank_main(rank, world, port, out):
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        # slowest replica wins
        t = bench.max_over_ranks(10.0 * (rank + 1), dist, "cpu")
        # the reference arm: rank 0 alone does work and prints; others return at once
        printed = io.StringIO()
        if rank != 0:
            with contextlib.redirect_stdout(printed):
                bench.run_reference(argparse.Namespace(steps=1, warmup=0))
        dist.barrier()
        out[rank] = (t, printed.getvalue())
    finally:
        dist.destroy_process_group()


@pytest.mark.timeout(120)
def test_two_gloo_ranks_max_time_and_rank0_only_reference():
    world = 2
    mgr = mp.get_context("spawn").Manager()
    out = mgr.dict()
    mp.start_processes(_rank_main, args=(world, _free_port(), out), nprocs=world, start_method="spawn")
    assert out[0][0] == 20.0 and out[1][0] == 20.0
    assert out[1][1] == ""


def test_whole_job_aggregate_is_weak_scaling():
    sys.path.insert(0, ROOT)
    import bench
    one = bench.whole_job_gbs(1, 2_147_483_648, 10, 0.01)
    assert abs(bench.whole_job_gbs(4, 2_147_483_648, 10, 0.01) - 4 * one) < 1e-6
    # the aggregate uses the slowest replica's time
    assert bench.whole_job_gbs(2, 100, 1, 2.0) == 2 * 100 / 2.0 / 1e9
