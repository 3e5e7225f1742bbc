"""bench.py's multi-rank path (replicas: every rank runs its own copy of the
workload, weak scaling, no data-path collective) on the CPU with two gloo
ranks: the max-over-ranks of a timed region, the barrier, the rank
environment, and that only rank 0 runs the reference arm."""
import argparse
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


def _rank_main(rank, world, port, q):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import bench

    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        r, w, l = bench.dist_env()
        bench.barrier_all(w)
        longest = bench.max_over_ranks(10.0 * (r + 1), w)  # rank r timed 10 (r + 1) ms
        bench.barrier_all(w)
        # whole-job frames/s as bench computes it: frames of every rank over the slowest rank
        fps = w * 100 / (longest / 1000.0)
        ran_reference = None
        if r != 0:
            args = argparse.Namespace(steps=1, warmup=0, gpus=w, sessions=2, ref_seconds=0.1)
            ran_reference = bench.run_reference(args)  # rank != 0: returns at once, prints nothing
        q.put((r, w, l, longest, fps, ran_reference))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_take_the_max_and_only_rank0_reports():
    ctx = mp.get_context("spawn")
    q = ctx.SimpleQueue()
    port = _free_port()
    mp.start_processes(_rank_main, args=(2, port, q), nprocs=2, join=True, start_method="spawn")
    got = sorted(q.get() for _ in range(2))
    assert [g[0] for g in got] == [0, 1]
    for r, w, l, longest, fps, ref in got:
        assert w == 2 and l == r
        assert longest == 20.0  # every rank sees the slowest rank's time
        assert fps == pytest.approx(2 * 100 / 0.020)
    assert got[1][5] is None
