"""The bench's multi-rank logic on CPU ranks (gloo, world size 2): the barrier
and the max over ranks that the timed region uses, the rank-0-only
reference arm, and the replicas' whole-job value.  Each GPU rank runs its own
replica of the workload (the path has no exchange step), so nothing else
crosses ranks."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank_main(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        import bench
        bench._barrier(world)
        # each rank times a different step; every rank reports the slowest
        got = bench._max_over_ranks(10.0 + 5.0 * rank, world)
        # the reference arm runs on rank 0 alone: other ranks return at once
        if rank != 0:
            bench.run_reference(None, rank, world)
        bench._barrier(world)
        out[rank] = got
    finally:
        dist.destroy_process_group()


def test_barrier_and_max_over_two_gloo_ranks():
    world = 2
    mgr = mp.get_context("spawn").Manager()
    out = mgr.dict()
    mp.start_processes(_rank_main, args=(world, _free_port(), out), nprocs=world, start_method="spawn", join=True)
    assert dict(out) == {0: 15.0, 1: 15.0}


def test_single_rank_helpers_are_identity():
    import bench
    bench._barrier(1)
    assert bench._max_over_ranks(3.5, 1) == 3.5
