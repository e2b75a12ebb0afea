"""The bench's multi-rank timing (replicas: barrier, max over ranks, whole-job
rate) on two CPU processes with the gloo backend."""
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


def _worker(rank, world, port, out):
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        seconds = 1.0 + rank  # rank 1 is the slow one
        slowest = bench.max_over_ranks(seconds, world, "cpu")
        rate = bench.aggregate_rate(world, 1000.0, slowest)
        dist.barrier()
        out[rank] = (slowest, rate)
    finally:
        dist.destroy_process_group()


def test_max_over_ranks_and_aggregate_rate_two_ranks():
    ctx = mp.get_context("spawn")
    with ctx.Manager() as m:
        out = m.dict()
        port = _free_port()
        procs = [ctx.Process(target=_worker, args=(r, 2, port, out)) for r in range(2)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(120)
            assert p.exitcode == 0
        for r in range(2):
            slowest, rate = out[r]
            assert slowest == 2.0              # every rank sees the slowest rank's time
            assert rate == 2 * 1000.0 / 2.0    # both replicas' work over that time


def test_single_rank_is_identity():
    import bench
    assert bench.max_over_ranks(3.5, 1) == 3.5
    assert bench.aggregate_rate(1, 10.0, 2.0) == 5.0
