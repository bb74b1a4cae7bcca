"""The N>1 host path of bench.py on CPU gloo ranks (world size 2): the max-over-ranks time and the
whole-job rate every rank derives from it.  No GPU is involved."""

import os
import socket

import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        import bench

        ms = bench.max_over_ranks(10.0 + 5.0 * rank, dist)  # rank 1 is the slow one
        rate = bench.whole_job_rate(1000, world, 4, ms)
        out.put((rank, ms, rate))
        dist.barrier()
    finally:
        dist.destroy_process_group()


@pytest.mark.timeout(120)
def test_bench_reduces_the_slowest_rank_over_gloo():
    world = 2
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=90) for _ in range(world))
    for p in procs:
        p.join(timeout=30)
        assert p.exitcode == 0
    assert [r[1] for r in res] == [15.0, 15.0]
    assert all(abs(r[2] - 2 * 1000 * 4 / 15e-3) < 1e-6 for r in res)


def test_bench_reduction_without_a_process_group():
    import bench

    assert bench.max_over_ranks(3.5) == 3.5
    assert bench.whole_job_rate(10, 1, 2, 1.0) == 20000.0
