"""The N>1 host path on CPU gloo ranks (world size 2): bench.py's max-over-ranks time and the
whole-job rate every rank derives from it, and the instance sharding of an ensemble
(direbm_gb300/shard.py): the balanced partition and the gather of every shard's state.  No GPU is
involved."""

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
        total = bench.sum_over_ranks(1000 + 500 * rank, dist)  # the shards' moments
        rate = bench.whole_job_rate(int(total), 4, ms)
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
    assert all(abs(r[2] - 2500 * 4 / 15e-3) < 1e-6 for r in res)


def test_bench_reduction_without_a_process_group():
    import bench

    assert bench.max_over_ranks(3.5) == 3.5
    assert bench.sum_over_ranks(7.0) == 7.0
    assert bench.whole_job_rate(10, 2, 1.0) == 20000.0


def test_bench_recognises_moments_in_cell_order():
    """The e2e leg loads its ensemble with presorted=True only when the moments are ordered by
    instance, then cell row, then cell column (the device checks the order as well)."""
    import numpy as np

    import bench

    sides, taus = bench.ensemble_spec(3)
    ib, x, f = bench.build_ensemble(sides, taus)
    assert bench.in_cell_order(ib, x)
    perm = np.random.default_rng(0).permutation(len(x))
    assert not bench.in_cell_order(ib[perm], x[perm])
    swapped = x.copy()
    swapped[[0, 1]] = swapped[[1, 0]]  # two neighbours of the first row, out of column order
    assert not bench.in_cell_order(ib, swapped)
    assert bench.in_cell_order(ib[:1], x[:1])


# ---- instance sharding (direbm_gb300/shard.py) ----------------------------------------------------

def test_partition_is_balanced_deterministic_and_complete():
    import numpy as np

    from direbm_gb300.shard import partition

    rng = np.random.default_rng(1)
    w = np.round(np.exp(rng.uniform(np.log(4096), np.log(262144), 256))).astype(np.int64)
    for world in (1, 2, 3, 4, 8):
        groups = partition(w, world)
        assert len(groups) == world
        allm = np.sort(np.concatenate(groups))
        np.testing.assert_array_equal(allm, np.arange(len(w)))  # every instance exactly once
        loads = np.array([w[g].sum() for g in groups])
        assert loads.max() <= w.sum() / world + w.max()  # greedy bound
        assert loads.max() <= 4.0 / 3.0 * max(w.sum() / world, w.max()) + 1
        for g, h in zip(groups, partition(w, world)):
            np.testing.assert_array_equal(g, h)
    # more ranks than instances: some ranks hold nothing
    groups = partition([5, 3], 4)
    assert [len(g) for g in groups] == [1, 1, 0, 0]


def test_local_rows_renumbers_members():
    import numpy as np

    from direbm_gb300.shard import local_rows

    inst = np.array([0, 0, 1, 2, 2, 2, 3])
    rows, local = local_rows(inst, np.array([1, 3]))
    np.testing.assert_array_equal(rows, [2, 6])
    np.testing.assert_array_equal(local, [0, 1])


def _gather_rank(rank, world, port, out):
    import numpy as np

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        from direbm_gb300.shard import gather_state, local_rows, max_over_ranks, partition

        # a global state: 5 instances of uneven sizes, rows instance-major
        sizes = [7, 3, 11, 2, 5]
        inst = np.repeat(np.arange(5), sizes)
        pos = np.stack([np.arange(len(inst), dtype=np.float64), -np.arange(len(inst), dtype=np.float64)], 1)
        f = np.arange(len(inst) * 9, dtype=np.float64).reshape(-1, 9)
        members = partition(sizes, world)[rank]
        rows, local = local_rows(inst, members)
        got = gather_state(torch.as_tensor(local), torch.as_tensor(pos[rows]), torch.as_tensor(f[rows]), members)
        slow = max_over_ranks(1.0 + rank)
        if rank == 0:
            gi, gp, gf = (t.numpy() for t in got)
            out.put((rank, gi.tolist(), bool(np.array_equal(gp, pos)), bool(np.array_equal(gf, f)), slow))
        else:
            out.put((rank, got is None, None, None, slow))
        dist.barrier()
    finally:
        dist.destroy_process_group()


@pytest.mark.timeout(120)
def test_gather_state_reassembles_the_ensemble_over_gloo():
    import numpy as np

    world = 2
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_gather_rank, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=90) for _ in range(world))
    for p in procs:
        p.join(timeout=30)
        assert p.exitcode == 0
    r0, r1 = res
    assert r0[1] == np.repeat(np.arange(5), [7, 3, 11, 2, 5]).tolist()
    assert r0[2] and r0[3]  # positions and f come back row for row
    assert r1[1] is True  # only the destination rank receives
    assert r0[4] == r1[4] == 2.0
