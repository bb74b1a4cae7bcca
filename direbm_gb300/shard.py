"""Instance sharding of a batched ensemble across ranks (one process per GPU).

The instances of an ensemble are independent: every interaction of the DiReBM step (dispersion by
c_k dx, thinning, refine and resampling within r) stays inside its instance.  An ensemble
therefore shards by instance with no exchange during the steps.  Each rank advances the
instances assigned to it in its own ``Simulation``; the host gathers states and counts when asked.

``partition`` balances the ranks by point count (the step's cost is linear in the moments):
longest-processing-time-first greedy assignment, so the largest rank load is at most 4/3 of the
optimum (and at most the average plus the largest instance).  It is deterministic.

``gather_state`` brings every rank's state to rank ``dst`` in global instance order.  It is plain
tensor communication (an all-gather of counts, then of row blocks padded to the largest count),
so it runs on NCCL with CUDA tensors and on gloo with host tensors.

The reference has no multi-GPU path: its GpuSimulator runs one domain on one device
(direbm/warp/simulator.py:25-77).
"""

from __future__ import annotations

import numpy as np
import torch


def partition(weights, world: int) -> list[np.ndarray]:
    """Split instance indices 0..len(weights)-1 into `world` groups of near-equal total weight.

    Instances are taken in decreasing weight (ties by index) and each goes to the rank with the
    smallest load so far (ties by rank).  Each group comes back sorted by instance index."""
    w = np.asarray(weights, dtype=np.int64)
    if world < 1:
        raise ValueError("partition: world must be >= 1")
    if (w < 0).any():
        raise ValueError("partition: weights must be non-negative")
    order = sorted(range(len(w)), key=lambda i: (-int(w[i]), i))
    load = [0] * world
    groups: list[list[int]] = [[] for _ in range(world)]
    for i in order:
        r = min(range(world), key=lambda k: (load[k], k))
        groups[r].append(i)
        load[r] += int(w[i])
    return [np.array(sorted(g), dtype=np.int64) for g in groups]


def local_rows(inst: np.ndarray, members: np.ndarray):
    """Rows of a global state (instance index per row) that belong to `members`, and those rows'
    instance indices renumbered 0..len(members)-1 in the order of `members`."""
    inst = np.asarray(inst, dtype=np.int64)
    members = np.asarray(members, dtype=np.int64)
    lut = np.full(int(max(inst.max(initial=-1), members.max(initial=-1))) + 1, -1, dtype=np.int64)
    lut[members] = np.arange(len(members))
    local = lut[inst] if len(inst) else np.zeros(0, np.int64)
    rows = np.flatnonzero(local >= 0)
    return rows, local[rows].astype(np.int32)


def _all_gather_rows(x: torch.Tensor, counts: list[int], group=None) -> list[torch.Tensor]:
    import torch.distributed as dist

    world = len(counts)
    n = max(counts) if counts else 0
    pad = torch.zeros((n,) + tuple(x.shape[1:]), dtype=x.dtype, device=x.device)
    pad[: x.shape[0]] = x
    bufs = [torch.empty_like(pad) for _ in range(world)]
    dist.all_gather(bufs, pad, group=group)
    return [b[:c] for b, c in zip(bufs, counts)]


def gather_state(inst: torch.Tensor, pos: torch.Tensor, f: torch.Tensor, members, group=None, dst: int = 0):
    """Every rank's state (local instance indices, positions, f) to rank `dst`, with the local
    indices mapped back to global ones through each rank's `members`; rows are ordered by global
    instance, each instance's rows in the order its rank holds them.  Returns (inst, pos, f) on
    `dst` and None elsewhere.  Collective: every rank of the group calls it."""
    import torch.distributed as dist

    world = dist.get_world_size(group)
    rank = dist.get_rank(group)
    dev = pos.device
    cnt = torch.tensor([int(inst.shape[0])], dtype=torch.int64, device=dev)
    cnts = [torch.zeros_like(cnt) for _ in range(world)]
    dist.all_gather(cnts, cnt, group=group)
    counts = [int(c.item()) for c in cnts]
    mem = torch.as_tensor(np.asarray(members, dtype=np.int64), device=dev)
    nm = torch.tensor([int(mem.shape[0])], dtype=torch.int64, device=dev)
    nms = [torch.zeros_like(nm) for _ in range(world)]
    dist.all_gather(nms, nm, group=group)
    mems = _all_gather_rows(mem, [int(v.item()) for v in nms], group)
    gi = [m[i.long()] for m, i in zip(mems, _all_gather_rows(inst.to(torch.int64), counts, group))]
    gp = _all_gather_rows(pos, counts, group)
    gf = _all_gather_rows(f, counts, group)
    if rank != dst:
        return None
    gi, gp, gf = torch.cat(gi), torch.cat(gp), torch.cat(gf)
    order = torch.sort(gi, stable=True).indices
    return gi[order].to(torch.int32), gp[order], gf[order]


def max_over_ranks(value: float, group=None) -> float:
    """The largest of a per-rank float (the slowest rank's time); the value itself without a
    process group."""
    import torch.distributed as dist

    if not dist.is_available() or not dist.is_initialized():
        return float(value)
    dev = "cuda" if dist.get_backend(group) == "nccl" else "cpu"
    t = torch.tensor([float(value)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX, group=group)
    return float(t.item())


class ShardedEnsemble:
    """This rank's share of a batched ensemble: a ``Simulation`` over the instances that
    ``partition`` assigns to it (by cell count), loaded from the global initial state.

    ``instances`` is the global list of ``Instance``; ``inst, pos, f`` the global initial state
    (host arrays).  Keyword arguments go to ``Simulation``.  ``step`` advances the local shard with
    no communication; ``gather`` brings the whole ensemble's state to rank 0."""

    def __init__(self, instances, inst, pos, f, rank: int, world: int, group=None, weights=None, **sim_kw):
        from .sim import Simulation

        if weights is None:
            weights = [int(np.prod(i.dims)) for i in instances]
        self.members = partition(weights, world)[rank]
        self.rank, self.world, self.group = rank, world, group
        rows, local = local_rows(inst, self.members)
        self.moments = int(len(rows))
        cap = sim_kw.pop("moment_capacity", None)
        self.sim = Simulation([instances[i] for i in self.members], moment_capacity=cap or max(self.moments, 1),
                              **sim_kw)
        self.sim.set_state(local, np.asarray(pos)[rows], np.asarray(f)[rows])

    def step(self, n: int = 1):
        self.sim.step(n)

    def gather(self, dst: int = 0):
        inst, pos, f = self.sim.state()
        if self.world == 1:
            return torch.as_tensor(self.members, device=inst.device)[inst.long()].to(torch.int32), pos, f
        import torch.distributed as dist

        if dist.get_backend(self.group) != "nccl":
            inst, pos, f = inst.cpu(), pos.cpu(), f.cpu()
        return gather_state(inst, pos, f, self.members, self.group, dst)

    def close(self):
        self.sim.close()
