"""Instance sharding on one GPU: the shards of an ensemble, each stepped in its own Simulation,
give bit for bit the state of the whole ensemble stepped in one Simulation (instances never
interact), and the partition keeps every instance exactly once."""

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _ensemble(n_inst=9, seed=4):
    from direbm_gb300.lattices import D2Q9, equilibrium
    from direbm_gb300.sim import Instance

    rng = np.random.default_rng(seed)
    sides = rng.integers(12, 40, n_inst)
    insts, xs, fs, ib = [], [], [], []
    for i, n in enumerate(sides):
        n = int(n)
        x = (np.indices((n, n)).reshape(2, -1).T[:, ::-1] + 0.5) + rng.uniform(-0.25, 0.25, (n * n, 2))
        x = np.mod(x, n)
        k = 2 * np.pi / n
        u = 0.03 * np.stack([np.sin(k * x[:, 1]), np.cos(k * x[:, 0])], 1)
        insts.append(Instance(dims=(n, n), periodic=True, tau=float(rng.uniform(0.55, 1.0))))
        xs.append(x)
        fs.append(equilibrium(np.ones(n * n), u, D2Q9))
        ib.append(np.full(n * n, i))
    return insts, np.concatenate(ib), np.concatenate(xs), np.concatenate(fs)


@pytest.mark.parametrize("precision", ["fp32dev", "fp64"])
def test_shards_match_the_whole_ensemble_bitwise(precision):
    from direbm_gb300.shard import ShardedEnsemble
    from direbm_gb300.sim import Simulation

    insts, ib, x, f = _ensemble()
    kw = dict(lattice="D2Q9", precision=precision, dx=1.0, r_res=1.5, cell=1.0)
    whole = Simulation(insts, moment_capacity=len(x), **kw)
    whole.set_state(ib, x, f)
    whole.step(6)
    wi, wp, wf = (t.cpu().numpy() for t in whole.state())
    whole.close()

    world = 3
    parts = [ShardedEnsemble(insts, ib, x, f, rank=r, world=world, **kw) for r in range(world)]
    seen = np.concatenate([p.members for p in parts])
    np.testing.assert_array_equal(np.sort(seen), np.arange(len(insts)))
    for p in parts:
        p.step(6)
    gi, gp, gf = [], [], []
    for p in parts:
        li, lp, lf = (t.cpu().numpy() for t in p.sim.state())
        gi.append(p.members[li.astype(np.int64)])
        gp.append(lp)
        gf.append(lf)
        p.close()
    gi, gp, gf = np.concatenate(gi), np.concatenate(gp), np.concatenate(gf)
    order = np.argsort(gi, kind="stable")
    np.testing.assert_array_equal(gi[order], wi)
    np.testing.assert_array_equal(gp[order], wp)
    np.testing.assert_array_equal(gf[order], wf)


def test_single_shard_gather_maps_to_global_instances():
    from direbm_gb300.shard import ShardedEnsemble

    insts, ib, x, f = _ensemble(4)
    p = ShardedEnsemble(insts, ib, x, f, rank=0, world=1, lattice="D2Q9", precision="fp32dev", dx=1.0, r_res=1.5,
                        cell=1.0)
    p.step(2)
    gi, gp, gf = p.gather()
    assert gi.dtype == torch.int32
    np.testing.assert_array_equal(np.unique(gi.cpu().numpy()), np.arange(4))
    p.close()
