"""Physics of the DiReBM step on the GPU: the rest state on a regular lattice is a fixed point, and
Taylor-Green decay follows the BGK viscosity up to a tau-independent numerical part (the
reference's finding, experiments/exp_numerical_viscosity.py: lambda = 2 (nu_phys + nu_num) k^2
with nu_phys = cs^2 (tau - 1/2) and nu_num roughly constant)."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _grid(n, jitter=0.0, seed=0):
    rng = np.random.default_rng(seed)
    x = (np.indices((n, n)).reshape(2, -1).T[:, ::-1] + 0.5).astype(np.float64)
    if jitter:
        x += rng.uniform(-jitter, jitter, size=x.shape)
    return np.mod(x, n)


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-14), ("fp32dev", 1e-6)])
def test_rest_state_on_a_lattice_is_a_fixed_point(precision, tol):
    from direbm_gb300.lattices import D2Q9, equilibrium
    from direbm_gb300.sim import Instance, Simulation

    n = 40
    x = _grid(n)
    f = equilibrium(np.ones(len(x)), np.zeros((len(x), 2)), D2Q9)
    sim = Simulation([Instance(dims=(n, n), tau=0.7)], lattice="D2Q9", precision=precision, dx=1.0, r_res=1.5,
                     cell=1.0, moment_capacity=2 * len(x))
    sim.set_state(None, x, f)
    sim.step(15)
    _, xg, fg = sim.state_numpy()
    assert len(xg) == len(x)
    u = (fg @ D2Q9.C) / fg.sum(1)[:, None]
    assert np.abs(u).max() < tol
    assert np.abs(fg.sum(1) - 1.0).max() < tol
    np.testing.assert_allclose(np.sort(xg[:, 0] + n * xg[:, 1]), np.sort(x[:, 0] + n * x[:, 1]), atol=1e-5)


def test_taylor_green_decay_follows_the_bgk_viscosity():
    from direbm_gb300.lattices import D2Q9, equilibrium
    from direbm_gb300.sim import Instance, Simulation

    n, steps, taus = 96, 40, (0.6, 0.8, 1.0)
    k = 2 * np.pi / n
    x = _grid(n, 0.25)

    def tg(p):
        return np.stack([-np.cos(k * p[:, 0]) * np.sin(k * p[:, 1]), np.sin(k * p[:, 0]) * np.cos(k * p[:, 1])], 1)

    f = equilibrium(np.ones(len(x)), 0.01 * tg(x), D2Q9)
    sim = Simulation([Instance(dims=(n, n), tau=t) for t in taus], lattice="D2Q9", precision="fp32dev", dx=1.0,
                     r_res=1.5, cell=1.0, moment_capacity=4 * len(x) * len(taus))
    sim.set_state(np.repeat(np.arange(len(taus)), len(x)).astype(np.int32), np.concatenate([x] * len(taus)),
                  np.concatenate([f] * len(taus)))
    amps = [[] for _ in taus]
    for s in range(steps + 1):
        ib, xg, fg = sim.state_numpy()
        u = (fg @ D2Q9.C) / fg.sum(1)[:, None]
        for i in range(len(taus)):
            sel = ib == i
            ref = tg(xg[sel])
            amps[i].append(float((u[sel] * ref).sum() / (ref * ref).sum()))
        if s < steps:
            sim.step(1)
    t = np.arange(5, steps + 1)
    nu_eff, resid = [], []
    for a in amps:
        la = np.log(np.asarray(a[5:]))
        slope, icpt = np.polyfit(t, la, 1)
        resid.append(float(np.abs(la - (slope * t + icpt)).max()))
        nu_eff.append(-slope / (2 * k * k))
    nu_phys = (np.asarray(taus) - 0.5) / 3.0
    b, a0 = np.polyfit(nu_phys, nu_eff, 1)
    assert max(resid) < 0.01  # exponential decay
    assert 0.7 < b < 1.3, (b, nu_eff)  # d nu_eff / d nu_phys = 1: the BGK viscosity
    assert a0 > 0, a0  # plus a positive numerical viscosity, independent of tau
