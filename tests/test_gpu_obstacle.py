"""Obstacles (bounce-back sphere / disc) and the inflow layer on the GPU against the oracle
(oracle/grid_step.py with Instance.obstacle / Instance.inflow): the same blocked directions, the
same control points (bit-exact cells), FP64 values to 1e-12, and the physical invariants (nothing
inside the solid, mass kept up to the removed points)."""

import numpy as np
import pytest

from _cases import around_obstacle, oracle_spec
from oracle import grid_step

pytestmark = pytest.mark.gpu


def _sim(lattice, instances, precision, dx=1.0, r_res=1.5, cell=1.0, cap=0):
    from direbm_gb300.sim import Instance, Simulation

    return Simulation([Instance(**i) for i in instances], lattice=lattice, precision=precision, dx=dx, r_res=r_res,
                      cell=cell, moment_capacity=cap)


def _inside(x, center, radius):
    return ((x - np.asarray(center)) ** 2).sum(1) < radius * radius


CASES = {
    "disc_d2q9": ("D2Q9", 40, (20.0, 20.0), 5.0, None),
    "disc_d2q9_inflow": ("D2Q9", 40, (20.0, 20.0), 5.0, ((0.04, 0.0), 3)),
    "sphere_d3q19": ("D3Q19", 24, (12.0, 12.0, 12.0), 4.0, None),
}


def _case(name):
    lattice, n, center, radius, inflow = CASES[name]
    D = len(center)
    x, f = around_obstacle(n, D, center, radius, seed=7, lattice=lattice)
    inst = dict(dims=(n,) * D, periodic=True, tau=0.6, obstacle=(center, radius), inflow=inflow)
    return lattice, inst, x, f, center, radius


@pytest.mark.parametrize("name", sorted(CASES))
def test_obstacle_step_matches_oracle_fp64(name):
    lattice, inst, x, f, center, radius = _case(name)
    spec = oracle_spec(lattice, [inst], 1.0, 1.5, 1.0)
    st = grid_step.from_world(spec, np.zeros(len(x), np.int64), x, f)
    assert grid_step.blocked(spec, st).any()
    ref = grid_step.step(spec, st)
    sim = _sim(lattice, [inst], "fp64", cap=2 * len(x))
    sim.set_state(None, x, f)
    sim.step(1)
    sim.check_status()
    _, xg, fg = sim.state_numpy()
    _, xo, fo = grid_step.to_world(spec, ref)
    assert len(xg) == len(xo)
    np.testing.assert_allclose(xg, xo, rtol=0, atol=1e-12)
    np.testing.assert_allclose(fg, fo, rtol=0, atol=1e-12 * np.abs(fo).max())


@pytest.mark.parametrize("precision", ["fp64", "fp32dev"])
@pytest.mark.parametrize("name", ["disc_d2q9", "sphere_d3q19"])
def test_nothing_enters_the_solid_and_mass_is_kept(name, precision):
    lattice, inst, x, f, center, radius = _case(name)
    sim = _sim(lattice, [inst], precision, cap=2 * len(x))
    sim.set_state(None, x, f)
    m0 = float(sim.conservation()[0, 0])
    for _ in range(5):
        sim.step(1)
        _, xg, fg = sim.state_numpy()
        assert not _inside(xg, center, radius).any()
        assert np.isfinite(fg).all()
    sim.check_status()
    m1 = float(sim.conservation()[0, 0])
    assert abs(m1 / m0 - 1.0) < 0.02  # bounce-back keeps component mass; removed points and gap fill move a little


def test_inflow_layer_imposes_its_velocity():
    lattice, inst, x, f, center, radius = _case("disc_d2q9_inflow")
    inst = dict(inst, inflow=((0.08, 0.0), 4))  # stronger than the initial 0.04
    sim = _sim(lattice, [inst], "fp32dev", cap=2 * len(x))
    sim.set_state(None, x, f)
    sim.step(3)
    _, xg, fg = sim.state_numpy()
    from oracle.lattices import BY_NAME

    C = BY_NAME[lattice].C
    u = (fg @ C) / fg.sum(1)[:, None]
    band = (xg[:, 0] >= 1.0) & (xg[:, 0] < 3.0)
    far = (xg[:, 0] >= 30.0) & (xg[:, 0] < 36.0)
    assert u[band, 0].mean() > u[far, 0].mean() + 0.01


def test_obstacle_runs_the_untiled_path_with_the_same_bits():
    lattice, inst, x, f, center, radius = _case("disc_d2q9")
    outs = []
    for tiles in (True, False):
        from direbm_gb300.sim import Instance, Simulation

        sim = Simulation([Instance(**inst)], lattice=lattice, precision="fp32dev", dx=1.0, r_res=1.5, cell=1.0,
                         moment_capacity=2 * len(x), tiles=tiles)
        sim.set_state(None, x, f)
        sim.step(3)
        outs.append([a.copy() for a in sim.state_numpy()])
    for a, b in zip(*outs):
        np.testing.assert_array_equal(a, b)
