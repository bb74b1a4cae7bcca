"""Parity at the benchmark configurations' own sizes (not only at small test cases).

* Taylor-Green, FP64 (the plain-DiReBM configuration): 128 x 128 points on a jittered grid in a
  periodic box, u0 = 0.05, tau 0.6, resampling radius 1.5h, thinning cell h, D2Q9.  The GPU step
  against the numpy oracle (oracle/grid_step.py), step by step for 10 steps from one shared start:
  integer structure exactly, positions to 1e-12 cells and f to 1e-12 relative.  The configuration
  runs 200 steps; those run on the GPU alone and are checked for FP64 mass conservation and for the
  decay of the Taylor-Green mode: its amplitude (the velocity field's projection on the initial
  mode) falls at every 10-step sample and ends below the physical viscous decay exp(-2 nu k^2 t),
  nu = (tau - 1/2)/3, since the method adds numerical viscosity.  The summed kinetic energy is not
  monotone: the first resampling of the jittered points adds velocity noise around the mode (the
  oracle shows the same), so the mode amplitude is the decaying quantity.
* The inverse problem (64k points, 16 mode coefficients and tau): the FP64 adjoint gradient against
  central differences of the FP64 fixed-structure torch chain (oracle/adjoint_ref.py) along three
  random directions of the 17 parameters, at the configuration's point count (256 x 256 = 65,536)
  over 10 steps with a checkpoint every 5 (the chain's CPU cost grows with steps x points; 10 steps
  keep this test near a minute).
"""

import numpy as np
import pytest
import torch

from oracle import adjoint_ref, grid_step
from tests._cases import oracle_spec, periodic_tg, tg_field

pytestmark = pytest.mark.gpu


def _rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


def _tg128():
    n = 128
    x, f = periodic_tg(n, "D2Q9", seed=0, u0=0.05)
    insts = [{"dims": (n, n), "tau": 0.6}]
    return n, x, f, insts


def test_taylor_green_128_fp64_matches_oracle_step_by_step():
    from direbm_gb300.sim import Instance, Simulation

    n, x, f, insts = _tg128()
    spec = oracle_spec("D2Q9", insts, 1.0, 1.5, 1.0)
    st = grid_step.from_world(spec, np.zeros(len(x), int), x, f)
    sim = Simulation([Instance(dims=(n, n), periodic=True, tau=0.6)], lattice="D2Q9", precision="fp64", dx=1.0,
                     r_res=1.5, cell=1.0)
    sim.set_state(None, x, f)
    for step in range(10):
        st = grid_step.step(spec, st)
        sim.step(1)
        _, xo, fo = grid_step.to_world(spec, st)
        _, xg, fg = sim.state_numpy()
        assert len(xg) == len(xo), (step, len(xg), len(xo))
        np.testing.assert_array_equal(np.floor(xg), np.floor(xo), err_msg=f"cells differ at step {step + 1}")
        assert np.abs(xg - xo).max() < 1e-12, (step, float(np.abs(xg - xo).max()))
        assert _rel(fg, fo) < 1e-12, (step, _rel(fg, fo))
    assert sim.status() == 0


def test_taylor_green_128_fp64_200_steps_conserves_mass_and_decays():
    from direbm_gb300.lattices import D2Q9
    from direbm_gb300.sim import Instance, Simulation

    n, x, f, _ = _tg128()
    sim = Simulation([Instance(dims=(n, n), periodic=True, tau=0.6)], lattice="D2Q9", precision="fp64", dx=1.0,
                     r_res=1.5, cell=1.0)
    sim.set_state(None, x, f)
    m0 = float(sim.conservation()[0, 0])

    def amplitude(xp, fp):
        u = (fp @ D2Q9.C) / fp.sum(1)[:, None]
        ut = tg_field(xp, n, 1.0, 2)
        return float((u * ut).sum() / (ut * ut).sum())

    amps = [amplitude(x, f)]
    for _ in range(20):
        sim.step(10)
        _, xg, fg = sim.state_numpy()
        amps.append(amplitude(xg, fg))
    assert sim.status() == 0
    assert abs(float(sim.conservation()[0, 0]) / m0 - 1.0) < 1e-12
    assert all(b < a for a, b in zip(amps, amps[1:])), amps
    k = 2.0 * np.pi / n
    physical = np.exp(-2.0 * ((0.6 - 0.5) / 3.0) * k * k * 200)
    assert 0.3 < amps[-1] / amps[0] < physical, (amps[-1] / amps[0], physical)


def _mode_problem(n):
    from direbm_gb300.adjoint import ModeField

    x, _ = periodic_tg(n, "D2Q9", seed=5, u0=0.0)
    return x, ModeField(n, seed=21, points=x), ModeField(n, seed=1000, points=x)


def _chain_loss(spec, tapes, order, x, field, target, coeffs, tau, lattice):
    """The inverse-problem loss through the FP64 fixed-structure torch chain of the recorded steps."""
    from direbm_gb300.adjoint import equilibrium, velocity

    xs = torch.as_tensor(x)[torch.as_tensor(order)]
    f = equilibrium(torch.ones(len(x), dtype=torch.float64), field(xs, coeffs), lattice)
    off = torch.as_tensor(tapes[0]["in_off"])
    for T in tapes:
        off, f = adjoint_ref.step_fixed(T, spec.lattice, float(spec.R), spec.base,
                                        [i.rho_rest for i in spec.instances], off, f, tau)
    cells = tapes[-1]["out_cell"]
    n = spec.instances[0].dims[0]
    pos = torch.stack([torch.as_tensor((cells % n).astype(np.float64)),
                       torch.as_tensor((cells // n).astype(np.float64))], 1) + off
    du = velocity(f, lattice) - target(pos * spec.cell, target.coeffs)
    return (du * du).sum(1).mean()


def test_inverse_problem_gradient_matches_finite_differences_at_64k_points():
    from direbm_gb300.adjoint import Tape, equilibrium, inverse_problem_loss
    from direbm_gb300.lattices import D2Q9
    from direbm_gb300.sim import Instance, Simulation

    n, steps, every = 256, 10, 5
    x, field, target = _mode_problem(n)
    sim = Simulation([Instance(dims=(n, n), periodic=True, tau=0.6)], lattice="D2Q9", precision="fp64", dx=1.0,
                     r_res=1.5, cell=1.0, moment_capacity=4 * len(x))
    coeffs = torch.tensor(field.coeffs, dtype=torch.float64, device="cuda", requires_grad=True)
    tau = torch.tensor([0.6], dtype=torch.float64, device="cuda", requires_grad=True)
    x_d = torch.as_tensor(x, device="cuda")
    loss = inverse_problem_loss(sim, x_d, field, coeffs, tau, target, steps, every)
    loss.backward()
    g = torch.cat([coeffs.grad, tau.grad]).cpu().numpy()
    assert np.all(np.isfinite(g)) and np.abs(g).max() > 0

    # the same trajectory recorded step by step, then central differences of the FP64 chain
    f0 = equilibrium(torch.ones(len(x), dtype=torch.float64, device="cuda"), field(x_d, coeffs.detach()), D2Q9)
    sim.set_tau([0.6])
    sim.set_state(None, x_d, f0)
    order = sim.import_order(len(x)).cpu().numpy()
    tape = Tape(sim)
    for _ in range(steps):
        tape.step()
    tapes = [tape.export(i) for i in range(steps)]
    spec = oracle_spec("D2Q9", [{"dims": (n, n), "tau": 0.6}], 1.0, 1.5, 1.0)
    with torch.no_grad():
        l0 = _chain_loss(spec, tapes, order, x, field, target, torch.as_tensor(field.coeffs),
                         torch.tensor([0.6], dtype=torch.float64), D2Q9)
    assert abs(float(l0) - loss.item()) <= 1e-12 * abs(loss.item())
    rng = np.random.default_rng(3)
    h = 1e-5
    for _ in range(3):
        v = rng.normal(size=17)
        with torch.no_grad():
            lp = _chain_loss(spec, tapes, order, x, field, target, torch.as_tensor(field.coeffs + h * v[:16]),
                             torch.tensor([0.6 + h * v[16]], dtype=torch.float64), D2Q9)
            lm = _chain_loss(spec, tapes, order, x, field, target, torch.as_tensor(field.coeffs - h * v[:16]),
                             torch.tensor([0.6 - h * v[16]], dtype=torch.float64), D2Q9)
        fd = float(lp - lm) / (2 * h)
        assert abs(fd - float(g @ v)) <= 1e-6 * abs(fd), (fd, float(g @ v))
    tape.close()
    sim.close()
