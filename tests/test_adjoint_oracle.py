"""The fixed-structure FP64 torch step (oracle/adjoint_ref.py) against the numpy oracle step, and its
autograd gradient against central finite differences (CPU)."""

import numpy as np
import pytest
import torch

from oracle import adjoint_ref, grid_step
from tests._cases import bounded_box, oracle_spec, periodic_tg, rest_pulse


def _tg_case():
    n = 24
    x, f = periodic_tg(n, "D2Q9", seed=3, u0=0.05)
    spec = oracle_spec("D2Q9", [{"dims": (n, n), "tau": 0.6}], 1.0, 1.5, 1.0, 4)
    st = grid_step.from_world(spec, np.zeros(len(x), np.int64), x, f)
    return spec, st


def _pulse_case(jitter=0.0):
    x, f = rest_pulse(6, "D2Q7", 1.5)
    x = x + np.random.default_rng(11).uniform(-jitter, jitter, size=x.shape)
    dims, origin = bounded_box(x, 0.25, 3.0)
    spec = oracle_spec("D2Q7", [{"dims": dims, "origin": origin, "periodic": False, "tau": 0.7}], 1.0, 1.0, 0.25, 4)
    st = grid_step.from_world(spec, np.zeros(len(x), np.int64), x, f)
    return spec, st


CASES = {"tg_d2q9": _tg_case, "pulse_d2q7": _pulse_case, "jittered_pulse_d2q7": lambda: _pulse_case(0.1)}
# Central differences need a point away from the kink of |y - p| at zero distance: on the exact
# lattice of the pulse case many components sit within rounding of a control point.
FD_CASES = ["tg_d2q9", "jittered_pulse_d2q7"]


def _run(spec, T, off, f, tau):
    return adjoint_ref.step_fixed(T, spec.lattice, float(spec.R), spec.base, [i.rho_rest for i in spec.instances],
                                  off, f, tau)


@pytest.mark.parametrize("case", sorted(CASES))
def test_fixed_step_reproduces_oracle_step(case):
    spec, st = CASES[case]()
    T, nxt = adjoint_ref.tape_from_oracle(spec, st)
    assert T["counts"]["refine"] > 0 and T["counts"]["resample"] > 0
    if "pulse" in case:
        assert T["counts"]["gapfill"] > 0
    tau = torch.tensor([i.tau for i in spec.instances], dtype=torch.float64)
    off, F = _run(spec, T, torch.as_tensor(st.off), torch.as_tensor(st.f), tau)
    np.testing.assert_allclose(off.numpy(), nxt.off, rtol=0, atol=1e-13)
    np.testing.assert_allclose(F.numpy(), nxt.f, rtol=1e-12, atol=1e-14)


@pytest.mark.parametrize("case", FD_CASES)
def test_fixed_step_gradient_matches_central_differences(case):
    spec, st = CASES[case]()
    T, _ = adjoint_ref.tape_from_oracle(spec, st)
    rng = np.random.default_rng(5)
    P, Q, D = T["counts"]["P"], spec.Q, spec.D
    wo = torch.as_tensor(rng.normal(size=(P, D)))
    wf = torch.as_tensor(rng.normal(size=(P, Q)))
    off0 = torch.as_tensor(st.off.astype(np.float64))
    f0 = torch.as_tensor(st.f)
    tau0 = torch.tensor([i.tau for i in spec.instances], dtype=torch.float64)

    def loss(off, f, tau):
        o, F = _run(spec, T, off, f, tau)
        return (o * wo).sum() + (F * wf).sum()

    off = off0.clone().requires_grad_(True)
    f = f0.clone().requires_grad_(True)
    tau = tau0.clone().requires_grad_(True)
    loss(off, f, tau).backward()
    vo = torch.as_tensor(rng.normal(size=off0.shape)) * 1e-3
    vf = torch.as_tensor(rng.normal(size=f0.shape)) * f0.abs().mean()
    vt = torch.ones_like(tau0) * 0.05
    g_dir = float((off.grad * vo).sum() + (f.grad * vf).sum() + (tau.grad * vt).sum())
    h = 1e-5
    with torch.no_grad():
        lp = float(loss(off0 + h * vo, f0 + h * vf, tau0 + h * vt))
        lm = float(loss(off0 - h * vo, f0 - h * vf, tau0 - h * vt))
    fd = (lp - lm) / (2 * h)
    assert abs(fd - g_dir) <= 1e-6 * max(abs(fd), 1e-12), (fd, g_dir)
