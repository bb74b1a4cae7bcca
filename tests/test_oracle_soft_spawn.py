"""Soft-outer spawn in the oracle (CPU).

The spawn rule is pinned to the reference's own CPU simulator: ``_soft_new_point``
(direbm/reference/simulator.py:153-166) evaluated on seeded sets of component directions,
committed as tests/golden/soft_spawn.npz by tests/golden/make_golden.py.  The oracle's step with
the spawn reproduces the purpose the reference tests for it (tests/test_reference.py:68-85): a
point pulse's front is more isotropic with the spawn than without.
"""

from pathlib import Path

import numpy as np

from oracle import grid_step as gs
from oracle.lattices import D2Q7
from oracle.physics import equilibrium

GOLD = Path(__file__).resolve().parent / "golden" / "soft_spawn.npz"


def test_spawn_point_matches_reference_golden():
    g = np.load(GOLD)
    labels, p, ref = g["labels"], g["p"], g["spawn"]
    n = np.zeros((len(labels), 7), dtype=np.int64)
    for j, lab in enumerate(labels):
        for i in lab[lab >= 0]:
            n[j, i] += 1
    acc = gs.direction_sum(n, np.asarray(D2Q7.C, dtype=np.float64))
    offset = 2.0 * (1.0 - np.sqrt(3.0) / 2.0)  # dx = 1
    sp, go = gs.spawn_point(p, acc, offset)
    assert np.array_equal(go, ~np.isnan(ref[:, 0]))
    assert (~go).sum() >= 2  # the balanced sets spawn nothing
    np.testing.assert_allclose(sp[go], ref[go], rtol=0, atol=1e-14)


def _pulse(ks, steps, rho=1.6):
    spec = gs.GridSpec(lattice=D2Q7, dx=1.0, r_res=1.0, cell=0.25, kappa_hard=4, kappa_soft=ks,
                       instances=[gs.Instance(dims=(96, 96), origin=(-48, -48), periodic=True, tau=0.6)])
    f = equilibrium(np.array([rho]), np.zeros((1, 2)), D2Q7)
    st = gs.from_world(spec, np.zeros(1, int), np.zeros((1, 2)), f)
    for _ in range(steps):
        st = gs.step(spec, st)
    _, x, fv = gs.to_world(spec, st)
    return x, fv


def front_anisotropy(x, sectors=36):
    """std / mean of the outermost radius per angular sector (tests/test_reference.py:68-79)."""
    r = np.linalg.norm(x, axis=1)
    th = np.arctan2(x[:, 1], x[:, 0]) % (2 * np.pi)
    edges = np.linspace(0, 2 * np.pi, sectors + 1)
    front = np.array([r[(th >= edges[k]) & (th < edges[k + 1])].max(initial=0.0) for k in range(sectors)])
    return front.std() / front.mean()


def test_oracle_spawn_reduces_front_anisotropy():
    x_off, _ = _pulse(0, 6)
    x_on, _ = _pulse(5, 6)
    assert len(x_on) > len(x_off)
    assert front_anisotropy(x_on) < 0.5 * front_anisotropy(x_off)


def test_oracle_spawn_threshold_at_kappa_hard_is_off():
    x0, f0 = _pulse(0, 3)
    x4, f4 = _pulse(4, 3)  # no kappa satisfies 4 < kappa <= 4
    assert np.array_equal(x0, x4) and np.array_equal(f0, f4)
