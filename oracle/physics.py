"""BGK physics restated in FP64 (test oracle).

Follows direbm/physics.py:16-55 (recover with the vacuum guard, second-order equilibrium with the
lattice's cs^2, BGK relaxation f + (feq - f)/tau), and the deviation form used by the FP32 store:
f_i = rho * W_i + dev_i, where the rest part rho*W_i carries no momentum (sum_i W_i c_i = 0).
"""

from __future__ import annotations

import numpy as np

from .lattices import D2Q7, Lattice


def recover(f, lattice: Lattice = D2Q7):
    """rho = sum f, u = sum f c / rho (u = 0 where rho == 0), direbm/physics.py:16-26."""
    f = np.asarray(f, dtype=np.float64)
    rho = f.sum(axis=-1)
    mom = f @ lattice.C
    safe = np.where(rho == 0.0, 1.0, rho)
    return rho, mom / safe[..., None]


def equilibrium(rho, u, lattice: Lattice = D2Q7):
    """Second-order equilibrium, direbm/physics.py:29-45."""
    rho = np.asarray(rho, dtype=np.float64)
    u = np.asarray(u, dtype=np.float64)
    inv = 1.0 / lattice.cs2
    cu = u @ lattice.C.T
    usq = (u * u).sum(axis=-1)
    br = 1.0 + inv * cu + 0.5 * inv * inv * cu * cu - 0.5 * inv * usq[..., None]
    return rho[..., None] * lattice.W * br


def collide(f, tau, lattice: Lattice = D2Q7):
    """BGK collision f + (feq - f)/tau, direbm/physics.py:48-55.  ``tau`` may be per-row."""
    f = np.asarray(f, dtype=np.float64)
    rho, u = recover(f, lattice)
    feq = equilibrium(rho, u, lattice)
    tau = np.asarray(tau, dtype=np.float64)
    if tau.ndim:
        tau = tau[..., None]
    return f + (feq - f) / tau


def collide_unguarded(f, tau, lattice: Lattice = D2Q7):
    """The GPU path's collision: u = mom / rho with no vacuum guard (direbm/warp/physics.py:45-62).

    The fused kernels divide by rho exactly like the Warp kernel did; a moment with rho == 0 gives
    non-finite velocity there too.  Kept separate so tests can state which form they check.
    """
    f = np.asarray(f, dtype=np.float64)
    rho = f.sum(axis=-1)
    u = (f @ lattice.C) / rho[..., None]
    feq = equilibrium(rho, u, lattice)
    tau = np.asarray(tau, dtype=np.float64)
    if tau.ndim:
        tau = tau[..., None]
    return f + (feq - f) / tau


def split_rest(f, lattice: Lattice = D2Q7):
    """Split f into (rho, dev) with f = rho*W + dev (the deviation store)."""
    f = np.asarray(f, dtype=np.float64)
    rho = f.sum(axis=-1)
    return rho, f - rho[..., None] * lattice.W
