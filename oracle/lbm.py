"""Hexagonal D2Q7 lattice Boltzmann restated in FP64 (test oracle).

Follows direbm/lbm.py:26-66: skewed axial indices (i, j) with physical position
i*(1,0) + j*(1/2, sqrt(3)/2); a step is BGK collision followed by periodic streaming, where
direction k moves by the axial shift (di, dj) of direbm/lbm.py:23.  The array layout here is the
reference's (nj, ni, Q); the CUDA store is structure-of-arrays (Q, nj, ni).
"""

from __future__ import annotations

import numpy as np

from .lattices import D2Q7
from .physics import collide, equilibrium, recover

OFFSETS = [(0, 0), (1, 0), (0, 1), (-1, 1), (-1, 0), (0, -1), (1, -1)]  # (di, dj) per direction
_S = np.sqrt(3.0) / 2.0


def rest_state(ni: int, nj: int, rho0: float = 1.0) -> np.ndarray:
    return equilibrium(np.full((nj, ni), float(rho0)), np.zeros((nj, ni, 2)), D2Q7)


def set_pulse(f: np.ndarray, rho_pulse: float) -> np.ndarray:
    nj, ni = f.shape[:2]
    f = f.copy()
    f[nj // 2, ni // 2] = equilibrium(np.float64(rho_pulse), np.zeros(2), D2Q7)
    return f


def stream(f: np.ndarray) -> np.ndarray:
    out = np.empty_like(f)
    for k, (di, dj) in enumerate(OFFSETS):
        out[..., k] = np.roll(f[..., k], shift=(dj, di), axis=(0, 1))
    return out


def step(f: np.ndarray, tau) -> np.ndarray:
    """collide then stream, direbm/lbm.py:60-62.  ``tau`` scalar."""
    return stream(collide(f, tau, D2Q7))


def run(f: np.ndarray, tau, steps: int) -> np.ndarray:
    for _ in range(steps):
        f = step(f, tau)
    return f


def shear_wave(ni: int, nj: int, amp: float, rho0: float = 1.0) -> np.ndarray:
    """Equilibrium of u_x = amp*sin(2*pi*j/nj), u_y = 0 (a function of the row only, so it is
    periodic on the skewed domain)."""
    j = np.arange(nj, dtype=np.float64)
    ux = amp * np.sin(2.0 * np.pi * j / nj)
    u = np.zeros((nj, ni, 2))
    u[..., 0] = ux[:, None]
    return equilibrium(np.full((nj, ni), float(rho0)), u, D2Q7)


def shear_amplitude(f: np.ndarray) -> float:
    """Projection of u_x onto sin(2*pi*j/nj)."""
    nj = f.shape[0]
    _, u = recover(f, D2Q7)
    s = np.sin(2.0 * np.pi * np.arange(nj) / nj)
    ux = u[..., 0].mean(axis=1)
    return float((ux * s).sum() / (s * s).sum())


def shear_decay_rate(tau: float, nj: int) -> float:
    """Analytic viscous decay rate nu*k^2 per step, nu = cs^2 (tau - 1/2), k = 2*pi/(nj*sqrt(3)/2)."""
    nu = D2Q7.cs2 * (tau - 0.5)
    k = 2.0 * np.pi / (nj * _S)
    return nu * k * k


def to_soa(f: np.ndarray) -> np.ndarray:
    return np.ascontiguousarray(np.moveaxis(f, -1, 0))


def from_soa(f: np.ndarray) -> np.ndarray:
    return np.ascontiguousarray(np.moveaxis(f, 0, -1))
