"""Seeded input builders shared by the GPU parity tests (numpy only)."""

from __future__ import annotations

import numpy as np

from oracle import grid_step
from oracle.lattices import BY_NAME
from oracle.physics import equilibrium


def tg_field(x, n, u0, D):
    k = 2.0 * np.pi / n
    u = np.zeros_like(x)
    u[:, 0] = -u0 * np.cos(k * x[:, 0]) * np.sin(k * x[:, 1])
    u[:, 1] = u0 * np.sin(k * x[:, 0]) * np.cos(k * x[:, 1])
    return u


def jittered_grid(n, D, seed=0, jitter=0.25, h=1.0):
    rng = np.random.default_rng(seed)
    x = (np.indices((n,) * D).reshape(D, -1).T + 0.5) * h
    x += rng.uniform(-jitter, jitter, size=x.shape) * h
    return x


def periodic_tg(n, lattice="D2Q9", seed=0, u0=0.05, jitter=0.25, rho=1.0):
    lat = BY_NAME[lattice]
    x = jittered_grid(n, lat.D, seed, jitter)
    x = np.mod(x, n)
    u = tg_field(x, n, u0, lat.D)
    f = equilibrium(np.full(len(x), rho), u, lat)
    return x, f


def rest_pulse(half, lattice="D2Q7", pulse=1.5):
    """The reference's 13x13-style rest block with a central pulse (tests/test_warp_simulator.py:10-21)."""
    lat = BY_NAME[lattice]
    pos, f = [], []
    for i in range(-half, half + 1):
        for j in range(-half, half + 1):
            pos.append([float(i), float(j)])
            rho = pulse if (pulse is not None and i == 0 and j == 0) else 1.0
            f.append(equilibrium(np.float64(rho), np.zeros(2), lat))
    return np.array(pos), np.stack(f)


def oracle_spec(lattice, instances, dx, r_res, cell, kappa_hard=4, dtype=np.float64):
    insts = [grid_step.Instance(dims=tuple(i["dims"]), origin=tuple(i.get("origin", (0,) * len(i["dims"]))),
                                periodic=i.get("periodic", True), tau=i.get("tau", 0.6),
                                rho_rest=i.get("rho_rest", 1.0), obstacle=i.get("obstacle"),
                                inflow=i.get("inflow")) for i in instances]
    return grid_step.GridSpec(lattice=BY_NAME[lattice], dx=dx, r_res=r_res, cell=cell, kappa_hard=kappa_hard,
                              instances=insts, dtype=dtype)


def bounded_box(pos, cell, margin):
    lo = np.floor((pos.min(0) - margin) / cell).astype(int)
    hi = np.ceil((pos.max(0) + margin) / cell).astype(int)
    return tuple(int(v) for v in hi - lo), tuple(int(v) for v in lo)


def around_obstacle(n, D, center, radius, seed=0, u0=0.04, lattice="D2Q9", jitter=0.25):
    """Jittered points on an n^D periodic box outside a sphere, uniform flow u0 along x."""
    lat = BY_NAME[lattice]
    x = np.mod(jittered_grid(n, D, seed, jitter), n)
    keep = ((x - np.asarray(center)) ** 2).sum(1) >= (radius + 0.5) ** 2
    x = x[keep]
    u = np.zeros_like(x)
    u[:, 0] = u0
    f = equilibrium(np.ones(len(x)), u, lat)
    return x, f
