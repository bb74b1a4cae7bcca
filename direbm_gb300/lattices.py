"""Velocity sets known to the library (host-side copies of the tables compiled into the kernels).

D2Q7 and D3Q13 are the reference's sets (direbm/constants.py:15-36, direbm/lattices.py:44-61);
D2Q9 and D3Q19 are the standard square and cubic sets.  ``equilibrium`` is the reference's
second-order form (direbm/physics.py:29-45) and is used for building initial states on the host.
"""

from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from . import _lib


@dataclass(frozen=True)
class Lattice:
    name: str
    id: int
    C: np.ndarray
    W: np.ndarray
    cs2: float

    @property
    def Q(self) -> int:
        return int(self.C.shape[0])

    @property
    def D(self) -> int:
        return int(self.C.shape[1])


_S = np.sqrt(3.0) / 2.0
_PHI = (1.0 + np.sqrt(5.0)) / 2.0
_ICO = np.array(
    [[0, 1, _PHI], [0, 1, -_PHI], [0, -1, _PHI], [0, -1, -_PHI], [1, _PHI, 0], [1, -_PHI, 0],
     [-1, _PHI, 0], [-1, -_PHI, 0], [_PHI, 0, 1], [_PHI, 0, -1], [-_PHI, 0, 1], [-_PHI, 0, -1]]
)
_ICO = _ICO / np.sqrt(1.0 + _PHI * _PHI)

D2Q7 = Lattice(
    "D2Q7", _lib.D2Q7,
    np.array([[0, 0], [1, 0], [0.5, _S], [-0.5, _S], [-1, 0], [-0.5, -_S], [0.5, -_S]], dtype=np.float64),
    np.array([0.5] + [1 / 12] * 6), 0.25,
)
D2Q9 = Lattice(
    "D2Q9", _lib.D2Q9,
    np.array([[0, 0], [1, 0], [0, 1], [-1, 0], [0, -1], [1, 1], [-1, 1], [-1, -1], [1, -1]], dtype=np.float64),
    np.array([4 / 9] + [1 / 9] * 4 + [1 / 36] * 4), 1.0 / 3.0,
)
D3Q13 = Lattice("D3Q13", _lib.D3Q13, np.vstack([np.zeros(3), _ICO]), np.array([0.4] + [0.05] * 12), 0.2)
D3Q19 = Lattice(
    "D3Q19", _lib.D3Q19,
    np.array([[0, 0, 0], [1, 0, 0], [-1, 0, 0], [0, 1, 0], [0, -1, 0], [0, 0, 1], [0, 0, -1],
              [1, 1, 0], [-1, -1, 0], [1, -1, 0], [-1, 1, 0], [1, 0, 1], [-1, 0, -1], [1, 0, -1],
              [-1, 0, 1], [0, 1, 1], [0, -1, -1], [0, 1, -1], [0, -1, 1]], dtype=np.float64),
    np.array([1 / 3] + [1 / 18] * 6 + [1 / 36] * 12), 1.0 / 3.0,
)

LATTICES = {lat.name: lat for lat in (D2Q7, D2Q9, D3Q13, D3Q19)}


def get(lattice) -> Lattice:
    if isinstance(lattice, Lattice):
        return lattice
    if isinstance(lattice, str):
        key = lattice.upper().replace("-ICO", "")
        if key in LATTICES:
            return LATTICES[key]
    for lat in LATTICES.values():
        if lattice == lat.id:
            return lat
    # a reference Lattice object (direbm.lattices.Lattice): match by table
    C = getattr(lattice, "C", None)
    if C is not None:
        for lat in LATTICES.values():
            if lat.C.shape == np.shape(C) and np.allclose(lat.C, C):
                return lat
    raise ValueError(f"unknown lattice {lattice!r}")


def equilibrium(rho, u, lattice=D2Q7) -> np.ndarray:
    """Host-side f_eq(rho, u) in FP64 (for building initial states)."""
    lat = get(lattice)
    rho = np.asarray(rho, dtype=np.float64)
    u = np.asarray(u, dtype=np.float64)
    inv = 1.0 / lat.cs2
    cu = u @ lat.C.T
    usq = (u * u).sum(axis=-1)
    br = 1.0 + inv * cu + 0.5 * inv * inv * cu * cu - 0.5 * inv * usq[..., None]
    return rho[..., None] * lat.W * br
