"""Velocity sets (test oracle).

D2Q7 and D3Q13-ico restate the reference's tables (direbm/constants.py:15-36,
direbm/lattices.py:44-61).  D2Q9 and D3Q19 are the standard square/cubic sets that the benchmark
configurations ask for; the reference has no table for them, so they are written from the
textbook definitions (weights 4/9, 1/9, 1/36 and 1/3, 1/18, 1/36; cs^2 = 1/3).  As in the
reference CPU simulator (direbm/reference/simulator.py:98), a direction c_i disperses by
c_i * dx, so the D2Q9 diagonals travel sqrt(2)*dx.
"""

from __future__ import annotations

from dataclasses import dataclass

import numpy as np


@dataclass(frozen=True)
class Lattice:
    C: np.ndarray  # (Q, D)
    W: np.ndarray  # (Q,)
    cs2: float
    name: str

    @property
    def D(self) -> int:
        return int(self.C.shape[1])

    @property
    def Q(self) -> int:
        return int(self.C.shape[0])


_S = np.sqrt(3.0) / 2.0
D2Q7 = Lattice(
    C=np.array([[0.0, 0.0], [1.0, 0.0], [0.5, _S], [-0.5, _S], [-1.0, 0.0], [-0.5, -_S], [0.5, -_S]]),
    W=np.array([0.5] + [1.0 / 12.0] * 6),
    cs2=0.25,
    name="D2Q7",
)

D2Q9 = Lattice(
    C=np.array([[0, 0], [1, 0], [0, 1], [-1, 0], [0, -1], [1, 1], [-1, 1], [-1, -1], [1, -1]], dtype=np.float64),
    W=np.array([4.0 / 9.0] + [1.0 / 9.0] * 4 + [1.0 / 36.0] * 4),
    cs2=1.0 / 3.0,
    name="D2Q9",
)

_PHI = (1.0 + np.sqrt(5.0)) / 2.0
_ICO = np.array(
    [
        [0, 1, _PHI], [0, 1, -_PHI], [0, -1, _PHI], [0, -1, -_PHI],
        [1, _PHI, 0], [1, -_PHI, 0], [-1, _PHI, 0], [-1, -_PHI, 0],
        [_PHI, 0, 1], [_PHI, 0, -1], [-_PHI, 0, 1], [-_PHI, 0, -1],
    ],
    dtype=np.float64,
)
_ICO = _ICO / np.linalg.norm(_ICO[0])
D3Q13 = Lattice(
    C=np.vstack([np.zeros(3), _ICO]),
    W=np.array([2.0 / 5.0] + [1.0 / 20.0] * 12),
    cs2=1.0 / 5.0,
    name="D3Q13",
)

_Q19 = [[0, 0, 0]]
_Q19 += [[1, 0, 0], [-1, 0, 0], [0, 1, 0], [0, -1, 0], [0, 0, 1], [0, 0, -1]]
_Q19 += [[1, 1, 0], [-1, -1, 0], [1, -1, 0], [-1, 1, 0],
         [1, 0, 1], [-1, 0, -1], [1, 0, -1], [-1, 0, 1],
         [0, 1, 1], [0, -1, -1], [0, 1, -1], [0, -1, 1]]
D3Q19 = Lattice(
    C=np.array(_Q19, dtype=np.float64),
    W=np.array([1.0 / 3.0] + [1.0 / 18.0] * 6 + [1.0 / 36.0] * 12),
    cs2=1.0 / 3.0,
    name="D3Q19",
)

BY_NAME = {"D2Q7": D2Q7, "D2Q9": D2Q9, "D3Q13": D3Q13, "D3Q19": D3Q19}
