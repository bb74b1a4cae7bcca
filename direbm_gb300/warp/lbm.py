"""GpuHexLBM with the reference's interface (direbm/warp/lbm.py:72-115).

``GpuHexLBM(ni, nj, tau, rho0=1.0, device=None)`` with ``set_pulse``, ``step``, ``macroscopic``,
``radius``, ``center`` and ``f`` (``.f.numpy()`` gives the (nj, ni, 7) FP32 populations, as the
Warp array did).  The engine is the fused collide-stream kernel of direbm_gb300.lbm.HexLBM.
"""

from __future__ import annotations

import numpy as np

from ..lattices import D2Q7, equilibrium
from ..lbm import HexLBM

_S = np.sqrt(3.0) / 2.0


class _FView:
    def __init__(self, owner):
        self._o = owner

    def numpy(self):
        return self._o._eng.get_f()[0].astype(np.float32)

    @property
    def shape(self):
        return (self._o.nj, self._o.ni, 7)


class GpuHexLBM:
    def __init__(self, ni, nj, tau, rho0=1.0, device=None, precision="fp32dev"):
        self.ni = int(ni)
        self.nj = int(nj)
        self.tau = float(tau)
        self.rho0 = float(rho0)
        self._eng = HexLBM(self.ni, self.nj, [self.tau], rho0=self.rho0, precision=precision, device=device)
        self.device = self._eng.device
        self.center = (self.ni // 2, self.nj // 2)

    @property
    def f(self):
        return _FView(self)

    def set_pulse(self, rho_pulse):
        ci, cj = self.center
        f = self._eng.get_f()[0]
        f[cj, ci] = equilibrium(np.float64(rho_pulse), np.zeros(2), D2Q7)
        self._eng.set_f(f, run=0)

    def step(self):
        self._eng.step(1)

    def macroscopic(self):
        rho, u = self._eng.macroscopic()
        return rho[0], u[0]

    def radius(self):
        ii, jj = np.meshgrid(np.arange(self.ni), np.arange(self.nj))
        ci, cj = self.center
        x = (ii + jj * 0.5) - (ci + cj * 0.5)
        y = (jj - cj) * _S
        return np.sqrt(x * x + y * y)


__all__ = ["GpuHexLBM"]
