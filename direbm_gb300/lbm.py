"""Batched hexagonal D2Q7 lattice Boltzmann on one GPU (host side of dbm_lbm_step).

Independent runs of the same ni x nj periodic hex lattice (each with its own tau) advance in one
launch.  Storage is structure-of-arrays (runs, 7, nj, ni); FP64 keeps f, FP32DEV keeps
f - W*rho0.  The step is collide-then-stream as in direbm/lbm.py:60-62.
"""

from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import _lib
from .lattices import D2Q7, equilibrium
from .sim import _require_cuda, _stream

OFFSETS = [(0, 0), (1, 0), (0, 1), (-1, 1), (-1, 0), (0, -1), (1, -1)]  # (di, dj), direbm/lbm.py:23
_S = np.sqrt(3.0) / 2.0


class HexLBM:
    def __init__(self, ni: int, nj: int, taus, rho0: float = 1.0, precision: str = "fp32dev", device=None):
        self.device = _require_cuda(device)
        self.lib = _lib.load()
        self.ni, self.nj = int(ni), int(nj)
        self.taus = np.atleast_1d(np.asarray(taus, dtype=np.float64))
        self.runs = len(self.taus)
        self.rho0 = float(rho0)
        if precision not in ("fp64", "fp32dev", "fp32"):
            raise ValueError("precision must be fp64 or fp32dev")
        self.precision = "fp64" if precision == "fp64" else "fp32dev"
        self._prec = _lib.FP64 if self.precision == "fp64" else _lib.FP32DEV
        dt = torch.float64 if self.precision == "fp64" else torch.float32
        shape = (self.runs, 7, self.nj, self.ni)
        self._a = torch.empty(shape, dtype=dt, device=self.device)
        self._b = torch.empty_like(self._a)
        self._c = torch.empty_like(self._a)
        self._tau = torch.as_tensor(self.taus, dtype=torch.float64, device=self.device)
        self.set_f(equilibrium(np.full((self.nj, self.ni), self.rho0), np.zeros((self.nj, self.ni, 2)), D2Q7))

    # f in the reference layout (nj, ni, 7) FP64, per run or broadcast to all runs
    def set_f(self, f, run=None):
        f = np.asarray(f, dtype=np.float64)
        soa = np.moveaxis(f, -1, -3)  # (..., 7, nj, ni)
        if self.precision == "fp32dev":
            soa = soa - (self.rho0 * D2Q7.W)[:, None, None]
        t = torch.as_tensor(np.ascontiguousarray(soa), dtype=self._a.dtype, device=self.device)
        if run is None:
            self._a.copy_(t.expand_as(self._a) if t.dim() == 3 else t)
        else:
            self._a[run].copy_(t)

    def get_f(self) -> np.ndarray:
        """f as FP64 numpy (runs, nj, ni, 7)."""
        a = self._a.to(torch.float64)
        if self.precision == "fp32dev":
            a = a + torch.as_tensor(self.rho0 * D2Q7.W, dtype=torch.float64, device=self.device)[:, None, None]
        return np.moveaxis(a.cpu().numpy(), 1, -1)

    def step(self, n: int = 1):
        if n <= 0:
            return
        with torch.cuda.device(self.device):
            _lib.check(self.lib.dbm_lbm_step(self._prec, self._a.data_ptr(), self._b.data_ptr(), self.ni, self.nj,
                                             self.runs, self._tau.data_ptr(), ctypes.c_double(self.rho0), int(n),
                                             self._c.data_ptr(), _stream()), "dbm_lbm_step")
        self._a, self._b = self._b, self._a

    @property
    def state(self) -> torch.Tensor:
        return self._a

    def macroscopic(self):
        """(rho (runs, nj, ni), u (runs, nj, ni, 2)) in FP64 numpy."""
        f = self.get_f()
        rho = f.sum(-1)
        mom = f @ D2Q7.C
        safe = np.where(rho == 0.0, 1.0, rho)
        return rho, mom / safe[..., None]

    def shear_amplitude(self) -> np.ndarray:
        """Projection of u_x onto sin(2 pi j / nj), per run (device reduction in FP64)."""
        a = self._a.to(torch.float64)
        cx = torch.as_tensor(D2Q7.C[:, 0], dtype=torch.float64, device=self.device)
        rho = a.sum(1) + (self.rho0 if self.precision == "fp32dev" else 0.0)
        mx = (a * cx[None, :, None, None]).sum(1)
        ux = (mx / rho).mean(-1)  # (runs, nj)
        s = torch.sin(2 * torch.pi * torch.arange(self.nj, dtype=torch.float64, device=self.device) / self.nj)
        return ((ux * s).sum(-1) / (s * s).sum()).cpu().numpy()
