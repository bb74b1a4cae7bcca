"""GpuSimulator with the reference's interface (direbm/warp/simulator.py:25-77).

``GpuSimulator(pos_m, f_m, tau, *, dx, alpha, kappa_hard, rho_rest, device)`` with ``step()``,
``moments() -> (positions (N, 2) FP32, f (N, Q) FP32)``, ``pos_m`` / ``f_m`` (``.shape[0]`` is the
moment count) and ``iteration``.  The engine is the fused batched step (direbm_gb300.sim) with a
single instance.

The reference domain is unbounded.  The fused step works on a dense cell grid, so an unbounded
run is kept in a bounded box that is re-planned as the material spreads: moments move by at most
max|c|*dx per step (every new moment is a weighted mean of component positions), so a box with a
margin of (replan_every + 1) steps of growth cannot be left before the next planning point; at
that point the box is re-centred on the current bounding box if needed.  The bounding box is a
device reduction (two D-vectors reach the host) and a re-plan moves the state device to device
through the world-position export and import (which re-derive each moment's cell, offset and, in
the FP32-deviation store, its FP32 density, so a re-planned run can differ from an unmoved one in
the last bits).
A device status bit (out_of_box) guards the invariant; ``step`` does not wait for the device, and
the status is read at the next planning point or state read, which raise if a bit is set.

Extra keyword arguments (not in the reference): ``lattice``, ``r_res`` (default dx), ``cell``
(default dx/alpha), ``precision`` ("fp32dev" or "fp64"), ``box`` ((lo, hi) world corners of a fixed
box), ``periodic`` (with ``box``), ``graphs``.
"""

from __future__ import annotations

import numpy as np
import torch

from ..lattices import D2Q7, equilibrium, get
from ..sim import Instance, Simulation
from ._arrays import DeviceArray

DX = 1.0
ALPHA = 4.0
KAPPA_HARD = 4


class GpuSimulator:
    def __init__(
        self,
        pos_m,
        f_m,
        tau,
        *,
        dx=DX,
        alpha=ALPHA,
        kappa_hard=KAPPA_HARD,
        rho_rest=1.0,
        device=None,
        lattice=D2Q7,
        r_res=None,
        cell=None,
        precision="fp32dev",
        box=None,
        periodic=False,
        replan_every=8,
        graphs=True,
    ):
        self.lattice = get(lattice)
        self.tau = float(tau)
        self.dx = float(dx)
        self.cell = float(dx / alpha if cell is None else cell)
        self.r_res = float(dx if r_res is None else r_res)
        self.kappa_hard = int(kappa_hard)
        self.rho_rest = float(rho_rest)
        self.precision = precision
        self.device = device
        self.graphs = graphs
        self.replan_every = max(1, int(replan_every))
        self.f_rest = equilibrium(np.float64(self.rho_rest), np.zeros(self.lattice.D), self.lattice)
        self.fixed_box = box is not None
        self.periodic = bool(periodic) and self.fixed_box
        self.iteration = 0
        self.replanned_at = []  # iterations at which the box moved (the state went through set_state)
        self._since_plan = 0
        self._sim = None
        self._box = None
        # float32 inputs (the reference's element type) go to the device as they are and are widened
        # there; anything else as float64
        pos, f = np.asarray(pos_m), np.asarray(f_m)
        dt = np.float32 if pos.dtype == np.float32 and f.dtype == np.float32 else np.float64
        pos = np.ascontiguousarray(pos, dtype=dt).reshape(-1, self.lattice.D)
        f = np.ascontiguousarray(f, dtype=dt).reshape(-1, self.lattice.Q)
        if self.fixed_box:
            lo = np.floor(np.asarray(box[0], dtype=np.float64) / self.cell).astype(int)
            hi = np.ceil(np.asarray(box[1], dtype=np.float64) / self.cell).astype(int)
            self._make(lo, hi, len(pos))
        else:
            self._plan(pos, len(pos))
        self._sim.set_state(None, pos, f)

    # ---- box planning ---------------------------------------------------------------------------
    def _growth(self) -> float:
        cmax = float(np.linalg.norm(self.lattice.C, axis=1).max()) * self.dx
        return (self.replan_every + 1) * cmax + self.r_res + 2 * self.cell

    def _make(self, lo, hi, m):
        dims = tuple(int(v) for v in (hi - lo))
        inst = Instance(dims=dims, origin=tuple(int(v) for v in lo), periodic=self.periodic, tau=self.tau,
                        rho_rest=self.rho_rest)
        cap = max(int(m), int(np.prod(dims)))
        if self._sim is not None:
            self._sim.close()
        self._sim = Simulation([inst], lattice=self.lattice, precision=self.precision, dx=self.dx, r_res=self.r_res,
                               cell=self.cell, kappa_hard=self.kappa_hard, moment_capacity=cap, graphs=self.graphs,
                               device=self.device)
        self._box = (np.asarray(lo), np.asarray(hi))

    def _plan(self, pos, m):
        """Box around the points `pos` (or any array whose rows span them, such as the (2, D)
        bounding box) for m moments."""
        if len(pos) == 0:
            lo = np.zeros(self.lattice.D)
            hi = np.zeros(self.lattice.D)
        else:
            lo, hi = pos.min(axis=0).astype(np.float64), pos.max(axis=0).astype(np.float64)
        g = self._growth()
        span = max(float((hi - lo).max()), 1.0)
        margin = g + 0.25 * span  # slack so that steady growth does not re-plan every time
        blo = np.floor((lo - margin) / self.cell).astype(int)
        bhi = np.ceil((hi + margin) / self.cell).astype(int)
        self._make(blo, bhi, m)

    def _maybe_replan(self):
        """Every replan_every steps: the bounding box of the moments, reduced on the device (2 D
        numbers reach the host), against the box; a re-plan moves the state device to device."""
        if self.fixed_box or self._since_plan < self.replan_every:
            return
        self._since_plan = 0
        self._sim.check_status()  # the steps since the last planning point, read once
        _, pos, f = self._sim.state()
        if pos.shape[0] == 0:
            return
        ext = torch.stack([pos.amin(0), pos.amax(0)]).cpu().numpy()
        g = self._growth()
        lo_c = np.floor((ext[0] - g) / self.cell)
        hi_c = np.ceil((ext[1] + g) / self.cell)
        blo, bhi = self._box
        if np.all(lo_c >= blo) and np.all(hi_c <= bhi):
            return
        self._plan(ext, pos.shape[0])
        self._sim.set_state(None, pos, f)
        self.replanned_at.append(self.iteration)

    # ---- reference API -----------------------------------------------------------------------------
    def step(self):
        """One step, queued without a host wait: the device status (out-of-box, non-finite) is read
        at the next planning point or state read, which raise on a bad bit."""
        self._maybe_replan()
        self._sim.step(1)
        self.iteration += 1
        self._since_plan += 1

    def check(self):
        """Raise if any step so far set a device status bit (host wait)."""
        self._sim.check_status()

    def moments(self):
        """(positions (N, D) FP32, f (N, Q) FP32) as numpy, rounded to float32 on the device."""
        self._sim.check_status()
        _, pos, f = self._sim.state(dtype=torch.float32)
        return pos.cpu().numpy(), f.cpu().numpy()

    @property
    def pos_m(self):
        self._sim.check_status()
        _, pos, _ = self._sim.state(dtype=torch.float32)
        return DeviceArray(pos)

    @property
    def f_m(self):
        self._sim.check_status()
        _, _, f = self._sim.state(dtype=torch.float32)
        return DeviceArray(f)

    @property
    def simulation(self) -> Simulation:
        return self._sim


__all__ = ["GpuSimulator"]
