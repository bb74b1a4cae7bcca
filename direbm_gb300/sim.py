"""Batched DiReBM simulation on one GPU (host side of the fused CUDA step).

``Simulation`` owns a ``dbm_sim`` handle (include/direbm_gb300.h): a batch of independent
instances -- each a box of cells, periodic or bounded, with its own tau and rest density --
advanced together by the fused step kernels.  It is the engine behind the drop-in
``direbm_gb300.warp.GpuSimulator`` (the reference's direbm/warp/simulator.py:25-77) and behind
the batched-ensemble benchmark.

Parameters follow the reference's names (dx, kappa_hard, rho_rest, tau) plus the
generalisations the benchmark configurations need: ``r_res`` (resampling radius; reference: dx),
``cell`` (thinning cell; reference: dx/alpha), ``lattice`` and ``precision``.
"""

from __future__ import annotations

import ctypes
from dataclasses import dataclass

import numpy as np
import torch

from . import _lib
from .lattices import get as get_lattice


@dataclass
class Instance:
    """One independent simulation box: ``dims`` cells per axis, world origin ``origin`` (cells)."""

    dims: tuple
    origin: tuple = (0, 0, 0)
    periodic: bool = True
    tau: float = 0.6
    rho_rest: float = 1.0
    obstacle: tuple | None = None  # (center (D,) world, radius world): solid sphere/disc, bounce-back
    inflow: tuple | None = None  # (u (D,), width in cells): inflow layer at the low-x face


_PREC = {"fp64": _lib.FP64, "fp32dev": _lib.FP32DEV, "fp32": _lib.FP32DEV}


def _require_cuda(device=None) -> torch.device:
    if not torch.cuda.is_available():
        raise _lib.DbmError("a CUDA device is required (the DiReBM kernels have no CPU path)")
    dev = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
    if dev.type != "cuda":
        raise _lib.DbmError(f"device {dev} is not a CUDA device")
    return dev


def _is_f32(a) -> bool:
    return getattr(a, "dtype", None) in (torch.float32, np.float32)


def _stream():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


class Simulation:
    def __init__(
        self,
        instances,
        *,
        lattice="D2Q9",
        precision="fp32dev",
        dx: float = 1.0,
        r_res: float | None = None,
        cell: float | None = None,
        alpha: float = 4.0,
        kappa_hard: int = 4,
        eps: float = 1e-6,
        moment_capacity: int = 0,
        graphs: bool = True,
        tiles: bool = True,
        kappa_soft: int = 0,
        device=None,
    ):
        self.device = _require_cuda(device)
        self.lib = _lib.load()
        self.lattice = get_lattice(lattice)
        if precision not in _PREC:
            raise ValueError(f"precision must be one of {sorted(_PREC)}")
        self.precision = "fp64" if _PREC[precision] == _lib.FP64 else "fp32dev"
        self.dx = float(dx)
        self.r_res = float(dx if r_res is None else r_res)
        self.cell = float(dx / alpha if cell is None else cell)
        self.kappa_hard = int(kappa_hard)
        self.eps = float(eps)
        self.instances = [inst if isinstance(inst, Instance) else Instance(**inst) for inst in instances]
        D = self.lattice.D
        self.ncells = int(sum(int(np.prod(inst.dims)) for inst in self.instances))
        self.kappa_soft = int(kappa_soft)
        if self.kappa_soft > 0:  # up to one spawned control point per thinning cell
            moment_capacity = max(int(moment_capacity), 2 * self.ncells)
        self.capacity = max(int(moment_capacity), self.ncells)  # rows of each state buffer
        desc = _lib.SimDesc(
            lattice=self.lattice.id, precision=_PREC[precision], dx=self.dx, r_res=self.r_res,
            cell=self.cell, kappa_hard=self.kappa_hard, eps=self.eps, moment_capacity=int(moment_capacity),
        )
        arr = (_lib.InstanceDesc * len(self.instances))()
        for i, inst in enumerate(self.instances):
            dims = tuple(int(v) for v in inst.dims)
            if len(dims) != D:
                raise ValueError(f"instance {i}: dims must have {D} entries")
            org = tuple(int(v) for v in inst.origin)[:D] + (0,) * (3 - D)
            arr[i].dims[:] = list(dims) + [1] * (3 - D)
            arr[i].origin[:] = list(org[:3])
            arr[i].periodic = 1 if inst.periodic else 0
            arr[i].tau = float(inst.tau)
            arr[i].rho_rest = float(inst.rho_rest)
        h = ctypes.c_void_p()
        with torch.cuda.device(self.device):
            _lib.check(self.lib.dbm_sim_create(ctypes.byref(desc), arr, len(self.instances), ctypes.byref(h)),
                       "dbm_sim_create")
        self._h = h
        _lib.check(self.lib.dbm_sim_set_option(self._h, 1, 1 if graphs else 0), "dbm_sim_set_option")
        _lib.check(self.lib.dbm_sim_set_option(self._h, 2, 1 if tiles else 0), "dbm_sim_set_option")
        if self.kappa_soft > 0:
            self.set_soft_spawn(self.kappa_soft)
        self.iteration = 0
        for i, inst in enumerate(self.instances):
            if inst.obstacle is not None:
                self.set_obstacle(i, *inst.obstacle)
            if inst.inflow is not None:
                self.set_inflow(i, *inst.inflow)

    # ---- lifecycle ------------------------------------------------------------------------------
    def close(self):
        if getattr(self, "_h", None):
            self.lib.dbm_sim_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self):
        return self._h

    @property
    def device_bytes(self) -> int:
        return int(self.lib.dbm_sim_device_bytes(self._h))

    # ---- state ----------------------------------------------------------------------------------
    def set_state(self, inst, pos, f, check: bool = True, presorted: bool = False):
        """Load moments: instance index (M,), world positions (M, D), distributions (M, Q).  With
        ``check=False`` the call does not wait for the load to finish: a moment outside its box then
        leaves the bad-input bit in ``status()`` (``check_status()`` raises on it) instead of raising
        here, so a caller that pipelines loads and steps keeps the device busy.  ``presorted=True``
        declares the moments in cell order (by instance, then cell: the order ``state()`` returns)
        and skips the sort; the state is the same, and a moment out of order sets the bad-input
        bit.  Positions and f both float32 (the reference GPU simulator's arrays) go to the device
        as they are and are widened there; anything else is converted to float64."""
        dev = self.device
        f32 = _is_f32(pos) and _is_f32(f)
        dt = torch.float32 if f32 else torch.float64
        pos = torch.as_tensor(pos, dtype=dt, device=dev).contiguous()
        f = torch.as_tensor(f, dtype=dt, device=dev).contiguous()
        M = int(pos.shape[0])
        if inst is None:
            inst = torch.zeros(M, dtype=torch.int32, device=dev)
        inst = torch.as_tensor(inst, dtype=torch.int32, device=dev).contiguous()
        if pos.shape != (M, self.lattice.D) or f.shape != (M, self.lattice.Q) or inst.shape != (M,):
            raise ValueError("set_state: expected inst (M,), pos (M, D), f (M, Q)")
        with torch.cuda.device(dev):
            if f32:
                name = "dbm_sim_set_state_f32"
                rc = self.lib.dbm_sim_set_state_f32(self._h, inst.data_ptr(), pos.data_ptr(), f.data_ptr(), M,
                                                    1 if presorted else 0, _stream())
            else:
                name = "dbm_sim_set_state_sorted" if presorted else "dbm_sim_set_state"
                rc = getattr(self.lib, name)(self._h, inst.data_ptr(), pos.data_ptr(), f.data_ptr(), M, _stream())
            _lib.check(rc, name)
            st = self.status(clear=True) if check else 0
        if st & _lib.ST_BAD_INPUT:
            raise _lib.DbmError("set_state: a moment lies outside its instance box"
                                + (" or out of cell order" if presorted else ""))
        self.iteration = 0

    def step(self, n: int = 1):
        with torch.cuda.device(self.device):
            _lib.check(self.lib.dbm_sim_step(self._h, int(n), _stream()), "dbm_sim_step")
        self.iteration += int(n)

    def step_partial(self, stage: int):
        with torch.cuda.device(self.device):
            _lib.check(self.lib.dbm_sim_step_partial(self._h, int(stage), _stream()), "dbm_sim_step_partial")
        if stage >= 6:
            self.iteration += 1

    STAGES = ("collide", "thin_refine", "sort", "weights", "gather", "emit")

    def profile_step(self) -> dict:
        """Advance one step stage by stage and return {stage: milliseconds} (CUDA events)."""
        ms = (ctypes.c_float * 6)()
        with torch.cuda.device(self.device):
            _lib.check(self.lib.dbm_sim_profile_step(self._h, ms, _stream()), "dbm_sim_profile_step")
        self.iteration += 1
        return dict(zip(self.STAGES, [float(v) for v in ms]))

    def count(self) -> int:
        m = ctypes.c_int64()
        with torch.cuda.device(self.device):
            _lib.check(self.lib.dbm_sim_count(self._h, ctypes.byref(m), _stream()), "dbm_sim_count")
        return int(m.value)

    def state(self, out=None, dtype=torch.float64):
        """(instance (M,) int32, positions (M, D), f (M, Q)) as CUDA tensors of ``dtype`` (float64,
        or float32: the state rounded once on the device).  With ``out`` = (inst, pos, f),
        contiguous CUDA tensors of at least M rows (pos and f both float64 or both float32), the
        state is written into their first M rows and those views are returned (no allocation)."""
        M = self.count()
        dev = self.device
        if out is not None:
            self._check_out(out, M, "state(out=...)")
            inst, pos, f = (o[:M] for o in out)
        else:
            if dtype not in (torch.float64, torch.float32):
                raise ValueError("state: dtype must be torch.float64 or torch.float32")
            D, Q = self.lattice.D, self.lattice.Q
            inst = torch.empty(M, dtype=torch.int32, device=dev)
            pos = torch.empty((M, D), dtype=dtype, device=dev)
            f = torch.empty((M, Q), dtype=dtype, device=dev)
        if M:
            self._export(inst, pos, f)
        return inst, pos, f

    def _check_out(self, out, rows, what):
        oi, op, of = out
        D, Q = self.lattice.D, self.lattice.Q
        ok = (oi.is_cuda and op.is_cuda and of.is_cuda and oi.dtype == torch.int32 and op.dtype == of.dtype
              and op.dtype in (torch.float64, torch.float32) and oi.is_contiguous() and op.is_contiguous()
              and of.is_contiguous() and oi.shape[0] >= rows and op.shape[0] >= rows and of.shape[0] >= rows
              and tuple(op.shape[1:]) == (D,) and tuple(of.shape[1:]) == (Q,))
        if not ok:
            raise ValueError(f"{what}: need contiguous CUDA int32 (>= {rows},), and fp64 or fp32 (>= {rows}, {D}) "
                             f"and (>= {rows}, {Q}) of one dtype")

    def _export(self, inst, pos, f):
        name = "dbm_sim_get_state_f32" if pos.dtype == torch.float32 else "dbm_sim_get_state"
        with torch.cuda.device(self.device):
            _lib.check(getattr(self.lib, name)(self._h, inst.data_ptr(), pos.data_ptr(), f.data_ptr(), _stream()), name)

    def state_numpy(self):
        inst, pos, f = self.state()
        return inst.cpu().numpy(), pos.cpu().numpy(), f.cpu().numpy()

    def state_into(self, out):
        """Write the state into ``out`` = (inst, pos, f): contiguous CUDA int32 (>= capacity,) and
        fp64 or fp32 (>= capacity, D) and (>= capacity, Q) buffers.  Unlike ``state()`` this does
        not wait for the step to finish (it needs no row count on the host): once the caller's
        stream reaches this point, rows [0, count()) hold the state, in its sorted order."""
        self._check_out(out, self.capacity, "state_into")
        self._export(*out)
        return out

    def status(self, clear: bool = False) -> int:
        v = ctypes.c_uint32()
        with torch.cuda.device(self.device):
            _lib.check(self.lib.dbm_sim_status(self._h, ctypes.byref(v), 1 if clear else 0, _stream()), "dbm_sim_status")
        return int(v.value)

    def check_status(self):
        st = self.status(clear=False)
        if st:
            names = [n for n, b in (("out_of_box", 1), ("capacity", 2), ("nonfinite", 4), ("bad_input", 8),
                                    ("internal", 16)) if st & b]
            raise _lib.DbmError(f"device status: {', '.join(names)}")

    def conservation(self) -> torch.Tensor:
        """Per-instance FP64 (mass, momentum...) of the current state, shape (n_inst, 1 + D)."""
        out = torch.empty((len(self.instances), 1 + self.lattice.D), dtype=torch.float64, device=self.device)
        with torch.cuda.device(self.device):
            _lib.check(self.lib.dbm_sim_conservation(self._h, out.data_ptr(), _stream()), "dbm_sim_conservation")
        return out

    def trace(self, name: str) -> torch.Tensor:
        """Copy an internal buffer (see include/direbm_gb300.h DBM_TRACE_*) into a uint8 tensor."""
        what = _lib.TRACE[name]
        need = ctypes.c_int64()
        with torch.cuda.device(self.device):
            _lib.check(self.lib.dbm_sim_trace(self._h, what, None, 0, ctypes.byref(need), _stream()), "dbm_sim_trace")
            buf = torch.empty(int(need.value), dtype=torch.uint8, device=self.device)
            _lib.check(self.lib.dbm_sim_trace(self._h, what, buf.data_ptr(), buf.numel(), ctypes.byref(need), _stream()),
                       "dbm_sim_trace")
        return buf

    # ---- obstacles and inflow --------------------------------------------------------------------
    def set_obstacle(self, inst: int, center, radius: float):
        """Solid sphere (disc in 2D) with bounce-back in instance `inst` (world units); radius <= 0
        removes it."""
        c = np.ascontiguousarray(np.asarray(center, dtype=np.float64).reshape(-1))
        if c.shape[0] != self.lattice.D:
            raise ValueError(f"center needs {self.lattice.D} coordinates")
        with torch.cuda.device(self.device):
            _lib.check(self.lib.dbm_sim_set_obstacle(self._h, int(inst), c.ctypes.data, float(radius)),
                       "dbm_sim_set_obstacle")
        self.instances[inst].obstacle = (tuple(c), float(radius)) if radius > 0 else None

    def set_inflow(self, inst: int, u, width: int):
        """Inflow layer: moments in the first `width` cell columns of instance `inst` are set to the
        equilibrium at velocity u with their own density; width 0 removes it."""
        v = np.ascontiguousarray(np.asarray(u, dtype=np.float64).reshape(-1))
        if v.shape[0] != self.lattice.D:
            raise ValueError(f"u needs {self.lattice.D} components")
        with torch.cuda.device(self.device):
            _lib.check(self.lib.dbm_sim_set_inflow(self._h, int(inst), v.ctypes.data, int(width)), "dbm_sim_set_inflow")
        self.instances[inst].inflow = (tuple(v), int(width)) if width > 0 else None

    # ---- launch configuration -------------------------------------------------------------------
    OPT_TILE_WIDTH, OPT_PERSISTENT, OPT_KAPPA_SOFT, OPT_BRICK_WIDTH, OPT_SHIFTED_WINDOWS = 3, 4, 5, 6, 7
    OPT_DENSE_STENCIL = 8

    def tiling(self) -> tuple:
        """(tile width in cells, persistent launches) of the 2D tiled kernels."""
        w, p = ctypes.c_int32(), ctypes.c_int32()
        _lib.check(self.lib.dbm_sim_get_tiling(self._h, ctypes.byref(w), ctypes.byref(p)), "dbm_sim_get_tiling")
        return int(w.value), bool(p.value)

    def set_tiling(self, tile_width: int | None = None, persistent: bool | None = None):
        """Tiles of tile_width x 256/tile_width cells and/or persistent launches (2D only).  Results
        are bit-identical for every setting; only the speed changes."""
        with torch.cuda.device(self.device):
            if tile_width is not None:
                _lib.check(self.lib.dbm_sim_set_option(self._h, self.OPT_TILE_WIDTH, int(tile_width)), "set tile width")
            if persistent is not None:
                _lib.check(self.lib.dbm_sim_set_option(self._h, self.OPT_PERSISTENT, 1 if persistent else 0),
                           "set persistent")

    def set_shifted_windows(self, on: bool):
        """2D FP32 store with whole-cell displacements (D2Q9, dx = cell) and r < 2 cells: build one
        table of window rows per reference point and shift it per direction (default on).  Results
        are bit-identical either way; only the speed changes."""
        with torch.cuda.device(self.device):
            _lib.check(self.lib.dbm_sim_set_option(self._h, self.OPT_SHIFTED_WINDOWS, 1 if on else 0),
                       "set shifted windows")

    def set_dense_stencil(self, on: bool):
        """With the shifted windows: stage a tile whose cells each hold at most one moment and one
        control point as a dense grid and run every window as a fixed 4 x 4 block of cells (default
        on); other tiles take the row-segment loops.  Results are bit-identical either way."""
        with torch.cuda.device(self.device):
            _lib.check(self.lib.dbm_sim_set_option(self._h, self.OPT_DENSE_STENCIL, 1 if on else 0),
                       "set dense stencil")

    def brick_width(self) -> int:
        """Cells along x of the 256-cell bricks the untiled window kernels give each block."""
        w = ctypes.c_int32()
        _lib.check(self.lib.dbm_sim_get_brick_width(self._h, ctypes.byref(w)), "dbm_sim_get_brick_width")
        return int(w.value)

    def set_brick_width(self, width: int):
        """Bricks of width x (256 / width) cells (2D) or width x by x bz (3D) for the untiled window
        kernels (3D, obstacles, the soft spawn, tiles off).  Results are bit-identical for every
        width; only the speed changes."""
        with torch.cuda.device(self.device):
            _lib.check(self.lib.dbm_sim_set_option(self._h, self.OPT_BRICK_WIDTH, int(width)), "set brick width")

    def set_soft_spawn(self, kappa_soft: int):
        """Soft-outer spawn (the CPU simulator's soft_mode="spawn", direbm/reference/simulator.py:
        126-166): control points with kappa_hard < kappa <= kappa_soft also emit one new control
        point 2(1 - sqrt(3)/2) dx ahead along their components' mean direction.  0 turns it off.
        Needs moment_capacity >= 2 x cells (the constructor's kappa_soft sets that up)."""
        with torch.cuda.device(self.device):
            _lib.check(self.lib.dbm_sim_set_option(self._h, self.OPT_KAPPA_SOFT, int(kappa_soft)), "set kappa_soft")
        self.kappa_soft = int(kappa_soft)

    # ---- parameters, checkpoints ----------------------------------------------------------------
    def set_tau(self, tau):
        """Replace every instance's tau (one value per instance, each > 1/2)."""
        t = np.ascontiguousarray(np.asarray(tau, dtype=np.float64).reshape(-1))
        if t.shape[0] != len(self.instances):
            raise ValueError(f"set_tau: expected {len(self.instances)} values")
        with torch.cuda.device(self.device):
            _lib.check(self.lib.dbm_sim_set_tau(self._h, t.ctypes.data, len(t)), "dbm_sim_set_tau")
        for inst, v in zip(self.instances, t):
            inst.tau = float(v)

    def snapshot(self) -> torch.Tensor:
        """The current state as a device blob (uint8 tensor); ``restore`` makes it current again."""
        need = ctypes.c_int64()
        with torch.cuda.device(self.device):
            _lib.check(self.lib.dbm_sim_snapshot(self._h, None, 0, ctypes.byref(need), _stream()), "dbm_sim_snapshot")
            blob = torch.empty(int(need.value), dtype=torch.uint8, device=self.device)
            _lib.check(self.lib.dbm_sim_snapshot(self._h, blob.data_ptr(), blob.numel(), ctypes.byref(need), _stream()),
                       "dbm_sim_snapshot")
        return blob

    def restore(self, blob: torch.Tensor, iteration: int | None = None):
        with torch.cuda.device(self.device):
            _lib.check(self.lib.dbm_sim_restore(self._h, blob.data_ptr(), blob.numel(), _stream()), "dbm_sim_restore")
        if iteration is not None:
            self.iteration = int(iteration)

    def import_order(self, m: int) -> torch.Tensor:
        """After ``set_state`` (before any step): input index of each sorted moment, int64 (m,)."""
        buf = self.trace("import_order")
        return buf.view(torch.int32)[:m].to(torch.int64)
