"""Reverse mode of the DiReBM step: a recorded tape, hand-written CUDA vector-Jacobian products,
and a ``torch.autograd.Function`` over a whole rollout with checkpoints.

The reference has no derivative of its step (differentiation is future work in the reference,
idea.md:250).  Here the step's discrete structure -- thinning membership, refine decisions,
resampling and gap-fill neighbour lists, sort order -- is recorded while the step runs
(``dbm_tape_step``) and held fixed; ``dbm_tape_backward`` applies the transpose of the step's
Jacobian for that structure (collision, dispersion, thinning centroids, the exp(f)-weighted refine
move, the (r - d)/sum(r - d) resampling weights and the gap fill).

``rollout`` runs ``steps`` steps forward with the simulator's own captured graphs and keeps a
device snapshot every ``checkpoint_every`` steps; its backward replays each segment from its
snapshot with the tape recording, then walks the segment's steps in reverse.  Memory is one
segment of tape plus the snapshots.
"""

from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import _lib
from .sim import Simulation, _stream


class TapeOverflow(_lib.DbmError):
    """A neighbour list outgrew the tape's estimate: restore the state of the first recorded step,
    clear the tape and record again (the estimate has grown, so the next recording fits)."""


def _check_tape(rc: int, what: str):
    if rc == 3:  # DBM_ERR_CAPACITY
        msg = _lib.load().dbm_last_error().decode()
        raise TapeOverflow(f"{what}: {msg}")
    _lib.check(rc, what)


class Tape:
    """Recorded steps of one ``Simulation`` (``dbm_tape``)."""

    def __init__(self, sim: Simulation):
        self.sim = sim
        self.lib = sim.lib
        h = ctypes.c_void_p()
        with torch.cuda.device(sim.device):
            _lib.check(self.lib.dbm_tape_create(sim.handle, ctypes.byref(h)), "dbm_tape_create")
        self._h = h
        self._counts = []
        self._twin = None

    def twin(self) -> "Tape":
        """A second tape of the same simulator (created once, kept with this one): the rollout's
        backward records one segment on one tape while the other tape's segment runs its VJPs."""
        if self._twin is None:
            self._twin = Tape(self.sim)
        return self._twin

    def close(self):
        if getattr(self, "_twin", None) is not None:
            self._twin.close()
            self._twin = None
        if getattr(self, "_h", None):
            self.lib.dbm_tape_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def clear(self):
        _lib.check(self.lib.dbm_tape_clear(self._h), "dbm_tape_clear")
        self._counts = []

    def step(self):
        """Advance the simulator one step and record it."""
        with torch.cuda.device(self.sim.device):
            _check_tape(self.lib.dbm_tape_step(self._h, _stream()), "dbm_tape_step")
        self.sim.iteration += 1
        self._counts.append(None)

    def set_estimate(self, pairs_per_row: float):
        """Initial list-size estimate (pairs per row; grown as steps are recorded)."""
        _lib.check(self.lib.dbm_tape_set_estimate(self._h, float(pairs_per_row)), "dbm_tape_set_estimate")

    def record(self, n: int):
        """Advance the simulator n steps, recording each."""
        with torch.cuda.device(self.sim.device):
            _check_tape(self.lib.dbm_tape_record(self._h, int(n), _stream()), "dbm_tape_record")
        self.sim.iteration += int(n)
        self._counts.extend([None] * int(n))  # read on first use (reading settles the tape)

    def backward_all(self, g_off_out: torch.Tensor, g_f_out: torch.Tensor, g_tau: torch.Tensor):
        """Every recorded step in reverse: cotangents of the last step's output -> those of the first
        step's input; d loss / d tau added into g_tau."""
        n = len(self._counts)
        if n == 0:
            raise ValueError("nothing recorded")
        sim = self.sim
        D, Q, dev = sim.lattice.D, sim.lattice.Q, sim.device
        last, first = self.counts(n - 1), self.counts(0)
        g_off_out = g_off_out.to(device=dev, dtype=torch.float64).contiguous()
        g_f_out = g_f_out.to(device=dev, dtype=torch.float64).contiguous()
        if g_off_out.shape != (last["P"], D) or g_f_out.shape != (last["P"], Q):
            raise ValueError(f"expected cotangents ({last['P']}, {D}) and ({last['P']}, {Q})")
        if g_tau.dtype != torch.float64 or not g_tau.is_contiguous() or g_tau.device != dev:
            raise ValueError("g_tau must be a contiguous FP64 tensor on the simulator's device")
        g_off_in = torch.empty((first["M"], D), dtype=torch.float64, device=dev)
        g_f_in = torch.empty((first["M"], Q), dtype=torch.float64, device=dev)
        with torch.cuda.device(dev):
            _check_tape(self.lib.dbm_tape_backward_all(self._h, g_off_out.data_ptr(), g_f_out.data_ptr(),
                                                       g_off_in.data_ptr(), g_f_in.data_ptr(), g_tau.data_ptr(),
                                                       _stream()), "dbm_tape_backward_all")
        return g_off_in, g_f_in

    def __len__(self) -> int:
        return int(self.lib.dbm_tape_length(self._h))

    def _query_counts(self, i: int) -> dict:
        c = (ctypes.c_int64 * 8)()
        _check_tape(self.lib.dbm_tape_counts(self._h, int(i), c), "dbm_tape_counts")
        return {"M": c[0], "P": c[1], "refine": c[2], "resample": c[3], "gapfill": c[4]}

    def counts(self, i: int) -> dict:
        """Moments in (M), control points out (P) and the pair counts of recorded step i."""
        if 0 <= i < len(self._counts):
            if self._counts[i] is None:
                self._counts[i] = self._query_counts(i)
            return self._counts[i]
        return self._query_counts(i)

    def backward(self, i: int, g_off_out: torch.Tensor, g_f_out: torch.Tensor, g_tau: torch.Tensor):
        """Cotangents of step i's output (offsets (P, D) in cell units, f (P, Q)) -> those of its
        input (M, D), (M, Q); d loss / d tau is added into g_tau (n_inst,).  All FP64 CUDA tensors."""
        c = self.counts(i)
        sim = self.sim
        D, Q = sim.lattice.D, sim.lattice.Q
        dev = sim.device
        if g_off_out.dtype != torch.float64 or not g_off_out.is_contiguous() or g_off_out.device != dev:
            g_off_out = g_off_out.to(device=dev, dtype=torch.float64).contiguous()
        if g_f_out.dtype != torch.float64 or not g_f_out.is_contiguous() or g_f_out.device != dev:
            g_f_out = g_f_out.to(device=dev, dtype=torch.float64).contiguous()
        if g_off_out.shape != (c["P"], D) or g_f_out.shape != (c["P"], Q):
            raise ValueError(f"tape backward {i}: expected cotangents ({c['P']}, {D}) and ({c['P']}, {Q})")
        if g_tau.dtype != torch.float64 or not g_tau.is_contiguous() or g_tau.device != dev:
            raise ValueError("g_tau must be a contiguous FP64 tensor on the simulator's device")
        g_off_in = torch.empty((c["M"], D), dtype=torch.float64, device=dev)
        g_f_in = torch.empty((c["M"], Q), dtype=torch.float64, device=dev)
        with torch.cuda.device(dev):
            _lib.check(self.lib.dbm_tape_backward(self._h, int(i), g_off_out.data_ptr(), g_f_out.data_ptr(),
                                                  g_off_in.data_ptr(), g_f_in.data_ptr(), g_tau.data_ptr(), _stream()),
                       "dbm_tape_backward")
        return g_off_in, g_f_in

    def export(self, i: int) -> dict:
        """Every recorded array of step i as numpy (see ``_lib.TAPE``), with D/Q-major arrays
        transposed to (n, D) / (n, Q)."""
        c = self.counts(i)
        sim = self.sim
        D, Q = sim.lattice.D, sim.lattice.Q
        sizes = {"M": c["M"], "P": c["P"], "QM": Q * c["M"], "DM": D * c["M"], "DP": D * c["P"], "P+1": c["P"] + 1,
                 "PQ+1": c["P"] * Q + 1, "nref": c["refine"], "Dnref": D * c["refine"], "nres": c["resample"],
                 "Dnres": D * c["resample"], "ngap": c["gapfill"], "Dngap": D * c["gapfill"],
                 "I+1": len(sim.instances) + 1}
        out = {"counts": c}
        for name, (what, dt, kind) in _lib.TAPE.items():
            n = sizes[kind]
            tdt = torch.float64 if dt == "f64" else torch.int32
            buf = torch.empty(max(n, 1), dtype=tdt, device=sim.device)
            need = ctypes.c_int64()
            with torch.cuda.device(sim.device):
                _lib.check(self.lib.dbm_tape_export(self._h, int(i), what, buf.data_ptr(), buf.numel() * buf.element_size(),
                                                    ctypes.byref(need), _stream()), "dbm_tape_export")
            a = buf[:n].cpu().numpy()
            if dt == "u32":
                a = a.view(np.uint32).astype(np.int64)
            if kind.startswith("D"):
                a = a.reshape(D, -1).T.copy()
            elif kind == "QM":
                a = a.reshape(Q, -1).T.copy()
            out[name] = a
        return out


class _Rollout(torch.autograd.Function):
    @staticmethod
    def forward(ctx, pos, f, tau, sim, tape, inst, steps, every, overlap):
        taus = tau.detach().to("cpu", torch.float64).numpy()
        sim.set_tau(taus)
        sim.set_state(inst, pos.detach(), f.detach())
        order = sim.import_order(pos.shape[0])
        snaps = []
        for s in range(steps):
            if s % every == 0:
                snaps.append(sim.snapshot())
            sim.step(1)
        final = sim.snapshot()
        inst_t, pos_t, f_t = sim.state()
        ctx.sim, ctx.tape, ctx.steps, ctx.every, ctx.overlap = sim, tape, steps, every, overlap
        ctx.snaps, ctx.final, ctx.taus = snaps, final, taus
        ctx.save_for_backward(order)
        ctx.mark_non_differentiable(inst_t)
        return inst_t, pos_t, f_t

    @staticmethod
    def backward(ctx, g_inst, g_pos, g_f):
        sim, tape = ctx.sim, ctx.tape
        (order,) = ctx.saved_tensors
        dev = sim.device
        D, Q = sim.lattice.D, sim.lattice.Q
        P = g_f.shape[0] if g_f is not None else g_pos.shape[0]
        g_off = (g_pos * sim.cell if g_pos is not None else torch.zeros((P, D), dtype=torch.float64, device=dev))
        g_f = g_f if g_f is not None else torch.zeros((P, Q), dtype=torch.float64, device=dev)
        g_tau = torch.zeros(len(sim.instances), dtype=torch.float64, device=dev)
        sim.set_tau(ctx.taus)
        nseg = len(ctx.snaps)
        # Two tapes, two streams: segment s is recorded (with one host synchronisation per step)
        # on the simulator's stream while the VJPs of segment s + 1 run from the other tape on a
        # second stream, so the VJP kernels fill the recording's gaps.  Each tape's VJPs read only
        # that tape, and a tape is cleared for its next segment only after its VJPs have finished;
        # the arithmetic is the same as one tape on one stream, bit for bit.
        overlap = ctx.overlap and nseg > 1
        tapes = [tape, tape.twin()] if overlap else [tape]
        main = torch.cuda.current_stream(dev)
        vjp = torch.cuda.Stream(device=dev) if overlap else main
        vjp.wait_stream(main)  # the output cotangents and g_tau
        free = [None] * len(tapes)  # per tape: event after its last VJP launch
        for i, seg in enumerate(reversed(range(nseg))):
            s0 = seg * ctx.every
            s1 = min(s0 + ctx.every, ctx.steps)
            slot = i % len(tapes)
            t = tapes[slot]
            if free[slot] is not None:
                main.wait_event(free[slot])
            for attempt in range(3):
                sim.restore(ctx.snaps[seg], s0)
                t.clear()
                try:
                    t.record(s1 - s0)
                    vjp.wait_stream(main)
                    with torch.cuda.stream(vjp):
                        g_off, g_f = t.backward_all(g_off, g_f, g_tau)
                    if overlap:
                        free[slot] = torch.cuda.Event()
                        free[slot].record(vjp)
                    break
                except TapeOverflow:
                    if attempt == 2:
                        raise
        main.wait_stream(vjp)
        if vjp is not main:
            # g_off and g_f were allocated on the VJP stream and are read below on the main
            # stream: tell the caching allocator, so their blocks are not handed to a later
            # allocation on the VJP stream before the main stream's reads have run
            g_off.record_stream(main)
            g_f.record_stream(main)
        for t in tapes:
            t.clear()
        sim.restore(ctx.final, ctx.steps)
        g_pos_in = torch.empty_like(g_off)
        g_f_in = torch.empty_like(g_f)
        g_pos_in[order] = g_off / sim.cell
        g_f_in[order] = g_f
        return g_pos_in, g_f_in, g_tau, None, None, None, None, None, None


def rollout(sim: Simulation, inst, pos: torch.Tensor, f: torch.Tensor, tau: torch.Tensor, steps: int,
            checkpoint_every: int = 10, tape: Tape | None = None, overlap: bool = True):
    """Differentiable ``steps``-step rollout of ``sim`` from moments (inst (M,), world positions
    pos (M, D), f (M, Q)) with per-instance ``tau`` (n_inst,).  Returns (inst, pos, f) of the final
    state in its sorted order; gradients flow to pos, f and tau.  The simulator is left at the
    final state.  ``overlap`` records one segment while the previous one runs its VJPs, on a
    second tape (``tape.twin()``, twice the tape memory); the gradients are the same either way."""
    if steps < 1 or checkpoint_every < 1:
        raise ValueError("steps and checkpoint_every must be >= 1")
    dev = sim.device
    pos = torch.as_tensor(pos, dtype=torch.float64, device=dev)
    f = torch.as_tensor(f, dtype=torch.float64, device=dev)
    tau = torch.as_tensor(tau, dtype=torch.float64, device=dev).reshape(-1)
    if inst is None:
        inst = torch.zeros(pos.shape[0], dtype=torch.int32, device=dev)
    inst = torch.as_tensor(inst, dtype=torch.int32, device=dev)
    tape = tape if tape is not None else Tape(sim)
    return _Rollout.apply(pos, f, tau, sim, tape, inst, int(steps), int(checkpoint_every), bool(overlap))


# ---- the inverse-problem workload: initial velocity from Fourier-mode coefficients ---------------

class ModeField:
    """Divergence-free 2D field on a periodic square of side L from ``modes`` Fourier modes:
        u(x) = sum_j e_j (a_j cos(2 pi k_j . x / L) + b_j sin(2 pi k_j . x / L)),  e_j = k_j^perp / |k_j|,
    with integer wave vectors |k_j,a| <= 4 drawn from ``seed``.  ``coeffs`` = (a_1, b_1, ..., a_n, b_n);
    the seeded default coefficients are scaled to an RMS speed of ``u_rms`` on the points given."""

    def __init__(self, L: float, seed: int, modes: int = 8, u_rms: float = 0.02, points=None):
        rng = np.random.default_rng(seed)
        ks = []
        while len(ks) < modes:
            k = rng.integers(-4, 5, size=2).astype(np.float64)
            if k.any():
                ks.append(k)
        self.L = float(L)
        self.k = np.array(ks)
        self.e = np.stack([-self.k[:, 1], self.k[:, 0]], axis=1) / np.linalg.norm(self.k, axis=1)[:, None]
        c = rng.normal(size=2 * modes)
        if points is not None:
            u = self(torch.as_tensor(points, dtype=torch.float64), torch.as_tensor(c))
            rms = float(torch.sqrt((u * u).sum(1).mean()))
            c = c * (u_rms / max(rms, 1e-30))
        self.coeffs = c

    def __call__(self, x: torch.Tensor, coeffs) -> torch.Tensor:
        coeffs = torch.as_tensor(coeffs, dtype=torch.float64, device=x.device)
        k = torch.as_tensor(self.k, dtype=torch.float64, device=x.device)
        e = torch.as_tensor(self.e, dtype=torch.float64, device=x.device)
        ph = (2 * np.pi / self.L) * (x @ k.T)  # (M, modes)
        amp = coeffs[0::2] * torch.cos(ph) + coeffs[1::2] * torch.sin(ph)
        return amp @ e


def equilibrium(rho: torch.Tensor, u: torch.Tensor, lattice) -> torch.Tensor:
    """The second-order equilibrium (direbm/physics.py:29-45) in torch, differentiable."""
    C = torch.as_tensor(lattice.C, dtype=u.dtype, device=u.device)
    W = torch.as_tensor(lattice.W, dtype=u.dtype, device=u.device)
    inv = 1.0 / lattice.cs2
    cu = u @ C.T
    usq = (u * u).sum(1, keepdim=True)
    return rho[:, None] * W[None, :] * (1 + inv * cu + 0.5 * inv * inv * cu * cu - 0.5 * inv * usq)


def velocity(f: torch.Tensor, lattice) -> torch.Tensor:
    C = torch.as_tensor(lattice.C, dtype=f.dtype, device=f.device)
    return (f @ C) / f.sum(1, keepdim=True)


def inverse_problem_loss(sim: Simulation, x0: torch.Tensor, field: ModeField, coeffs: torch.Tensor, tau: torch.Tensor,
                         target: ModeField, steps: int, checkpoint_every: int = 10, tape: Tape | None = None,
                         overlap: bool = True):
    """L = mean over final moments of |u(f_T) - u*(x_T)|^2, u* the target field at the final
    positions; the initial moments sit at x0 with unit density and velocity field(x0; coeffs)."""
    rho0 = torch.ones(x0.shape[0], dtype=torch.float64, device=x0.device)
    f0 = equilibrium(rho0, field(x0, coeffs), sim.lattice)
    _, pos, f = rollout(sim, None, x0, f0, tau, steps, checkpoint_every, tape, overlap)
    du = velocity(f, sim.lattice) - target(pos, target.coeffs)
    return (du * du).sum(1).mean()
