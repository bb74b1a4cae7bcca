"""Benchmark: batched-ensemble DiReBM step on one GB300 (point-steps/s), one JSON line.

Workload (the batched-ensemble configuration): 256 independent periodic 2D D2Q9 runs in one
launch; point counts log-uniform in [4096, 262144] (seed 1); each run is a jittered grid (spacing
h = dx = 1, jitter U(+-0.25)) in a periodic square of side round(sqrt(M)); tau U(0.55, 1.0);
initial velocity = 8 random divergence-free Fourier modes (seed 100 + i) scaled to RMS 0.02;
resampling radius 1.5h, thinning cell h; FP32-deviation store; CUDA graphs.  Synthetic data
(no dataset is involved).  The state (~15.5 M moments, ~0.8 GB) is far larger than L2 (129 MB),
so L2 is not flushed between steps.

Keys beyond the base contract:
  roofline      dominant kernel's algorithmic bytes / its CUDA-event duration vs measured HBM peak
  step_roofline the whole step against the per-point-step byte model of the method
  full_run      the configuration's 100-step run from the initial state, mean and per 10 steps
  fp64          the same workload in the FP64 store (5 timed steps: GB300 FP64 is slow)
  accuracy      velocity L2 error vs the FP64 oracle on a 4096-point instance, and against the
                FP64 GPU step after 1/10/50/200 steps beside FP64 from the FP32-rounded start
  accuracy_ensemble  FP32DEV vs FP64 on the whole ensemble after 10 steps (same comparison)
  lbm           hexagonal D2Q7 shear wave 1024x1024 (FP32DEV and FP64), node-steps/s
  adjoint       inverse problem on 64k points, 100 steps, checkpoint every 10: adjoint steps/s, its
                cost relative to the forward step, FP32DEV gradient error vs FP64
  sphere        3D flow past a bounce-back sphere (D3Q19, ~2 M points, inflow), FP32DEV and FP64
  cpu_baseline  the CPU oracle (numpy restatement of the reference step) on the host cores, and
                the reference's own CPU simulator (one process and one per core)

Usage: python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
"""

from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

N_INST = 256
M_MIN, M_MAX = 4096, 262144
R_RES, CELL, DX = 1.5, 1.0, 1.0
U_RMS = 0.02
METRIC = "point-steps/s on 1 GB300, FP32 vs FP64 at equal L2 error; adjoint step/s"

# Algorithmic bytes per unit for the roofline, FP32DEV D2Q9 2D (Q = 9, D = 2): each input read
# once and each output written once; windows re-read from L1/L2 are not counted.
Q9, D2 = 9, 2
KERNEL_BYTES = {
    # per moment: read rho + dev (40) + cell (4) + offsets (8); per occupied cell: start (4),
    # write occupancy, refined cell, offsets (16)
    "thin_refine": ("moment+cell", 4 * (1 + Q9) + 4 + 4 * D2, 4 + 16),
    # per component: read offsets (8) + cell (4) once per moment, write sw (4); CP reads (12/CP)
    "weights": ("moment+cp", 4 * D2 + 4 + 4 * Q9, 12),
    # per moment: offsets + rho + dev + sw (8+4+36+36) + starts; per CP: cell+offsets (12) + cpf (72) + mask (4)
    "gather": ("moment+cp", 4 * D2 + 4 * (1 + Q9) + 4 * Q9 + 4, 12 + 8 * Q9 + 4),
    # per CP: read cpf (72) + mask (4) + cell/off (12); write rho + dev (40)
    "emit": ("cp", 0, 8 * Q9 + 4 + 12 + 4 * (1 + Q9)),
    # per moment: read rho + dev, write dev
    "collide": ("moment", 4 * (1 + Q9) + 4 + 4 * Q9, 0),
    # per CP, radix path: 3 passes x (hist read 4 + scatter read 8 + write 8) + compaction (8) +
    # finalize (24); the 2D tiled path places points without a sort and moves fewer bytes
    "sort": ("cp", 0, 3 * 20 + 8 + 24),
}

# DRAM bytes per input moment measured by ncu (dram__bytes_read.sum + dram__bytes_write.sum) for
# one launch of k_gather_ds (the dense-stencil gather this workload runs) on a 4.18 M-moment case
# of this workload (its first 64 members, 16x16 tiles): 419.6 MB read + 267.4 MB written.  Traffic
# grows with the moments, so a full launch's traffic is this times M.
KERNEL_TRAFFIC_PER_MOMENT = {"gather": 164.2}

# Per point-step byte model of the method (components materialised as 12-byte sort records):
# B = M(Qs+b_p) + Nc k_b + 2 Nc k_b + 3(Nc k_b + M(Qs+b_p)) + 3 P b_p + P(Qs+b_p), with P ~ M,
# s = 4, b_p = 8D (int cell + FP32 offset per axis), k_b = 12 -> 956 B for D2Q9 FP32.
def step_bytes_per_point(Q=9, D=2, s=4):
    bp = 8 * D
    kb = 12
    Nc = Q
    return (Q * s + bp) + Nc * kb + 2 * Nc * kb + 3 * (Nc * kb + (Q * s + bp)) + 3 * bp + (Q * s + bp)


# ---- workload ---------------------------------------------------------------------------------

def ensemble_spec(n_inst=N_INST, seed=1):
    rng = np.random.default_rng(seed)
    M = np.exp(rng.uniform(np.log(M_MIN), np.log(M_MAX), N_INST))[:n_inst]
    sides = np.maximum(np.round(np.sqrt(M)).astype(int), 16)
    taus = rng.uniform(0.55, 1.0, N_INST)[:n_inst]
    return sides, taus


def fourier_velocity(x, n, seed, modes=8, u_rms=U_RMS):
    rng = np.random.default_rng(seed)
    u = np.zeros_like(x)
    for _ in range(modes):
        k = np.zeros(2)
        while not k.any():
            k = rng.integers(-4, 5, size=2).astype(np.float64)
        e = np.array([-k[1], k[0]]) / np.linalg.norm(k)  # divergence-free direction
        phase = rng.uniform(0, 2 * np.pi)
        amp = rng.normal()
        u += amp * e[None, :] * np.sin(2 * np.pi * (x @ k) / n + phase)[:, None]
    rms = np.sqrt((u * u).sum(1).mean())
    return u * (u_rms / max(rms, 1e-30))


def instance_points(n, seed):
    rng = np.random.default_rng(seed)
    x = (np.indices((n, n)).reshape(2, -1).T[:, ::-1] + 0.5).astype(np.float64)
    x += rng.uniform(-0.25, 0.25, size=x.shape)
    return np.mod(x, n)


def build_ensemble(sides, taus, members=None):
    """Initial state of the ensemble members `members` (all by default): member i's points and
    velocity field come from seed 100 + i whatever shard it lands in; instance indices are local
    (0.. in the order of `members`)."""
    from direbm_gb300.lattices import D2Q9, equilibrium

    members = range(len(sides)) if members is None else members
    xs, fs, ib = [], [], []
    for li, i in enumerate(members):
        n = int(sides[i])
        x = instance_points(n, 100 + int(i))
        u = fourier_velocity(x, n, 100 + int(i))
        xs.append(x)
        fs.append(equilibrium(np.ones(len(x)), u, D2Q9))
        ib.append(np.full(len(x), li, dtype=np.int32))
    return np.concatenate(ib), np.concatenate(xs), np.concatenate(fs)


def make_sim(sides, taus, precision, cap, graphs=True, device=None):
    from direbm_gb300.sim import Instance, Simulation

    insts = [Instance(dims=(int(n), int(n)), periodic=True, tau=float(t)) for n, t in zip(sides, taus)]
    return Simulation(insts, lattice="D2Q9", precision=precision, dx=DX, r_res=R_RES, cell=CELL,
                      moment_capacity=cap, graphs=graphs, device=device)


# ---- clocks ------------------------------------------------------------------------------------

class ClockSampler:
    FIELDS = "clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown," \
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown," \
             "clocks_event_reasons.sw_power_cap"

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.lines = []
        self._t = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self._t = threading.Thread(target=self._read, daemon=True)
            self._t.start()
        except Exception:
            self.proc = None
        time.sleep(0.25)

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            p = [v.strip() for v in ln.split(",")]
            if len(p) < 8:
                continue
            try:
                sm.append(float(p[0]))
                smax.append(float(p[1]))
            except ValueError:
                continue
            for nm, v in zip(names, p[4:8]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": float(max(smax)) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


# ---- measurement legs --------------------------------------------------------------------------

def timed_steps(sim, steps, warmup):
    import torch

    for _ in range(warmup):
        sim.step(1)
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    from direbm_gb300 import _lib

    l0 = _lib.launch_count()
    ev0.record()
    sim.step(steps)
    ev1.record()
    torch.cuda.synchronize()
    return ev0.elapsed_time(ev1), _lib.launch_count() - l0


def full_run_leg(sim, ib, x, f, steps=100, chunk=10):
    """The configuration's whole run: `steps` steps from the initial state (graphs captured by two
    untimed steps before the reset), timed in chunks of `chunk` steps with CUDA events.  The step
    slows as the run goes on: refine moves leave ~1 % of cells holding two moments by step 100,
    and the window kernels then take the two-item path in almost every tile."""
    import torch

    sim.set_state(ib, x, f)
    sim.step(2)
    sim.set_state(ib, x, f)
    torch.cuda.synchronize()
    chunks = []
    for _ in range(steps // chunk):
        ms, _ = timed_steps(sim, chunk, 0)
        chunks.append(ms / chunk)
    sim.check_status()
    M = len(x)
    mean = float(np.mean(chunks))
    return {"steps": steps, "ms_per_step": mean, "value": M / (mean * 1e-3), "unit": "point-steps/s",
            "ms_per_step_by_chunk": [round(c, 3) for c in chunks], "chunk": chunk}


def roofline_from_profile(sim, M, P, peak):
    prof = {k: [] for k in sim.STAGES}
    for _ in range(3):
        for k, v in sim.profile_step().items():
            prof[k].append(v)
    avg = {k: float(np.mean(v)) for k, v in prof.items()}
    dom = max(avg, key=avg.get)
    unit, per_m, per_c = KERNEL_BYTES[dom]
    nbytes = per_m * M + per_c * (P if unit != "moment+cell" else sim.ncells)
    achieved = nbytes / (avg[dom] * 1e-3) / 1e9
    per_m = KERNEL_TRAFFIC_PER_MOMENT.get(dom)
    traffic = int(per_m * M) if per_m else None
    return dom, avg, {"kernel": dom, "bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                      "frac": achieved / peak, "traffic": traffic, "algorithmic_bytes_per_launch": int(nbytes),
                      "ms_per_launch": avg[dom], "peak_source": "measured (MEASURED_PEAKS.json hbm_gbs)",
                      "traffic_source": "ncu DRAM bytes of a 4.18 M-moment launch, scaled by moments"
                      if per_m else None}


def velocity_l2(f, lat):
    rho = f.sum(1)
    return (f @ lat.C) / rho[:, None]


def fp32_rounded(x, f, lat, rho_rest=1.0):
    """The state as the FP32-deviation store holds it: positions as integer cell + FP32 offset, f as
    the rest equilibrium plus an FP32 deviation.  An FP64 run from this state differs from the FP64
    run from (x, f) only by the input rounding of the FP32 store."""
    c = np.floor(x)
    xr = c + (x - c).astype(np.float32).astype(np.float64)
    rest = rho_rest * lat.W[None, :]
    fr = rest + (f - rest).astype(np.float32).astype(np.float64)
    return xr, fr


def accuracy_leg(steps=10, table=(1, 10, 50, 200)):
    """FP32DEV and FP64 GPU vs the FP64 oracle on one 64x64 instance (the smallest ensemble size)
    after `steps` steps; then, after each step count of `table`, FP32DEV against the FP64 GPU step
    (itself within 1e-12 of the oracle) beside the FP64 step started from the FP32-rounded state
    against the same FP64 step (the method's own response to the FP32 store's input rounding)."""
    from oracle import grid_step
    from oracle.lattices import D2Q9 as OD2Q9

    n = 64
    x = instance_points(n, 100)
    u = fourier_velocity(x, n, 100)
    from direbm_gb300.lattices import D2Q9, equilibrium

    f = equilibrium(np.ones(len(x)), u, D2Q9)
    spec = grid_step.GridSpec(lattice=OD2Q9, dx=DX, r_res=R_RES, cell=CELL, kappa_hard=4,
                              instances=[grid_step.Instance(dims=(n, n), periodic=True, tau=0.8)])
    st = grid_step.run(spec, grid_step.from_world(spec, np.zeros(len(x), int), x, f), steps)
    _, xo, fo = grid_step.to_world(spec, st)
    uo = velocity_l2(fo, OD2Q9)
    out = {"instance": "64x64 periodic D2Q9, tau 0.8, 8 modes RMS 0.02", "steps": steps}
    for prec in ("fp32dev", "fp64"):
        sim = make_sim([n], [0.8], prec, 0)
        sim.set_state(None, x, f)
        sim.step(steps)
        _, xg, fg = sim.state_numpy()
        same = len(xg) == len(xo) and np.abs(xg - xo).max() < 1e-3
        if same:
            ug = velocity_l2(fg, OD2Q9)
            err = float(np.sqrt(((ug - uo) ** 2).sum() / (uo ** 2).sum()))
        else:
            err = None
        out[prec] = {"velocity_l2_rel": err, "points_match": bool(same), "moments": int(len(xg)),
                     "max_pos_err": float(np.abs(xg - xo).max()) if len(xg) == len(xo) else None}
        sim.close()
    # error against step count
    xr, fr = fp32_rounded(x, f, D2Q9)
    starts = {"fp32dev": (x, f), "fp64": (x, f), "fp64_rounded_start": (xr, fr)}
    sims = {k: make_sim([n], [0.8], "fp32dev" if k == "fp32dev" else "fp64", 0) for k in starts}
    for k, sm in sims.items():
        sm.set_state(None, *starts[k])
    rows, done = [], 0
    for t in table:
        for sm in sims.values():
            sm.step(t - done)
        done = t
        st_ = {k: sm.state_numpy() for k, sm in sims.items()}
        row = {"steps": t}
        for k in ("fp32dev", "fp64_rounded_start"):
            row[k + "_vs_fp64"] = compare_states(st_[k], st_["fp64"], [n], D2Q9)
        rows.append(row)
    for sm in sims.values():
        sm.close()
    out["vs_fp64_gpu_by_steps"] = rows
    return out


def _cell_keys(inst, xp, sides):
    """Global cell index of each point (instance-major, row-major inside a square instance)."""
    side = np.asarray(sides, dtype=np.int64)
    offs = np.concatenate([[0], np.cumsum(side * side)])
    c = np.floor(xp).astype(np.int64)
    return offs[inst] + c[:, 0] + side[inst] * c[:, 1]


def _binned_velocity(inst, xp, fp, sides, lat, b):
    """Mass-weighted velocity of each b x b block of cells: sum f c / sum f over its points."""
    side = np.asarray(sides, dtype=np.int64)
    nb = -(-side // b)
    offs = np.concatenate([[0], np.cumsum(nb * nb)])
    c = np.floor(xp).astype(np.int64) // b
    key = offs[inst] + c[:, 0] + nb[inst] * c[:, 1]
    nbin = int(offs[-1])
    mass = np.bincount(key, weights=fp.sum(1), minlength=nbin)
    mom = fp @ lat.C
    u = np.stack([np.bincount(key, weights=mom[:, a], minlength=nbin) for a in range(mom.shape[1])], 1)
    return u / np.maximum(mass, 1e-300)[:, None]


def _powers(z, kmax):
    """Columns z^k for k = -kmax .. kmax (|z| = 1, so z^-k = conj(z^k))."""
    out = np.empty((len(z), 2 * kmax + 1), np.complex128)
    out[:, kmax] = 1.0
    w = np.ones_like(z)
    for k in range(1, kmax + 1):
        w = w * z
        out[:, kmax + k] = w
        out[:, kmax - k] = np.conj(w)
    return out


def _low_modes(inst, xp, fp, sides, lat, kmax=4):
    """Fourier coefficients of the momentum field sum_p j_p exp(-2 pi i k.x_p / n) over the wave
    vectors |k_x|, |k_y| <= kmax of each instance (the band of the initial velocity field)."""
    inst = np.asarray(inst, np.int64)
    order = np.argsort(inst, kind="stable")
    bounds = np.searchsorted(inst[order], np.arange(len(sides) + 1))
    ks = np.arange(-kmax, kmax + 1)
    j = fp @ lat.C
    out = np.zeros((len(sides), 2, len(ks), len(ks)), np.complex128)
    for i, n in enumerate(sides):
        sel = order[bounds[i]:bounds[i + 1]]
        if len(sel) == 0:
            continue
        ex, ey = (_powers(np.exp(-2j * np.pi / float(n) * xp[sel, a]), kmax) for a in range(2))
        for a in range(2):
            out[i, a] = (ex * j[sel, a][:, None]).T @ ey
    return out


def compare_states(a, b, sides, lat, bins=4):
    """State a against state b (each (inst, pos, f) of one ensemble).

    Per point: velocity L2 over the cells where each holds exactly one point (the point sets can
    differ where a near-tie decision went the other way), and over the subset whose points also
    agree in position to 1e-5 cells.  Per field: the L2 of the mass-weighted velocity of each
    bins x bins block of cells, and of the momentum field's Fourier coefficients in the band of the
    initial field (|k_x|, |k_y| <= 4): the macroscopic flow, against which the choice a point made
    at a near tie is a local, small-scale perturbation."""
    (ia_, xa, fa), (ib_, xb, fb) = a, b
    ia_ = np.zeros(len(xa), np.int64) if ia_ is None else np.asarray(ia_, np.int64)
    ib_ = np.zeros(len(xb), np.int64) if ib_ is None else np.asarray(ib_, np.int64)
    ka, kb = _cell_keys(ia_, xa, sides), _cell_keys(ib_, xb, sides)
    ncell = int((np.asarray(sides, dtype=np.int64) ** 2).sum())
    ca, cb = np.bincount(ka, minlength=ncell), np.bincount(kb, minlength=ncell)
    pa, pb = np.zeros(ncell, np.int64), np.zeros(ncell, np.int64)
    pa[ka] = np.arange(len(ka))  # the point of each single-point cell
    pb[kb] = np.arange(len(kb))
    common = np.flatnonzero((ca == 1) & (cb == 1))
    sa, sb = pa[common], pb[common]
    va, vb = velocity_l2(fa[sa], lat), velocity_l2(fb[sb], lat)
    dpos = np.abs(xa[sa] - xb[sb]).max(1)
    agree = dpos < 1e-5

    def l2(m):
        return float(np.sqrt(((va[m] - vb[m]) ** 2).sum() / (vb[m] ** 2).sum())) if m.any() else None

    Ua, Ub = _binned_velocity(ia_, xa, fa, sides, lat, bins), _binned_velocity(ib_, xb, fb, sides, lat, bins)
    La, Lb = _low_modes(ia_, xa, fa, sides, lat), _low_modes(ib_, xb, fb, sides, lat)
    return {"moments": [int(len(xa)), int(len(xb))], "velocity_l2_rel": l2(np.ones(len(common), bool)),
            "matched_cells_frac": float(len(common) / max(len(kb), 1)),
            "positions_differ_gt_1e-5": int((~agree).sum()), "velocity_l2_rel_positions_agree": l2(agree),
            "max_pos_err_positions_agree": float(dpos[agree].max()) if agree.any() else None,
            f"binned{bins}x{bins}_velocity_l2_rel": float(np.sqrt(((Ua - Ub) ** 2).sum() / (Ub ** 2).sum())),
            "low_mode_momentum_l2_rel": float(np.linalg.norm(La - Lb) / np.linalg.norm(Lb))}


def ensemble_accuracy_leg(sides, taus, ib, x, f, steps=10, timed=5):
    """FP32DEV vs FP64 on the full benchmark ensemble (all on the GPU, `steps` steps), beside the
    FP64 step from the FP32-rounded initial state vs FP64, plus the FP64 store's own timing over
    `timed` of those steps (after one warm-up)."""
    from direbm_gb300.lattices import D2Q9

    M = len(x)
    sim = make_sim(sides, taus, "fp32dev", M)
    sim.set_state(ib, x, f)
    sim.step(steps)
    s32 = sim.state_numpy()
    sim.close()
    sim = make_sim(sides, taus, "fp64", M)
    sim.set_state(ib, x, f)
    sim.step(1)
    ms64, _ = timed_steps(sim, timed, 0)
    sim.step(steps - 1 - timed)
    s64 = sim.state_numpy()
    xr, fr = fp32_rounded(x, f, D2Q9)
    sim.set_state(ib, xr, fr)
    sim.step(steps)
    s64r = sim.state_numpy()
    sim.close()
    fp64 = {"value": M * timed / (ms64 * 1e-3), "unit": "point-steps/s", "ms_per_step": ms64 / timed,
            "steps": timed, "warmup": 1}
    out = {"steps": steps,
           "fp32dev_vs_fp64": compare_states(s32, s64, sides, D2Q9),
           "fp64_rounded_start_vs_fp64": compare_states(s64r, s64, sides, D2Q9),
           "note": "all three runs on the GPU; the FP64 step matches the FP64 oracle to 1e-12 at test sizes "
                   "(128x128 over 10 steps). Points whose positions differ by more than 1e-5 took a thinning, "
                   "refine or resampling decision that met a near tie (a distance within ~1e-7 of r, a "
                   "component within ~1e-7 of a cell face, a kappa count or gap-fill threshold at its edge) "
                   "the other way; the FP64 run from the FP32-rounded start shows the same effect from input "
                   "rounding alone"}
    return fp64, out


def lbm_leg(steps=1000, warmup=5):
    import torch

    from direbm_gb300.lattices import D2Q7, equilibrium
    from direbm_gb300.lbm import HexLBM

    ni = nj = 1024
    jrow = np.arange(nj, dtype=np.float64)
    u = np.zeros((nj, ni, 2))
    u[..., 0] = (0.01 * np.sin(2 * np.pi * jrow / nj))[:, None]
    f_shear = equilibrium(np.ones((nj, ni)), u, D2Q7)
    kk = 2 * np.pi / (nj * np.sqrt(3.0) / 2.0)
    taus = np.linspace(0.55, 1.0, 8)
    res = {"config": "hex D2Q7 shear wave 1024x1024, amplitude 0.01, 8 runs tau 0.55..1.0", "steps": steps}
    for prec, s in (("fp32dev", 4), ("fp64", 8)):
        lb = HexLBM(ni, nj, taus, precision=prec)
        lb.set_f(f_shear)
        a0 = lb.shear_amplitude()
        lb.step(warmup)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        lb.step(steps)
        e1.record()
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1)
        a1 = lb.shear_amplitude()
        lam = -np.log(a1 / a0) / (steps + warmup)
        lam_ref = 0.25 * (taus - 0.5) * kk * kk  # nu k^2, nu = cs^2 (tau - 1/2)
        nodes = ni * nj * len(taus)
        gbs = nodes * steps * 2 * 7 * s / (ms * 1e-3) / 1e9
        res[prec] = {"node_steps_per_s": nodes * steps / (ms * 1e-3), "ms_per_step": ms / steps,
                     "achieved_gbs": gbs, "decay_rate_rel_err_max": float(np.abs(lam / lam_ref - 1).max())}
    return res


def in_cell_order(ib, x):
    """Whether the moments are ordered by instance, then cell (row by row), with cells of size CELL:
    the order set_state(presorted=True) takes without sorting.  The ensemble's jittered grids,
    generated row by row one point per cell, are."""
    c = np.floor(np.asarray(x) / CELL).astype(np.int64)
    k = (np.asarray(ib, dtype=np.int64) << 42) + (c[:, 1] << 21) + c[:, 0]
    return bool(len(k) < 2 or (np.diff(k) >= 0).all())


def e2e_leg(sim, ib, x, f, steps=8, warmup=1, io="f32"):
    """Same metric through the public API with host buffers: every step copies the state from pinned
    host memory, loads it, steps once, exports it and copies it back.  One untimed step first, so
    that the output tensors' first allocation is not timed.  io = "f32": positions and f cross the
    host boundary as float32, the element type of the reference's GPU simulator arrays
    (92 -> 48 bytes per moment each way; the device state is the same as from their float64
    widening); io = "f64": as float64.  The host<->device copies move 0.7 / 1.4 GB each way per
    step; their rate depends on the host side (NUMA placement, other jobs), so the line also
    reports the copy bandwidth seen on a separate timed copy."""
    import torch

    M = len(x)
    hdt, tdt = (np.float32, torch.float32) if io == "f32" else (np.float64, torch.float64)
    row = 4 + (2 + 9) * np.dtype(hdt).itemsize  # bytes per moment: instance, position, f
    presorted = in_cell_order(ib, x)  # the load then skips its sort (the device checks the order)
    h_inst = torch.from_numpy(ib.astype(np.int32)).pin_memory()
    h_pos = torch.from_numpy(np.ascontiguousarray(x, dtype=hdt)).pin_memory()
    h_f = torch.from_numpy(np.ascontiguousarray(f, dtype=hdt)).pin_memory()
    d_inst = torch.empty(M, dtype=torch.int32, device="cuda")
    d_pos = torch.empty((M, 2), dtype=tdt, device="cuda")
    d_f = torch.empty((M, 9), dtype=tdt, device="cuda")
    o_inst = torch.empty(M, dtype=torch.int32).pin_memory()
    o_pos = torch.empty((M, 2), dtype=tdt).pin_memory()
    o_f = torch.empty((M, 9), dtype=tdt).pin_memory()
    def one_step():
        d_inst.copy_(h_inst, non_blocking=True)
        d_pos.copy_(h_pos, non_blocking=True)
        d_f.copy_(h_f, non_blocking=True)
        sim.set_state(d_inst, d_pos, d_f, presorted=presorted)
        sim.step(1)
        gi, gp, gf = sim.state(dtype=tdt)
        m2 = gi.shape[0]
        o_inst[:m2].copy_(gi, non_blocking=True)
        o_pos[:m2].copy_(gp, non_blocking=True)
        o_f[:m2].copy_(gf, non_blocking=True)

    for _ in range(warmup):
        one_step()
    torch.cuda.synchronize()
    # copy bandwidth alone (the largest array, each way)
    c0, c1, c2 = (torch.cuda.Event(enable_timing=True) for _ in range(3))
    c0.record()
    d_f.copy_(h_f, non_blocking=True)
    c1.record()
    o_f.copy_(d_f, non_blocking=True)
    c2.record()
    torch.cuda.synchronize()
    h2d_gbs = h_f.numel() * h_f.element_size() / (c0.elapsed_time(c1) * 1e-3) / 1e9
    d2h_gbs = h_f.numel() * h_f.element_size() / (c1.elapsed_time(c2) * 1e-3) / 1e9
    t0 = time.perf_counter()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    points = 0
    h2d = d2h = 0
    for _ in range(steps):
        d_inst.copy_(h_inst, non_blocking=True)
        d_pos.copy_(h_pos, non_blocking=True)
        d_f.copy_(h_f, non_blocking=True)
        sim.set_state(d_inst, d_pos, d_f, presorted=presorted)
        points += M
        sim.step(1)
        gi, gp, gf = sim.state(dtype=tdt)
        m2 = gi.shape[0]
        o_inst[:m2].copy_(gi, non_blocking=True)
        o_pos[:m2].copy_(gp, non_blocking=True)
        o_f[:m2].copy_(gf, non_blocking=True)
        h2d += M * row
        d2h += m2 * row
    e1.record()
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    ms = e0.elapsed_time(e1)
    serial = {"value": points / (ms * 1e-3), "ms_per_step": ms / steps, "wall_s": wall}
    piped = _e2e_pipelined(sim, M, h_inst, h_pos, h_f, steps, warmup, (o_inst, o_pos, o_f, m2), presorted, tdt, row)
    serial["h2d_bytes_per_step"], serial["d2h_bytes_per_step"] = int(h2d // steps), int(d2h // steps)
    # the device-side parts of a step alone (CUDA events, median of 5): the load of resident inputs,
    # the step from the loaded state, and the export into capacity-sized buffers
    out = tuple(torch.empty((sim.capacity,) + tuple(t.shape[1:]), dtype=t.dtype, device="cuda")
                for t in (d_inst, d_pos, d_f))

    def med_ms(fn, before=None):
        r = []
        for _ in range(5):
            if before:
                before()
            torch.cuda.synchronize()
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record()
            fn()
            b.record()
            torch.cuda.synchronize()
            r.append(a.elapsed_time(b))
        return float(np.median(r))

    load = lambda: sim.set_state(d_inst, d_pos, d_f, check=False, presorted=presorted)
    parts = {"load_ms": med_ms(load), "step_after_load_ms": med_ms(lambda: sim.step(1), before=load),
             "export_ms": med_ms(lambda: sim.state_into(out))}
    sim.check_status()
    del out
    return {"value": piped["value"], "unit": "point-steps/s", "h2d_bytes_per_step": int(piped["h2d_bytes_per_step"]),
            "d2h_bytes_per_step": int(piped["d2h_bytes_per_step"]), "ms_per_step": piped["ms_per_step"],
            "wall_s": piped["wall_s"],
            "steps": steps, "warmup": warmup, "copy_gbs": {"h2d": h2d_gbs, "d2h": d2h_gbs}, "serial": serial,
            "result_equals_serial": piped["result_equals_serial"],
            "repetitions_ms_per_step": piped["repetitions_ms_per_step"], "statistic": "median of 5 repetitions",
            "presorted": presorted, "io": io, "device_parts": parts,
            "path": "Simulation.set_state(check=False, presorted=<input in cell order>)/step/state_into (C ABI "
                    "dbm_sim_*) with pinned host buffers and "
                    "no host wait inside a step; each step's host-to-device copy on its own stream overlaps the "
                    "previous step, each step's device-to-host copy of the whole output buffers (capacity rows) on a "
                    "third stream overlaps the next (two buffer slots each way); status and count read after the run"}


def e2e_both(sim, ib, x, f):
    """The e2e leg through float32 host buffers (the reported figure) with the float64 one beside it."""
    e2e = e2e_leg(sim, ib, x, f, io="f32")
    e64 = e2e_leg(sim, ib, x, f, io="f64")
    e2e["f64_io"] = {k: e64[k] for k in ("value", "ms_per_step", "h2d_bytes_per_step", "d2h_bytes_per_step",
                                         "copy_gbs", "repetitions_ms_per_step", "result_equals_serial",
                                         "device_parts")}
    return e2e


def _e2e_pipelined(sim, M, h_inst, h_pos, h_f, steps, warmup, serial_out, presorted, tdt, row):
    """The e2e steps with the copies overlapped: inputs of step i+1 go up while step i computes, and
    results of step i come down while step i+1 computes.  Every step still copies its whole input
    from pinned host memory and its whole result back, inside the timed region."""
    import torch

    dev = "cuda"
    main = torch.cuda.current_stream()
    s_up, s_down = torch.cuda.Stream(), torch.cuda.Stream()
    cap = max(M, sim.ncells)
    din = [(torch.empty(M, dtype=torch.int32, device=dev), torch.empty((M, 2), dtype=tdt, device=dev),
            torch.empty((M, 9), dtype=tdt, device=dev)) for _ in range(2)]
    dout = [(torch.empty(cap, dtype=torch.int32, device=dev), torch.empty((cap, 2), dtype=tdt, device=dev),
             torch.empty((cap, 9), dtype=tdt, device=dev)) for _ in range(2)]
    hout = [(torch.empty(cap, dtype=torch.int32).pin_memory(), torch.empty((cap, 2), dtype=tdt).pin_memory(),
             torch.empty((cap, 9), dtype=tdt).pin_memory()) for _ in range(2)]
    ev = {n: [torch.cuda.Event() for _ in range(2)] for n in ("in", "used", "out", "down")}

    def upload(slot):
        with torch.cuda.stream(s_up):
            s_up.wait_event(ev["used"][slot])  # the step that read this slot has loaded it
            for d, h in zip(din[slot], (h_inst, h_pos, h_f)):
                d.copy_(h, non_blocking=True)
            ev["in"][slot].record(s_up)

    last = {}

    def run(n):
        for sl in (0, 1):
            ev["used"][sl].record(main)
            ev["down"][sl].record(main)
        upload(0)
        for i in range(n):
            sl = i % 2
            if i + 1 < n:
                upload(1 - sl)
            main.wait_event(ev["in"][sl])
            sim.set_state(*din[sl], check=False, presorted=presorted)  # status checked after the run
            ev["used"][sl].record(main)
            sim.step(1)
            main.wait_event(ev["down"][sl])  # this slot's previous result has left the device
            sim.state_into(dout[sl])  # no host wait: the whole buffers go down, count() read after
            ev["out"][sl].record(main)
            with torch.cuda.stream(s_down):
                s_down.wait_event(ev["out"][sl])
                for h, d in zip(hout[sl], dout[sl]):
                    h.copy_(d, non_blocking=True)
                ev["down"][sl].record(s_down)
            last.update(slot=sl)
        main.wait_stream(s_down)
        main.wait_stream(s_up)

    run(max(warmup, 1))
    torch.cuda.synchronize()
    # five repetitions of `steps` steps: the host side of this box is shared, so a repetition can be
    # slowed by other jobs' copies; the median is reported and every repetition listed
    reps = []
    for _ in range(5):
        t0 = time.perf_counter()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        run(steps)
        e1.record()
        torch.cuda.synchronize()
        reps.append((e0.elapsed_time(e1), time.perf_counter() - t0))
    ms, wall = sorted(reps)[len(reps) // 2]
    sim.check_status()  # set_state's deferred bad-input check, and every step's status bits
    # same input every step and deterministic kernels: the last result equals the serial path's
    oi, op, of, m_serial = serial_out
    hi, hp, hf = hout[last["slot"]]
    m2 = sim.count()
    n = min(m_serial, 1 << 20)
    same = (m2 == m_serial and torch.equal(hi[:n], oi[:n]) and torch.equal(hp[:n], op[:n])
            and torch.equal(hf[:n], of[:n]))
    return {"value": M * steps / (ms * 1e-3), "ms_per_step": ms / steps, "wall_s": wall,
            "result_equals_serial": bool(same), "repetitions_ms_per_step": [r[0] / steps for r in reps],
            "h2d_bytes_per_step": M * row, "d2h_bytes_per_step": cap * row}


def adjoint_leg(n=256, steps=100, every=10, tau=0.6, precisions=("fp32dev", "fp64")):
    """Inverse problem: one periodic D2Q9 run of n x n = 64k jittered points, unit density, initial
    velocity from 8 Fourier modes (16 coefficients, seed 21, RMS 0.02); loss = mean |u(f_T) - u*(x_T)|^2
    against a target 8-mode field (seed 1000); gradient w.r.t. the 16 coefficients and tau through
    the checkpointed adjoint (checkpoint every `every` steps).  Times the plain forward (graphs),
    the forward with checkpoints and the backward (recomputation + tape + VJP) with CUDA events,
    in FP32DEV and FP64, and compares the two gradients."""
    import torch

    from direbm_gb300.adjoint import ModeField, Tape, inverse_problem_loss
    from direbm_gb300.lattices import D2Q9, equilibrium as eq_np

    x = instance_points(n, 5)
    field = ModeField(n, seed=21, points=x)
    target = ModeField(n, seed=1000, points=x)
    x_d = torch.as_tensor(x, device="cuda")
    out = {"config": f"{n}x{n} jittered points, periodic D2Q9, tau {tau}, r 1.5h, cell h, {steps} steps, "
                     f"checkpoint every {every}; 16 mode coefficients + tau", "steps": steps, "checkpoint_every": every}
    grads = {}
    for prec in precisions:
        sim = make_sim([n], [tau], prec, 4 * len(x))
        # plain forward step (captured graphs), the reference cost of one step
        f0 = eq_np(np.ones(len(x)), field(torch.as_tensor(x), torch.as_tensor(field.coeffs)).numpy(), D2Q9)
        sim.set_state(None, x, f0)
        ms_plain, _ = timed_steps(sim, steps, 3)
        tape = Tape(sim)
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
        res = None
        for rep in range(2):  # the first repetition warms up allocations
            coeffs = torch.tensor(field.coeffs, dtype=torch.float64, device="cuda", requires_grad=True)
            tt = torch.tensor([tau], dtype=torch.float64, device="cuda", requires_grad=True)
            torch.cuda.synchronize()
            ev[0].record()
            loss = inverse_problem_loss(sim, x_d, field, coeffs, tt, target, steps, every, tape)
            ev[1].record()
            loss.backward()
            ev[2].record()
            torch.cuda.synchronize()
            res = (float(loss.item()), torch.cat([coeffs.grad, tt.grad]).cpu().numpy(), ev[0].elapsed_time(ev[1]),
                   ev[1].elapsed_time(ev[2]))
        loss_v, g, ms_f, ms_b = res
        grads[prec] = g
        step_ms = ms_plain / steps
        out[prec] = {
            "loss": loss_v, "forward_ms_per_step": step_ms, "forward_ckpt_ms_per_step": ms_f / steps,
            "backward_ms_per_step": ms_b / steps, "adjoint_steps_per_s": steps / (ms_b * 1e-3),
            "gradient_steps_per_s": steps / ((ms_f + ms_b) * 1e-3),
            "backward_over_forward": (ms_b / steps) / step_ms, "gradient_over_forward": ((ms_f + ms_b) / steps) / step_ms,
            "grad_norm": float(np.linalg.norm(g)), "dL_dtau": float(g[-1]),
        }
        tape.close()
        sim.close()
    if "fp32dev" in grads and "fp64" in grads:
        out["fp32dev_grad_rel_err_vs_fp64"] = float(np.linalg.norm(grads["fp32dev"] - grads["fp64"]) /
                                                     np.linalg.norm(grads["fp64"]))
        out["fp32dev_loss_rel_err_vs_fp64"] = abs(out["fp32dev"]["loss"] / out["fp64"]["loss"] - 1.0)
    return out


def sphere_leg(steps=20, steps64=10):
    """Flow past a sphere (the 3D obstacle configuration): D3Q19, periodic box of 160 x 112 x 112
    cells (h = dx = 1) with one jittered point per cell outside a bounce-back sphere of radius 16h
    at (40, 56, 56) (~2.0 M points), uniform initial and inflow velocity 0.04 along x (inflow layer
    of 2 cell columns), tau 0.56, r 1.5h.  Uniform point density: cell thinning at cell h keeps at
    most one point per cell, so a 4x denser seeding near the sphere would be thinned back to this
    density in the first step.  FP32DEV and FP64 point-steps/s and their velocity difference."""
    import torch

    from direbm_gb300.lattices import D3Q19, equilibrium
    from direbm_gb300.sim import Instance, Simulation

    dims = (160, 112, 112)
    center, radius, u0 = (40.0, 56.0, 56.0), 16.0, 0.04
    rng = np.random.default_rng(3)
    x = (np.indices(dims).reshape(3, -1).T + 0.5).astype(np.float64)
    x += rng.uniform(-0.25, 0.25, size=x.shape)
    x = np.mod(x, np.asarray(dims, dtype=np.float64))
    x = x[((x - np.asarray(center)) ** 2).sum(1) >= (radius + 0.5) ** 2]
    u = np.zeros_like(x)
    u[:, 0] = u0
    f = equilibrium(np.ones(len(x)), u, D3Q19)
    out = {"config": "D3Q19 sphere r=16h in 160x112x112 periodic box, inflow 0.04 (2 columns), tau 0.56, "
                     "uniform 1 point/cell outside the sphere", "points": int(len(x))}
    states = {}
    for prec, n in (("fp32dev", steps), ("fp64", steps64)):
        inst = Instance(dims=dims, periodic=True, tau=0.56, obstacle=(center, radius), inflow=((u0, 0.0, 0.0), 2))
        sim = Simulation([inst], lattice="D3Q19", precision=prec, dx=DX, r_res=R_RES, cell=CELL,
                         moment_capacity=int(1.2 * len(x)))
        sim.set_state(None, x, f)
        m0 = float(sim.conservation()[0, 0])
        if prec == "fp32dev":  # brick width of the untiled 3D kernels, by timing (results do not depend on it)
            from direbm_gb300.autotune import autotune

            out["brick_width"] = autotune(sim, steps=1, use_cache=False)["brick_width"]
        else:
            sim.set_brick_width(out["brick_width"])
        sim.step(1)  # warm-up (graph capture)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        sim.step(n)
        e1.record()
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1)
        sim.check_status()
        pts = sim.count()
        out[prec] = {"point_steps_per_s": pts * n / (ms * 1e-3), "ms_per_step": ms / n, "steps": n,
                     "mass_drift": float(sim.conservation()[0, 0]) / m0 - 1.0}
        sim.close()
        # the same 1 + steps64 steps again for the FP32DEV vs FP64 comparison
        sim = Simulation([inst], lattice="D3Q19", precision=prec, dx=DX, r_res=R_RES, cell=CELL,
                         moment_capacity=int(1.2 * len(x)))
        sim.set_state(None, x, f)
        sim.step(1 + steps64)
        states[prec] = sim.state_numpy()
        sim.close()
    # the FP64 run again from the FP32-rounded start: the method's own response to input rounding
    sim = Simulation([inst], lattice="D3Q19", precision="fp64", dx=DX, r_res=R_RES, cell=CELL,
                     moment_capacity=int(1.2 * len(x)))
    sim.set_state(None, *fp32_rounded(x, f, D3Q19))
    sim.step(1 + steps64)
    states["fp64_rounded_start"] = sim.state_numpy()
    sim.close()

    def cmp3(a, b, bins=4):
        """Velocity L2 over the cells where each run holds exactly one point, over the subset whose
        positions also agree to 1e-5, and of the mass-weighted velocity of bins^3 blocks of cells."""
        (_, xa, fa), (_, xb, fb) = a, b

        def key(xp, div=1):
            c = np.floor(xp).astype(np.int64) // div
            nd = [-(-d // div) for d in dims]
            return (c[:, 2] * nd[1] + c[:, 1]) * nd[0] + c[:, 0]

        ka, kb = key(xa), key(xb)
        ua, ia0, ca = np.unique(ka, return_index=True, return_counts=True)
        ub, ib0, cb = np.unique(kb, return_index=True, return_counts=True)
        common, pa, pb = np.intersect1d(ua[ca == 1], ub[cb == 1], return_indices=True)
        sa, sb = ia0[ca == 1][pa], ib0[cb == 1][pb]
        va, vb = velocity_l2(fa[sa], D3Q19), velocity_l2(fb[sb], D3Q19)
        agree = np.abs(xa[sa] - xb[sb]).max(1) < 1e-5

        def l2(m):
            return float(np.sqrt(((va[m] - vb[m]) ** 2).sum() / (vb[m] ** 2).sum())) if m.any() else None

        def binned(xp, fp):
            k = key(xp, bins)
            nbin = int(np.prod([-(-d // bins) for d in dims]))
            mass = np.bincount(k, weights=fp.sum(1), minlength=nbin)
            mom = fp @ D3Q19.C
            u = np.stack([np.bincount(k, weights=mom[:, a], minlength=nbin) for a in range(3)], 1)
            return u / np.maximum(mass, 1e-300)[:, None]

        Ua, Ub = binned(xa, fa), binned(xb, fb)
        return {"points": [int(len(xa)), int(len(xb))], "velocity_l2_rel": l2(np.ones(len(common), bool)),
                "matched_cells_frac": len(common) / max(len(xb), 1),
                "positions_differ_gt_1e-5": int((~agree).sum()), "velocity_l2_rel_positions_agree": l2(agree),
                f"binned{bins}x{bins}x{bins}_velocity_l2_rel": float(np.sqrt(((Ua - Ub) ** 2).sum() / (Ub ** 2).sum()))}

    out["compared_after_steps"] = 1 + steps64
    out["fp32dev_vs_fp64"] = cmp3(states["fp32dev"], states["fp64"])
    out["fp64_rounded_start_vs_fp64"] = cmp3(states["fp64_rounded_start"], states["fp64"])
    out["speedup_fp32dev_vs_fp64"] = out["fp32dev"]["point_steps_per_s"] / out["fp64"]["point_steps_per_s"]
    return out


# ---- CPU oracle legs -----------------------------------------------------------------------------

def _oracle_instance_steps(args):
    n, tau, seed, steps = args
    from direbm_gb300.lattices import D2Q9, equilibrium
    from oracle import grid_step
    from oracle.lattices import D2Q9 as OD2Q9

    x = instance_points(n, seed)
    u = fourier_velocity(x, n, seed)
    f = equilibrium(np.ones(len(x)), u, D2Q9)
    spec = grid_step.GridSpec(lattice=OD2Q9, dx=DX, r_res=R_RES, cell=CELL, kappa_hard=4,
                              instances=[grid_step.Instance(dims=(n, n), periodic=True, tau=tau)])
    st = grid_step.from_world(spec, np.zeros(len(x), int), x, f)
    t0 = time.perf_counter()
    pts = 0
    for _ in range(steps):
        pts += len(st.cell)
        st = grid_step.step(spec, st)
    return pts, time.perf_counter() - t0


REF_SIM_DIR = ROOT / "baseline" / "_ref"  # the reference's CPU package (oracle/install_reference.py)


def _reference_simulator_job(args):
    """The reference's own CPU simulator (direbm.reference.Simulator, unoptimised pure Python) on an
    n x n block of config-1 density (spacing h = dx = 1, jitter U(+-0.25)) with the Taylor-Green
    velocity u0 = 0.05, D2Q9 built from the reference's generic Lattice, tau 0.6, in the reference's
    own unbounded form (r = dx, thinning radius dx/4).  Returns (input point-steps, seconds)."""
    n, steps, seed = args
    sys.path.insert(0, str(REF_SIM_DIR))
    from direbm.lattices import Lattice
    from direbm.physics import equilibrium
    from direbm.reference import Moment, Simulator

    d2q9 = Lattice(C=np.array([[0, 0], [1, 0], [0, 1], [-1, 0], [0, -1], [1, 1], [-1, 1], [-1, -1], [1, -1]], float),
                   W=np.array([4 / 9] + [1 / 9] * 4 + [1 / 36] * 4), cs2=1.0 / 3.0, name="D2Q9")
    rng = np.random.default_rng(seed)
    x = (np.indices((n, n)).reshape(2, -1).T[:, ::-1] + 0.5).astype(np.float64)
    x += rng.uniform(-0.25, 0.25, size=x.shape)
    k = 2 * np.pi / n
    u = 0.05 * np.stack([-np.cos(k * x[:, 0]) * np.sin(k * x[:, 1]), np.sin(k * x[:, 0]) * np.cos(k * x[:, 1])], 1)
    f = equilibrium(np.ones(len(x)), u, d2q9)
    sim = Simulator([Moment(f=f[i].copy(), x=x[i].copy()) for i in range(len(x))], tau=0.6, lattice=d2q9)
    t0 = time.perf_counter()
    pts = 0
    for _ in range(steps):
        pts += len(sim.moments)
        sim.step()
    return pts, time.perf_counter() - t0


def reference_simulator_leg(n=12, steps=2):
    """The reference's own CPU step timed on this host: one process, then one process per core on
    independent seeds (aggregate point-steps/s).  None when the reference is not installed."""
    import multiprocessing as mp

    if not (REF_SIM_DIR / "direbm" / "__init__.py").exists():
        return None
    cores = os.cpu_count() or 1
    ctx = mp.get_context("spawn")  # this process already holds a CUDA context
    with ctx.Pool(cores) as pool:
        pts1, sec1 = pool.apply(_reference_simulator_job, ((n, steps, 0),))
        t0 = time.perf_counter()
        res = pool.map(_reference_simulator_job, [(n, steps, s) for s in range(cores)])
        wall = time.perf_counter() - t0
    ptsn = sum(p for p, _ in res)
    sample = (f"{n}x{n} block of config-1 density, TG u0 0.05, D2Q9, tau 0.6, first {steps} steps (the moment "
              f"count grows from {n * n} as the unbounded block spreads), reference form r = dx, cell dx/4")
    return {"kind": "reference", "what": "direbm.reference.Simulator (the reference's CPU path, pure Python)",
            "one_process": {"value": pts1 / sec1, "unit": "point-steps/s", "cores": 1, "seconds": sec1},
            "all_cores": {"value": ptsn / wall, "unit": "point-steps/s", "cores": cores, "seconds": wall},
            "sample": sample}


def cpu_baseline_leg(n=128, steps=2, lbm_steps=3):
    pts, sec = _oracle_instance_steps((n, 0.8, 100, steps))
    out = {"value": pts / sec, "unit": "point-steps/s", "cores": 1, "kind": "port",
           "sample": f"numpy oracle of the step, one {n}x{n} periodic D2Q9 instance, {steps} steps, {sec:.1f} s"}
    # the hex LBM on one host thread: the numpy oracle (the reference's HexLBM restated), one
    # 1024 x 1024 run of the shear wave, FP64
    from oracle import lbm as olbm

    f0 = olbm.shear_wave(1024, 1024, 0.01)
    olbm.run(f0, 0.7, 1)
    t0 = time.perf_counter()
    olbm.run(f0, 0.7, lbm_steps)
    sec = time.perf_counter() - t0
    out["lbm"] = {"value": 1024 * 1024 * lbm_steps / sec, "unit": "node-steps/s", "cores": 1, "kind": "port",
                  "sample": f"numpy oracle HexLBM, one 1024x1024 run, {lbm_steps} steps, {sec:.1f} s"}
    ref = reference_simulator_leg()
    out["reference_simulator"] = ref if ref is not None else {
        "unavailable": "the reference package is not installed under baseline/_ref (oracle/install_reference.py)"}
    return out


# The reference arm steps real ensemble members no larger than this (a third of the ensemble), so
# that one timed step of all host cores stays within a few seconds.
REF_ARM_MAX_POINTS = 16384


def ensemble_config(n_inst=N_INST):
    """The benchmark workload's description, shared by both arms."""
    sides, _ = ensemble_spec(n_inst)
    return {"workload": f"batched ensemble: {n_inst} periodic 2D D2Q9 runs, M log-uniform 4k-256k (seed 1), "
                        "tau U(0.55,1), 8 Fourier modes RMS 0.02, r 1.5h, cell h, FP32-deviation store",
            "moments": int((np.asarray(sides, dtype=np.int64) ** 2).sum()), "instances": int(n_inst),
            "store": "fp32dev", "graphs": True, "l2": "state (~0.8 GB) larger than L2, no flush"}


def run_reference(args):
    """The reference arm: the CPU oracle (numpy restatement of the reference GPU step) on all host
    cores.  Each timed step, every core steps one member of the benchmark ensemble itself (its own
    size, seed, tau and velocity field), cycling through the members of at most REF_ARM_MAX_POINTS
    points."""
    import multiprocessing as mp

    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    cores = os.cpu_count() or 1
    sides, taus = ensemble_spec(args.instances)
    members = [i for i in range(len(sides)) if int(sides[i]) ** 2 <= REF_ARM_MAX_POINTS]

    def jobs(r):
        return [(int(sides[i]), float(taus[i]), 100 + i, 1)
                for i in (members[(r * cores + w) % len(members)] for w in range(cores))]

    ctx = mp.get_context("spawn")
    with ctx.Pool(cores) as pool:
        for r in range(args.warmup):
            pool.map(_oracle_instance_steps, jobs(r))
        t0 = time.perf_counter()
        pts = 0
        for r in range(args.steps):
            pts += sum(p for p, _ in pool.map(_oracle_instance_steps, jobs(args.warmup + r)))
        sec = time.perf_counter() - t0
    value = pts / sec
    sample = (f"{cores} worker processes, each stepping one ensemble member per timed step (members with at most "
              f"{REF_ARM_MAX_POINTS} points: {len(members)} of {len(sides)}, sizes "
              f"{int(min(sides[members]) ** 2)}-{int(max(sides[members]) ** 2)}), FP64 numpy")
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "point-steps/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": sec / args.steps * 1e3,
        "higher_is_better": True, "scaling": "strong", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": ensemble_config(args.instances),
        "cpu_baseline": {"value": value, "unit": "point-steps/s", "cores": cores, "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": "point-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# ---- main ----------------------------------------------------------------------------------------

def max_over_ranks(ms: float, dist=None) -> float:
    """The slowest rank's time (every rank gets it); a plain float without a process group."""
    if dist is None or not dist.is_initialized():
        return float(ms)
    from direbm_gb300.shard import max_over_ranks as mor

    return mor(ms)


def sum_over_ranks(v: float, dist=None) -> float:
    if dist is None or not dist.is_initialized():
        return float(v)
    import torch

    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(v)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


def whole_job_rate(moments_total: int, steps: int, ms: float) -> float:
    """Point-steps/s of the whole job: the ranks share one ensemble (each steps its shard of the
    instances, strong scaling), so the work is all moments x steps over the slowest rank's time."""
    return moments_total * steps / (ms * 1e-3)


def run_ours(args):
    import torch

    from direbm_gb300 import _lib

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    peaks = json.loads((ROOT / "MEASURED_PEAKS.json").read_text()) if (ROOT / "MEASURED_PEAKS.json").exists() else {}
    peak = float(peaks.get("hbm_gbs", 6800.0))

    sides, taus = ensemble_spec(args.instances)
    # one ensemble, its instances partitioned over the ranks by point count (no exchange while
    # stepping); at N = 1 the one shard is the whole ensemble
    from direbm_gb300.shard import partition

    members = partition(np.asarray(sides, dtype=np.int64) ** 2, world)[rank]
    ib, x, f = build_ensemble(sides, taus, members)
    M = len(x)
    M_total = int((np.asarray(sides, dtype=np.int64) ** 2).sum())
    sim = make_sim(sides[members], taus[members], "fp32dev", M)
    sim.set_state(ib, x, f)
    from direbm_gb300.autotune import autotune

    tuning = autotune(sim, steps=2, use_cache=False)  # tile shape / persistent launches, by timing

    clk = ClockSampler(local)
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    clk.start()
    ms, launches = timed_steps(sim, args.steps, args.warmup)
    clocks = clk.stop()
    ms = max_over_ranks(ms, dist)
    P = sim.count()
    sim.check_status()
    value = whole_job_rate(M_total, args.steps, ms)
    moments_after = int(sum_over_ranks(P, dist))

    if world > 1:  # the whole ensemble's result: every shard's state gathered on rank 0
        from direbm_gb300.shard import gather_state

        gi, gp, gf = sim.state()
        got = gather_state(gi, gp, gf, members)
        e2e = e2e_leg(sim, ib, x, f)
        e2e_ms = max_over_ranks(e2e["ms_per_step"], dist)
        h2d = sum_over_ranks(e2e["h2d_bytes_per_step"], dist)
        d2h = sum_over_ranks(e2e["d2h_bytes_per_step"], dist)
        sim.close()
        if rank == 0:
            print(json.dumps({
                "metric": METRIC, "value": value, "unit": "point-steps/s", "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
                "scaling": "strong", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
                "config": {**ensemble_config(args.instances), "parallelism": f"instance shards x{world}"},
                "shards": {"moments_max_rank": int(max_over_ranks(M, dist)), "moments_total": M_total,
                           "gathered_moments": int(got[0].shape[0]), "moments_after_steps": moments_after},
                "e2e": {"value": M_total / (e2e_ms * 1e-3), "unit": "point-steps/s",
                        "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h), "ms_per_step": e2e_ms},
                "gpu_launches": int(launches), "clocks": clocks}), flush=True)
        else:
            max_over_ranks(M, dist)
        dist.barrier()
        dist.destroy_process_group()
        return

    dom, stage_ms, roof = roofline_from_profile(sim, sim.count(), P, peak)
    step_ms = ms / args.steps
    bpp = step_bytes_per_point()
    step_roof = {"bytes_per_point_step": bpp, "achieved": bpp * M / (step_ms * 1e-3) / 1e9, "peak": peak,
                 "unit": "GB/s"}
    step_roof["frac"] = step_roof["achieved"] / peak

    if args.legs == "main":  # kernel-only run (profiling): no side legs
        print(json.dumps({"metric": METRIC, "value": value, "unit": "point-steps/s", "ms_per_step": step_ms,
                          "moments": int(M), "stage_ms": stage_ms, "roofline": roof, "gpu_launches": int(launches),
                          "tiling": tuning}),
              flush=True)
        sim.close()
        return
    run100 = full_run_leg(sim, ib, x, f)
    e2e = e2e_both(sim, ib, x, f)
    sim.close()

    # FP64 store on the same workload, and FP32DEV vs FP64 after the same steps on the whole ensemble
    fp64, acc_ens = ensemble_accuracy_leg(sides, taus, ib, x, f)

    acc = accuracy_leg()
    lbm = lbm_leg()
    adj = adjoint_leg()
    sph = sphere_leg()
    cpu = cpu_baseline_leg()
    line = {
        "metric": METRIC, "value": value, "unit": "point-steps/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": step_ms, "higher_is_better": True, "scaling": "strong",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": ensemble_config(args.instances),
        "tiling": {"tile_width": tuning["tile_width"], "persistent": tuning["persistent"],
                   "timings_ms": tuning["timings"]},
        "roofline": roof, "stage_ms": stage_ms, "step_roofline": step_roof, "full_run": run100,
        "cpu_baseline": cpu, "e2e": e2e, "gpu_launches": int(launches), "clocks": clocks,
        "fp64": fp64, "speedup_fp32dev_vs_fp64": value / world / fp64["value"], "accuracy": acc,
        "accuracy_ensemble": acc_ens, "lbm": lbm,
        "adjoint": adj, "sphere": sph,
    }
    print(json.dumps(line), flush=True)
    if dist:
        dist.barrier()
        dist.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--instances", type=int, default=N_INST, help="first N ensemble members (profiling runs)")
    ap.add_argument("--legs", default="all",
                    choices=["all", "main", "adjoint", "sphere", "lbm", "e2e", "accuracy", "cpu", "profile"],
                    help="main = timed step only; adjoint / sphere / lbm / e2e / accuracy / cpu = that leg only; "
                         "profile = --profile-steps graph steps, then one eager step stage by stage (for ncu)")
    ap.add_argument("--profile-steps", type=int, default=0, help="profile leg: steps before the eager one")
    ap.add_argument("--adjoint-n", type=int, default=256, help="adjoint leg: points per side")
    ap.add_argument("--adjoint-steps", type=int, default=100, help="adjoint leg: rollout steps")
    ap.add_argument("--adjoint-every", type=int, default=10, help="adjoint leg: checkpoint interval")
    ap.add_argument("--adjoint-precisions", default="fp32dev,fp64", help="adjoint leg: stores to run")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.legs == "lbm" and args.impl == "ours":
        import torch

        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        print(json.dumps({"lbm": lbm_leg()}), flush=True)
        return
    if args.legs == "sphere" and args.impl == "ours":
        import torch

        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        print(json.dumps({"sphere": sphere_leg()}), flush=True)
        return
    if args.legs == "e2e" and args.impl == "ours":
        import torch

        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        sides, taus = ensemble_spec(args.instances)
        ib, x, f = build_ensemble(sides, taus)
        sim = make_sim(sides, taus, "fp32dev", len(x))
        sim.set_state(ib, x, f)
        print(json.dumps({"e2e": e2e_both(sim, ib, x, f)}), flush=True)
        sim.close()
        return
    if args.legs == "accuracy" and args.impl == "ours":
        import torch

        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        sides, taus = ensemble_spec(args.instances)
        ib, x, f = build_ensemble(sides, taus)
        fp64, acc_ens = ensemble_accuracy_leg(sides, taus, ib, x, f)
        print(json.dumps({"fp64": fp64, "accuracy_ensemble": acc_ens, "accuracy": accuracy_leg()}), flush=True)
        return
    if args.legs == "profile" and args.impl == "ours":
        # the first --instances members, 16x16 tiles without persistence (the autotuner's choice on
        # the full ensemble), --profile-steps steps, then one step launched stage by stage
        import torch

        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        sides, taus = ensemble_spec(args.instances)
        ib, x, f = build_ensemble(sides, taus)
        sim = make_sim(sides, taus, "fp32dev", len(x))
        sim.set_tiling(16, False)
        sim.set_state(ib, x, f)
        sim.step(args.profile_steps)
        print(json.dumps({"moments": len(x), "steps_before": args.profile_steps, "stage_ms": sim.profile_step()}),
              flush=True)
        sim.check_status()
        sim.close()
        return
    if args.legs == "cpu" and args.impl == "ours":
        print(json.dumps({"cpu_baseline": cpu_baseline_leg()}), flush=True)
        return
    if args.legs == "adjoint" and args.impl == "ours":
        import torch

        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        print(json.dumps({"adjoint": adjoint_leg(args.adjoint_n, args.adjoint_steps, args.adjoint_every,
                                                 precisions=tuple(args.adjoint_precisions.split(",")))}), flush=True)
        return
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
