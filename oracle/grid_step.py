"""The DiReBM step on a dense cell grid (test oracle for the fused CUDA pipeline).

This restates the reference GPU step (direbm/warp/simulator.py:50-73 -> collide, disperse,
create_control_points, refine_control_points, resample in direbm/warp/propagation.py) in the data
layout the CUDA pipeline uses, with the generalisations the benchmark configurations need:
any velocity set, a resampling radius ``r_res`` separate from ``dx``, a thinning cell ``cell``
separate from dx/alpha, periodic boxes, and a batch of independent instances.

Representation (shared with the CUDA pipeline; everything in units of the thinning cell):
  * a moment sits at integer cell coordinates S (inside its instance's box) plus an offset
    ``off`` in [0, 1) per axis; world position = (origin + S + off) * cell;
  * moments are kept sorted by global cell index (instance base + row-major cell index), stable;
  * direction k disperses by cd_k = c_k * dx / cell; the component of moment m lands in cell
    S + floor(off + cd_k)  (propagation.py:39-51 with the division folded into the cell units).

Step, in order (each line cites the reference function it follows):
  1. collide every moment, per-instance tau, no vacuum guard       (warp/physics.py:45-62)
  2. thin: one control point (CP) per occupied cell, at the centroid of the components landing
     there                                                         (propagation.py:130-153)
  3. refine: kappa = number of distinct directions among components within r (inclusive); keep the
     CP if kappa <= kappa_hard, else move it to the exp(f)-weighted mean position, computed as
     p + sum(e^f e)/sum(e^f) with e the component's displacement from p  (propagation.py:77-112)
  4. stable-sort the CPs by the cell of their refined position (the next step's moment order)
  5. per component: sw = sum over CPs within r of (r - d); dropped if sw <= 0 (propagation.py:156-178)
  6. per CP and direction: f = sum over components within r of (r - d)*(1/sw) * f (propagation.py:179-186)
  7. gap fill: directions with f < eps get (r / sum_{CPs within r, also empty}(r - d)) * f_rest;
     emptiness is judged on the pre-fill values; emit one moment per CP      (propagation.py:189-218)
Optional soft-outer spawn (kappa_soft > 0; the reference CPU simulator's rule,
direbm/reference/simulator.py:126-166, which its Warp path omits): a CP with kappa_hard < kappa <=
kappa_soft also emits one new CP at p + n * 2(1 - sqrt(3)/2) dx, with p the CP's position before
its move and n the normalised sum of the direction vectors c of the components within r; no spawn
when |sum| <= 1e-8.  New CPs are not refined; they join the CP set before stage 4 (after the
regular CPs of the same cell).

The radius test uses one canonical operation order (each step rounded, no fused multiply-add),
with dS the integer cell difference (component cell - reference cell), cd = c*dx/cell and p the
reference point's offset in its cell:
    c = (float(dS) + cd) - p ;  e = off + c ;  d2 = sum e*e ;  inside = sqrt(d2) <= R
(c is shared by every candidate of one window cell, so a kernel pays one add per axis per
candidate).  It is evaluated in the working precision (float64, or float32 for the FP32 store),
so integer decisions are bit-identical to the CUDA kernels.  Sums are in float64 here unless
the kernel's order is reproduced (thinning centroids and refine sums, see ordered_sums); the
CUDA FP64 path then agrees bit for bit up to exp() rounding, the FP32 path to its stated
tolerance.

Parity pinning: stage 2 reduces to the reference tests' own numpy restatement of cell thinning
(tests/test_warp_propagation.py:27-36) when all components of an unbounded domain are given, and
stage 3 reproduces the ring fixtures of tests/test_warp_propagation.py:79-112; both are checked in
tests/test_oracle_golden.py.
"""

from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

from .lattices import Lattice
from .physics import collide_unguarded, equilibrium


@dataclass
class Instance:
    dims: tuple  # cells per axis
    origin: tuple = None  # world cell of local cell 0 (integer per axis)
    periodic: bool = True
    tau: float = 0.6
    rho_rest: float = 1.0
    obstacle: tuple = None  # (center (D,) world units, radius world units): a solid sphere / disc
    inflow: tuple = None  # (u (D,), width in cells): moments in the first `width` cell columns
    #                       are reset to the equilibrium at velocity u (their own density)


@dataclass
class GridSpec:
    lattice: Lattice
    dx: float
    r_res: float
    cell: float
    kappa_hard: int
    instances: list
    eps: float = 1e-6
    dtype: type = np.float64  # working precision of the decision arithmetic
    kappa_soft: int = 0  # soft-outer spawn for kappa_hard < kappa <= kappa_soft (0: off)
    base: np.ndarray = field(init=False)
    ncells: int = field(init=False)

    def __post_init__(self):
        D = self.lattice.D
        sizes = [int(np.prod(inst.dims)) for inst in self.instances]
        for inst in self.instances:
            assert len(inst.dims) == D
            if inst.origin is None:
                inst.origin = (0,) * D
        self.base = np.concatenate([[0], np.cumsum(sizes)]).astype(np.int64)
        self.ncells = int(self.base[-1])

    @property
    def D(self):
        return self.lattice.D

    @property
    def Q(self):
        return self.lattice.Q

    @property
    def cd(self):
        return (self.lattice.C * self.dx / self.cell).astype(self.dtype)

    @property
    def R(self):
        return self.dtype(self.r_res / self.cell)

    @property
    def soft_offset(self):
        """Spawn distance in cell units: 2(1 - sqrt(3)/2) dx (direbm/reference/simulator.py:27), FP64."""
        return 2.0 * (1.0 - np.sqrt(3.0) / 2.0) * float(self.dx) / float(self.cell)

    def dims_arr(self):
        return np.array([inst.dims for inst in self.instances], dtype=np.int64)

    def periodic_arr(self):
        return np.array([inst.periodic for inst in self.instances], dtype=bool)

    def tau_arr(self):
        return np.array([inst.tau for inst in self.instances], dtype=np.float64)

    def f_rest(self):
        W = self.lattice.W
        return np.array([inst.rho_rest * W for inst in self.instances])


# ---- cell indexing ----------------------------------------------------------------------------

def decode(spec: GridSpec, g):
    g = np.asarray(g, dtype=np.int64)
    b = np.searchsorted(spec.base, g, side="right") - 1
    local = g - spec.base[b]
    dims = spec.dims_arr()[b]
    coords = np.zeros((len(g), spec.D), dtype=np.int64)
    rem = local
    for a in range(spec.D):
        coords[:, a] = rem % dims[:, a]
        rem = rem // dims[:, a]
    return b, coords


def encode(spec: GridSpec, b, coords):
    """Global cell of (unwrapped) coords; -1 where a non-periodic instance has no such cell."""
    b = np.asarray(b, dtype=np.int64)
    coords = np.asarray(coords, dtype=np.int64)
    dims = spec.dims_arr()[b]
    per = spec.periodic_arr()[b]
    wrapped = np.where(per[:, None], np.mod(coords, dims), coords)
    inside = np.all((wrapped >= 0) & (wrapped < dims), axis=1)
    lin = np.zeros(len(b), dtype=np.int64)
    stride = np.ones(len(b), dtype=np.int64)
    for a in range(spec.D):
        lin += wrapped[:, a] * stride
        stride *= dims[:, a]
    return np.where(inside, spec.base[b] + lin, -1)


@dataclass
class GridState:
    cell: np.ndarray  # (M,) int64 global cell, sorted
    off: np.ndarray  # (M, D) offsets in [0,1), working dtype
    f: np.ndarray  # (M, Q) float64


def from_world(spec: GridSpec, inst_idx, pos, f):
    """World positions -> sorted grid state (s = x / cell in float64, floor, offset = s - floor,
    offset rounded to the working precision and clamped below 1)."""
    pos = np.asarray(pos, dtype=np.float64)
    inst_idx = np.asarray(inst_idx, dtype=np.int64)
    s = pos / np.float64(spec.cell)
    fl = np.floor(s)
    off = (s - fl).astype(spec.dtype)
    one_below = np.nextafter(spec.dtype(1.0), spec.dtype(0.0))
    off = np.minimum(off, one_below)
    origin = np.array([spec.instances[b].origin for b in inst_idx], dtype=np.int64).reshape(len(inst_idx), spec.D)
    coords = fl.astype(np.int64) - origin
    g = encode(spec, inst_idx, coords)
    if np.any(g < 0):
        raise ValueError("moment outside its instance box")
    order = np.argsort(g, kind="stable")
    return GridState(cell=g[order], off=off[order], f=np.asarray(f, dtype=np.float64)[order])


def to_world(spec: GridSpec, st: GridState):
    b, coords = decode(spec, st.cell)
    origin = np.array([spec.instances[i].origin for i in b], dtype=np.int64).reshape(len(b), spec.D)
    x = ((origin + coords).astype(np.float64) + st.off.astype(np.float64)) * np.float64(spec.cell)
    return b, x, st.f


# ---- canonical distance ------------------------------------------------------------------------

def disp(spec: GridSpec, dS, cd, p, off):
    """e = off + ((float(dS) + cd) - p), each step rounded in the working precision."""
    dt = spec.dtype
    c = ((dS.astype(dt) + np.asarray(cd, dt)).astype(dt) - p.astype(dt)).astype(dt)
    return (off.astype(dt) + c).astype(dt)


def norm(spec: GridSpec, e):
    dt = spec.dtype
    s = (e[:, 0] * e[:, 0]).astype(dt)
    for a in range(1, e.shape[1]):
        s = (s + (e[:, a] * e[:, a]).astype(dt)).astype(dt)
    return np.sqrt(s).astype(dt)


def _offsets(D, lo, hi):
    rng = np.arange(lo, hi + 1)
    grids = np.meshgrid(*([rng] * D), indexing="ij")
    return np.stack([gr.ravel() for gr in grids], axis=1)


def opposite(lattice):
    """Index of -c_k for every direction k."""
    C = lattice.C
    return np.array([int(np.flatnonzero(np.all(np.abs(C + C[k]) < 1e-12, axis=1))[0]) for k in range(len(C))])


def _obstacle_local(spec: GridSpec, b):
    """Sphere center in instance-local cell units and squared radius in cell units (FP64)."""
    inst = spec.instances[b]
    ctr = np.asarray(inst.obstacle[0], dtype=np.float64) / np.float64(spec.cell) - np.asarray(inst.origin, np.float64)
    r = np.float64(inst.obstacle[1]) / np.float64(spec.cell)
    return ctr, r * r


def inside_obstacle(spec: GridSpec, b, coords, off, shift=None):
    """Whether points (instance b, local integer cell coords, offsets [+ FP64 shift]) lie inside
    their instance's obstacle: end_a = ((double)S_a - ctr_a) + ((double)off_a [+ shift_a]),
    inside <=> sum_a end_a^2 < r^2, every operation in FP64 in this order (the kernels' order)."""
    b = np.asarray(b)
    out = np.zeros(len(b), dtype=bool)
    for bi in np.unique(b):
        if spec.instances[bi].obstacle is None:
            continue
        sel = b == bi
        ctr, r2 = _obstacle_local(spec, bi)
        o = np.asarray(off, dtype=np.float64)[sel]
        if shift is not None:
            o = o + np.asarray(shift, dtype=np.float64)[sel]
        rel = np.asarray(coords, dtype=np.float64)[sel] - ctr[None, :]
        end = rel + o
        d2 = end[:, 0] * end[:, 0]
        for a in range(1, spec.D):
            d2 = d2 + end[:, a] * end[:, a]
        out[sel] = d2 < r2
    return out


def blocked(spec: GridSpec, st: GridState):
    """(M, Q) bool: slot k of moment m is blocked when its dispersion end point (moment position +
    c_k dx) lies inside the instance's obstacle (bounce-back; the rest direction never is)."""
    M, Q = len(st.cell), spec.Q
    out = np.zeros((M, Q), dtype=bool)
    if all(inst.obstacle is None for inst in spec.instances) or M == 0:
        return out
    b, S = decode(spec, st.cell)
    cd64 = spec.lattice.C * np.float64(spec.dx) / np.float64(spec.cell)
    for k in range(1, Q):
        out[:, k] = inside_obstacle(spec, b, S, st.off.astype(np.float64), np.broadcast_to(cd64[k], (M, spec.D)))
    return out


def components(spec: GridSpec, st: GridState):
    """All (m, k) components (slots): moment index, slot direction, instance, source coords and
    t = off + displacement (working dtype), plus the label (the direction the component carries)
    and whether the slot is blocked.  An unblocked slot k sits at off + cd_k with label k; a blocked
    slot bounces back: it stays at off (displacement 0) with the opposite label, carrying f*_k."""
    M, Q = len(st.cell), spec.Q
    b, S = decode(spec, st.cell)
    m = np.repeat(np.arange(M), Q)
    k = np.tile(np.arange(Q), M)
    blk = blocked(spec, st).reshape(-1)
    cdv = np.where(blk[:, None], spec.dtype(0), spec.cd[k]).astype(spec.dtype)
    t = (st.off[m].astype(spec.dtype) + cdv).astype(spec.dtype)
    lab = np.where(blk, opposite(spec.lattice)[k], k)
    return m, k, b[m], S[m], t, lab, blk, cdv


# ---- the stages --------------------------------------------------------------------------------

def collide_state(spec: GridSpec, st: GridState):
    b, S = decode(spec, st.cell)
    fs = collide_unguarded(st.f, spec.tau_arr()[b], spec.lattice)
    for bi, inst in enumerate(spec.instances):
        if inst.inflow is None:
            continue
        sel = (b == bi) & (S[:, 0] < int(inst.inflow[1]))
        if sel.any():
            rho = st.f[sel].sum(1)
            u = np.broadcast_to(np.asarray(inst.inflow[0], dtype=np.float64), (int(sel.sum()), spec.D))
            fs[sel] = equilibrium(rho, u, spec.lattice)
    return fs


def ordered_sums(group, order_keys, vals, ngroups):
    """Per-group sequential sums of ``vals`` (N, ...) in the order given by ``order_keys`` (a list
    of key arrays, most significant first): each group is summed left to right with one rounding
    per addition, which is how one CUDA thread accumulates it."""
    vals = np.asarray(vals, dtype=np.float64)
    out = np.zeros((ngroups,) + vals.shape[1:])
    if len(group) == 0:
        return out
    idx = np.lexsort(tuple(reversed([group] + list(order_keys))))
    g = group[idx]
    v = vals[idx]
    head = np.ones(len(g), dtype=bool)
    head[1:] = g[1:] != g[:-1]
    starts = np.flatnonzero(head)
    lens = np.diff(np.append(starts, len(g)))
    gid = g[starts]
    acc = np.zeros((len(starts),) + vals.shape[1:])
    for j in range(int(lens.max())):
        live = lens > j
        acc[live] = acc[live] + v[starts[live] + j]
    out[gid] = acc
    return out


def _so_keys(dS, D):
    """Window offsets (z, y, x) as sort keys, in the kernels' loop nesting (z outer, x inner)."""
    z = dS[:, 2] if D == 3 else np.zeros(len(dS), np.int64)
    return [z, dS[:, 1], dS[:, 0]]


def thin(spec: GridSpec, st: GridState):
    """Stage 2.  Returns (occupied global cells sorted, count per CP, centroid rel (P,D),
    component landing cell per (m,k) (or -1 outside a non-periodic box)).  The centroid sum runs
    in the kernel's order: direction, then source-cell offset, then moment."""
    m, k, b, S, t, lab, blk, _ = components(spec, st)
    fl = np.floor(t).astype(np.int64)
    C = encode(spec, b, S + fl)
    rel = ((-fl).astype(spec.dtype) + t).astype(spec.dtype)
    ok = C >= 0
    cells, inv = np.unique(C[ok], return_inverse=True)
    cnt = np.bincount(inv, minlength=len(cells))
    so = -fl[ok]
    bo = blk[ok]
    # kernel order: regular components by (direction, source offset, moment), then the bounced ones
    # (which land in their own cell) by (moment, direction)
    keys = [bo.astype(np.int64), np.where(bo, 0, k[ok])] + _so_keys(so, spec.D) + [m[ok], np.where(bo, k[ok], 0)]
    sums = ordered_sums(inv, keys, rel[ok].astype(np.float64), len(cells))
    cen = (sums / cnt[:, None]).astype(spec.dtype)
    return cells, cnt, cen, C


def _pairs_comp_cp(spec, st, cp_cell, cp_off, comps=None):
    """(component, CP) pairs within R.  CPs are (global cell, offset), any number per cell.
    Returns comp index into the (m,k) list, CP index, d, the displacement e of the component from
    the CP (canonical order, see disp) and the integer cell difference dS = S - G."""
    if comps is None:
        comps = components(spec, st)
    m, k, b, S, t, lab, blk, cdv = comps
    fl = np.floor(t).astype(np.int64)
    order = np.argsort(cp_cell, kind="stable")
    cs = cp_cell[order]
    Rc = int(np.ceil(float(spec.R)))
    ci_all, pj_all, d_all, q_all, ds_all = [], [], [], [], []
    for o in _offsets(spec.D, -Rc - 1, Rc + 1):
        G = encode(spec, b, S + fl + o)
        lo = np.searchsorted(cs, G, side="left")
        hi = np.searchsorted(cs, G, side="right")
        cnt = np.where(G >= 0, hi - lo, 0)
        if cnt.sum() == 0:
            continue
        ci = np.repeat(np.arange(len(m)), cnt)
        within = np.arange(cnt.sum()) - np.repeat(np.cumsum(cnt) - cnt, cnt)
        pj = order[np.repeat(lo, cnt) + within]
        dS = -(fl[ci] + o)
        e = disp(spec, dS, cdv[ci], cp_off[pj], st.off[m[ci]])
        d = norm(spec, e)
        keep = d <= spec.R
        ci_all.append(ci[keep])
        pj_all.append(pj[keep])
        d_all.append(d[keep])
        q_all.append(e[keep])
        ds_all.append(dS[keep])
    if not ci_all:
        z = np.zeros(0, np.int64)
        return z, z, np.zeros(0, spec.dtype), np.zeros((0, spec.D), spec.dtype), np.zeros((0, spec.D), np.int64)
    return (np.concatenate(ci_all), np.concatenate(pj_all), np.concatenate(d_all), np.concatenate(q_all),
            np.concatenate(ds_all))


def refine(spec: GridSpec, st: GridState, fstar, cells, cen):
    """Stage 3.  Returns (mask, kappa, final global cell, final offset) per CP (thinning order)."""
    comps = components(spec, st)
    m, k, b, S, t, lab, blk, _ = comps
    ci, pj, d, e, dS = _pairs_comp_cp(spec, st, cells, cen, comps)
    P = len(cells)
    mask = np.zeros(P, dtype=np.int64)
    np.bitwise_or.at(mask, pj, np.left_shift(1, lab[ci]))
    kappa = np.array([bin(int(x)).count("1") for x in mask], dtype=np.int64)
    w = np.exp(fstar[m[ci], k[ci]])
    # sums in the kernel's order: regular components by direction, (2D FP32: the first moment of
    # each cell before the others,) window offset (z, y, x), moment; then bounced ones by window
    # offset, moment, direction
    bc = blk[ci]
    later = np.zeros(len(st.cell), dtype=np.int64)  # not the first moment of its cell
    if spec.dtype == np.float32 and spec.D == 2:
        later[1:] = st.cell[1:] == st.cell[:-1]
    keys = ([bc.astype(np.int64), np.where(bc, 0, k[ci]), np.where(bc, 0, later[m[ci]])] + _so_keys(dS, spec.D)
            + [m[ci], np.where(bc, k[ci], 0)])
    sw = ordered_sums(pj, keys, w, P)
    sx = ordered_sums(pj, keys, w[:, None] * e.astype(np.float64), P)
    move = kappa > spec.kappa_hard
    npos = cen.astype(spec.dtype).copy()
    step_ = (sx[move] / sw[move, None]).astype(spec.dtype)
    npos[move] = (npos[move] + step_).astype(spec.dtype)
    shift = np.floor(npos).astype(np.int64)
    off = (npos - shift.astype(spec.dtype)).astype(spec.dtype)
    over = off >= spec.dtype(1.0)
    off[over] = 0
    shift[over] += 1
    bcp, F = decode(spec, cells)
    G = encode(spec, bcp, F + shift)
    return mask, kappa, G, off


def direction_sum(n, C):
    """Sum of direction vectors from per-direction counts n (P, Q): acc = acc + n_k * c_k for
    k = 0..Q-1, FP64, one rounding per operation."""
    acc = np.zeros((n.shape[0], C.shape[1]))
    for q in range(C.shape[0]):
        acc = acc + n[:, q:q + 1].astype(np.float64) * C[q][None, :]
    return acc


def spawn_point(p, acc, offset):
    """p + (acc / |acc|) * offset and whether |acc| > 1e-8 (direbm/reference/simulator.py:153-166:
    c_sum, norm, normal, p.x + normal * _SOFT_OFFSET * dx), FP64, |acc| = sqrt(sum_a acc_a^2)."""
    nrm2 = acc[:, 0] * acc[:, 0]
    for a in range(1, acc.shape[1]):
        nrm2 = nrm2 + acc[:, a] * acc[:, a]
    nrm = np.sqrt(nrm2)
    go = nrm > 1e-8
    safe = np.where(go, nrm, 1.0)
    return p + (acc / safe[:, None]) * offset, go


def soft_spawn(spec: GridSpec, st: GridState, cells, cen, kappa):
    """Soft-outer spawn (direbm/reference/simulator.py:126-166).  Returns (global cell, offset) of the
    spawned CP per thinning CP (cell -1: none, or outside a bounded box).

    The direction sum follows the kernel's order, in FP64: the regular components as per-direction
    counts, acc = acc + n_k * c_k for k = 0..Q-1; the bounced ones (label opp(k)) one by one in
    window / moment / slot order into a second sum; then sum = acc + bounced.  The new point is
    cen + (sum / |sum|) * offset, |sum| = sqrt(sum_a sum_a^2), every operation rounded in FP64,
    split into cell + offset and the offset rounded to the working precision."""
    P = len(cells)
    G2 = np.full(P, -1, dtype=np.int64)
    off2 = np.zeros((P, spec.D), dtype=spec.dtype)
    soft = (kappa > spec.kappa_hard) & (kappa <= spec.kappa_soft)
    if spec.kappa_soft <= 0 or not soft.any():
        return G2, off2
    comps = components(spec, st)
    m, k, b, S, t, lab, blk, _ = comps
    ci, pj, d, e, dS = _pairs_comp_cp(spec, st, cells, cen, comps)
    C = np.asarray(spec.lattice.C, dtype=np.float64)
    reg = ~blk[ci]
    n = np.zeros((P, spec.Q), dtype=np.int64)
    np.add.at(n, (pj[reg], k[ci[reg]]), 1)
    acc = direction_sum(n, C)
    bc = ~reg
    if bc.any():
        keys = _so_keys(dS[bc], spec.D) + [m[ci[bc]], k[ci[bc]]]
        acc = acc + ordered_sums(pj[bc], keys, C[lab[ci[bc]]], P)
    sp, go = spawn_point(cen.astype(np.float64), acc, spec.soft_offset)
    go &= soft
    if not go.any():
        return G2, off2
    sp = sp[go]
    shift = np.floor(sp)
    o = (sp - shift).astype(spec.dtype)
    shift = shift.astype(np.int64)
    over = o >= spec.dtype(1.0)
    o[over] = 0
    shift[over] += 1
    bcp, F = decode(spec, cells[go])
    G2[go] = encode(spec, bcp, F + shift)
    off2[go] = o
    return G2, off2


def sort_cps(G):
    """Stage 4: stable ascending sort by final cell (ties keep thinning order)."""
    return np.argsort(G, kind="stable")


def weights(spec: GridSpec, st: GridState, cp_cell, cp_off, comps=None):
    """Stage 5.  sw per component (m,k) plus the pair list (ci, pj, d)."""
    if comps is None:
        comps = components(spec, st)
    m = comps[0]
    ci, pj, d, _, _ = _pairs_comp_cp(spec, st, cp_cell, cp_off, comps)
    wv = (spec.R - d).astype(np.float64)
    sw = np.zeros(len(m))
    np.add.at(sw, ci, wv)
    return sw, ci, pj, wv


def gather(spec: GridSpec, st: GridState, fstar, cp_cell, cp_off):
    """Stages 5+6.  Returns cp_f (P,Q) before gap fill and sw per component."""
    comps = components(spec, st)
    m, k, lab = comps[0], comps[1], comps[5]
    sw, ci, pj, wv = weights(spec, st, cp_cell, cp_off, comps)
    live = sw[ci] > 0.0
    P = len(cp_cell)
    cp_f = np.zeros((P, spec.Q))
    inv = np.zeros_like(sw)
    np.divide(1.0, sw, out=inv, where=sw > 0.0)
    # a component lands in the control point's f at its label (the opposite direction if it bounced)
    np.add.at(cp_f, (pj[live], lab[ci[live]]), (wv[live] * inv[ci[live]]) * fstar[m[ci[live]], k[ci[live]]])
    return cp_f, sw.reshape(-1, spec.Q)


def gapfill(spec: GridSpec, cp_cell, cp_off, cp_f):
    """Stage 7 (CP-CP distance from each CP's own perspective)."""
    P = len(cp_cell)
    empty = cp_f < spec.eps
    b, F = decode(spec, cp_cell)
    order = np.argsort(cp_cell, kind="stable")
    cs = cp_cell[order]
    Rc = int(np.ceil(float(spec.R)))
    a_all, c_all, w_all = [], [], []
    for o in _offsets(spec.D, -Rc - 1, Rc + 1):
        G = encode(spec, b, F + o)
        lo = np.searchsorted(cs, G, side="left")
        hi = np.searchsorted(cs, G, side="right")
        cnt = np.where(G >= 0, hi - lo, 0)
        if cnt.sum() == 0:
            continue
        ai = np.repeat(np.arange(P), cnt)
        within = np.arange(cnt.sum()) - np.repeat(np.cumsum(cnt) - cnt, cnt)
        cj = order[np.repeat(lo, cnt) + within]
        e = disp(spec, np.broadcast_to(o, (len(ai), spec.D)), 0.0, cp_off[ai], cp_off[cj])
        d = norm(spec, e)
        keep = d <= spec.R
        a_all.append(ai[keep])
        c_all.append(cj[keep])
        w_all.append((spec.R - d[keep]).astype(np.float64))
    ai = np.concatenate(a_all)
    cj = np.concatenate(c_all)
    ww = np.concatenate(w_all)
    out = cp_f.copy()
    f_rest = spec.f_rest()[b]
    for i in range(spec.Q):
        sel = empty[cj, i]
        s = np.zeros(P)
        np.add.at(s, ai[sel], ww[sel])
        fill = empty[:, i] & (s > 0.0)
        out[fill, i] = (float(spec.R) / s[fill]) * f_rest[fill, i]
    return out, empty


def step(spec: GridSpec, st: GridState, trace: dict | None = None) -> GridState:
    fstar = collide_state(spec, st)
    cells, cnt, cen, comp_cell = thin(spec, st)
    mask, kappa, G, off = refine(spec, st, fstar, cells, cen)
    if spec.kappa_soft > 0:  # spawned CPs follow the regular ones (slot order of the kernels)
        G2, off2 = soft_spawn(spec, st, cells, cen, kappa)
        G = np.concatenate([G, G2])
        off = np.concatenate([off, off2])
    keep = G >= 0
    if keep.any() and any(inst.obstacle is not None for inst in spec.instances):
        bq, Fq = decode(spec, np.where(keep, G, 0))
        keep &= ~inside_obstacle(spec, bq, Fq, off.astype(np.float64))  # solid: the point is removed
    order = sort_cps(np.where(keep, G, np.iinfo(np.int64).max))
    order = order[keep[order]]
    cp_cell = G[order]
    cp_off = off[order]
    cp_f, sw = gather(spec, st, fstar, cp_cell, cp_off)
    f_new, empty = gapfill(spec, cp_cell, cp_off, cp_f)
    if trace is not None:
        trace.update(
            fstar=fstar, thin_cells=cells, thin_count=cnt, centroid=cen, comp_cell=comp_cell,
            mask=mask, kappa=kappa, final_cell=G, final_off=off, order=order, sw=sw,
            cp_f=cp_f, empty=empty,
        )
    return GridState(cell=cp_cell, off=cp_off, f=f_new)


def run(spec: GridSpec, st: GridState, steps: int) -> GridState:
    for _ in range(steps):
        st = step(spec, st)
    return st
