"""The GPU path's stage functions on explicit component arrays (test oracle).

Restates direbm/warp/propagation.py (and the physics kernels of direbm/warp/physics.py) with the
same data layout the reference returns: positions (N, 2), values (N,), directions (N,), moments
(M, 7) -- all FP32 as in the Warp kernels.  Integer decisions (cell keys, the inclusive radius
test, the gap-fill emptiness test) are evaluated in exact IEEE FP32 so they match a CUDA kernel
that uses round-to-nearest intrinsics without contraction.  Where the reference sums in an order
that its tests do not pin (hash-grid query order, float atomics), this restatement sums in FP64;
tests compare those sums with an FP32 tolerance.
"""

from __future__ import annotations

import numpy as np

from .lattices import D2Q7, Lattice

F32 = np.float32


def disperse(pos_m, f_m, dx, lattice: Lattice = D2Q7):
    """pos_c[Q*i+k] = pos_m[i] + C[k]*dx; val_c = f[i,k]; dir_c = k (propagation.py:21-36)."""
    pos_m = np.asarray(pos_m, dtype=F32)
    f_m = np.asarray(f_m, dtype=F32)
    cdx = (lattice.C.astype(F32) * F32(dx)).astype(F32)  # C[k]*dx in fp32
    pos_c = (pos_m[:, None, :] + cdx[None, :, :]).astype(F32).reshape(-1, 2)
    val_c = f_m.reshape(-1).copy()
    dir_c = np.tile(np.arange(lattice.Q, dtype=np.int32), len(pos_m))
    return pos_c, val_c, dir_c


def cell_keys(pos_c, cs):
    """Integer cell (floor(x/cs), floor(y/cs)) with FP32 division (propagation.py:39-51)."""
    pos_c = np.asarray(pos_c, dtype=F32)
    q = (pos_c / F32(cs)).astype(F32)
    return np.floor(q).astype(np.int64)


def create_control_points(pos_c, cs):
    """Cell thinning (propagation.py:130-153): stable sort by (ix, iy), runs, sequential FP32
    centroid in sorted order.  Returns (cp_pos (P,2) fp32, order, run_start, run_len)."""
    pos_c = np.asarray(pos_c, dtype=F32)
    cells = cell_keys(pos_c, cs)
    # the reference packs (ix+B)*S + (iy+B): x-major, y-minor order
    order = np.lexsort((cells[:, 1], cells[:, 0]))  # stable; ties keep component index order
    sc = cells[order]
    if len(sc) == 0:
        return np.zeros((0, 2), F32), order, np.zeros(0, np.int64), np.zeros(0, np.int64)
    head = np.ones(len(sc), dtype=bool)
    head[1:] = np.any(sc[1:] != sc[:-1], axis=1)
    starts = np.flatnonzero(head)
    lens = np.diff(np.append(starts, len(sc)))
    sp = pos_c[order]
    acc = np.zeros((len(starts), 2), dtype=F32)
    for j in range(int(lens.max())):
        live = lens > j
        acc[live] = (acc[live] + sp[starts[live] + j]).astype(F32)
    cp = (acc / lens.astype(F32)[:, None]).astype(F32)
    return cp, order, starts, lens


def _dist32(a, b):
    """|a - b| in FP32: sub, square, add, sqrt -- each rounded (no fused multiply-add)."""
    d = (a - b).astype(F32)
    s = (d[..., 0] * d[..., 0]).astype(F32) + (d[..., 1] * d[..., 1]).astype(F32)
    return np.sqrt(s.astype(F32)).astype(F32)


def pairs_within(qpos, tpos, radius):
    """All (query, target) index pairs with FP32 distance <= radius, plus that distance."""
    qpos = np.asarray(qpos, dtype=F32)
    tpos = np.asarray(tpos, dtype=F32)
    r = F32(radius)
    if len(qpos) == 0 or len(tpos) == 0:
        return np.zeros(0, np.int64), np.zeros(0, np.int64), np.zeros(0, F32)
    qc = np.floor(qpos.astype(np.float64) / float(radius)).astype(np.int64)
    tc = np.floor(tpos.astype(np.float64) / float(radius)).astype(np.int64)
    base = tc.min(axis=0) - 4
    span = int((tc.max(axis=0) - base).max()) + 8
    tkey = (tc[:, 0] - base[0]) * span + (tc[:, 1] - base[1])
    torder = np.argsort(tkey, kind="stable")
    tks = tkey[torder]
    qi_all, ti_all = [], []
    for ox in range(-2, 3):
        for oy in range(-2, 3):
            cx = qc[:, 0] + ox - base[0]
            cy = qc[:, 1] + oy - base[1]
            ok = (cx >= 0) & (cy >= 0) & (cx < span) & (cy < span)
            key = cx * span + cy
            lo = np.searchsorted(tks, key, side="left")
            hi = np.searchsorted(tks, key, side="right")
            cnt = np.where(ok, hi - lo, 0)
            qi = np.repeat(np.arange(len(qpos)), cnt)
            starts = np.repeat(lo, cnt)
            within = np.arange(cnt.sum()) - np.repeat(np.cumsum(cnt) - cnt, cnt)
            qi_all.append(qi)
            ti_all.append(torder[starts + within])
    qi = np.concatenate(qi_all)
    ti = np.concatenate(ti_all)
    d = _dist32(tpos[ti], qpos[qi])
    keep = d <= r
    return qi[keep], ti[keep], d[keep]


def refine_control_points(cp_pos, pos_c, val_c, dir_c, dx, kappa_hard):
    """propagation.py:77-112: kappa = popcount of directions within dx (inclusive); keep if
    kappa <= kappa_hard else move to the exp(f)-weighted centroid.  Returns (new_pos, kappa)."""
    cp_pos = np.asarray(cp_pos, dtype=F32)
    pos_c = np.asarray(pos_c, dtype=F32)
    val_c = np.asarray(val_c, dtype=F32)
    dir_c = np.asarray(dir_c, dtype=np.int64)
    pi, ci, _ = pairs_within(cp_pos, pos_c, dx)
    mask = np.zeros(len(cp_pos), dtype=np.int64)
    np.bitwise_or.at(mask, pi, np.left_shift(1, dir_c[ci]))
    kappa = np.array([bin(int(m)).count("1") for m in mask], dtype=np.int64)
    w = np.exp(val_c[ci].astype(np.float64))
    sw = np.zeros(len(cp_pos))
    sx = np.zeros((len(cp_pos), 2))
    np.add.at(sw, pi, w)
    np.add.at(sx, pi, w[:, None] * pos_c[ci].astype(np.float64))
    move = kappa > kappa_hard
    new = cp_pos.astype(np.float64).copy()
    new[move] = sx[move] / sw[move, None]
    return new, kappa


def resample(pos_c, val_c, dir_c, cp_pos, dx, f_rest, eps=1e-6, Q=7):
    """propagation.py:156-218: scatter with (dx-d)/sum normalisation over each component's CPs
    (components with no CP within dx are dropped), then fill empty directions (f < eps, judged
    on the pre-fill values) with (dx / sum_{empty nbrs}(dx-d)) * f_rest.  Returns (pos, f, empty)."""
    pos_c = np.asarray(pos_c, dtype=F32)
    val_c = np.asarray(val_c, dtype=F32)
    dir_c = np.asarray(dir_c, dtype=np.int64)
    cp_pos = np.asarray(cp_pos, dtype=F32)
    f_rest = np.asarray(f_rest, dtype=np.float64)
    P = len(cp_pos)
    dxf = F32(dx)
    ci, pi, d = pairs_within(pos_c, cp_pos, dx)
    w = (dxf - d).astype(np.float64)
    sw = np.zeros(len(pos_c))
    np.add.at(sw, ci, w)
    live = sw[ci] > 0.0
    cp_f = np.zeros((P, Q))
    np.add.at(cp_f, (pi[live], dir_c[ci[live]]), (w[live] / sw[ci[live]]) * val_c[ci[live]].astype(np.float64))
    empty = cp_f < eps
    a, b, dd = pairs_within(cp_pos, cp_pos, dx)
    ww = (dxf - dd).astype(np.float64)
    out = cp_f.copy()
    for i in range(Q):
        sel = empty[b, i]
        s = np.zeros(P)
        np.add.at(s, a[sel], ww[sel])
        fill = empty[:, i] & (s > 0.0)
        out[fill, i] = (float(dx) / s[fill]) * f_rest[i]
    return cp_pos.astype(np.float64), out, empty
