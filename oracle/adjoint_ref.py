"""FP64 torch restatement of one DiReBM step with its discrete structure held fixed (test oracle
for the CUDA adjoint; test infrastructure only, never imported by the product).

A "tape" (a dict of numpy arrays, the layout ``direbm_gb300.adjoint.Tape.export`` returns) fixes
thinning membership, refine decisions and pairs, the sort order, resampling pairs, dropped
components, gap-filled directions and gap-fill pairs.  ``step_fixed`` evaluates the step as a
smooth function of (input offsets, input f, tau) for that structure, in float64 torch, so that
torch.autograd gives the reference gradient and central differences give the finite-difference
check.  Every pair displacement is the recorded one plus the change of its two end points:
    e(x) = e_rec + (x_item - x_item,rec) - (p_ref - p_ref,rec)
which is exactly how the step's canonical displacement (oracle/grid_step.py: disp) depends on the
continuous offsets (the integer cell differences are constants).  At the recorded point the output
equals the step's own output (oracle/grid_step.py: step) to rounding.

``tape_from_oracle`` records the same structure with the numpy oracle (oracle/grid_step.py), which
pins it to the reference's step: direbm/warp/propagation.py:130-218 (thinning, refine, resample,
gap fill) and direbm/warp/physics.py:45-62 (collision).
"""

from __future__ import annotations

import numpy as np
import torch

from . import grid_step as gs

NONE = -1


# ---- recording with the numpy oracle -----------------------------------------------------------

def _csr(rows, nrows):
    """Stable grouping of pair indices by row: (start (nrows+1,), order of the pairs)."""
    order = np.argsort(rows, kind="stable")
    counts = np.bincount(rows, minlength=nrows)
    start = np.concatenate([[0], np.cumsum(counts)]).astype(np.int64)
    return start, order


def tape_from_oracle(spec: gs.GridSpec, st: gs.GridState) -> tuple[dict, gs.GridState]:
    """Run one oracle step and record its structure; returns (tape, next state)."""
    Q, D = spec.Q, spec.D
    M = len(st.cell)
    trace = {}
    nxt = gs.step(spec, st, trace)
    fstar = trace["fstar"]
    cells, cnt, cen = trace["thin_cells"], trace["thin_count"], trace["centroid"]
    order = trace["order"]
    P = len(order)
    comps = gs.components(spec, st)
    # refine pairs (thin CP index) -> rows in sorted order, moved CPs only
    ci, pj, d, e, _ = gs._pairs_comp_cp(spec, st, cells, cen, comps)
    moved_thin = trace["kappa"] > spec.kappa_hard
    sorted_of_thin = np.full(len(cells), -1, dtype=np.int64)
    sorted_of_thin[order] = np.arange(P)
    keep = (sorted_of_thin[pj] >= 0) & moved_thin[pj]
    rows = sorted_of_thin[pj[keep]] * Q + comps[1][ci[keep]]
    rstart, rord = _csr(rows, P * Q)
    # resampling pairs
    cp_cell, cp_off = nxt.cell, nxt.off
    ci2, pj2, d2, e2, _ = gs._pairs_comp_cp(spec, st, cp_cell, cp_off, comps)
    k2 = comps[1][ci2]
    gstart, gord = _csr(pj2 * Q + k2, P * Q)
    # gap-fill pairs (as oracle/grid_step.py: gapfill enumerates them)
    empty = trace["empty"]
    ebits = (empty.astype(np.int64) << np.arange(Q)).sum(1)
    b, F = gs.decode(spec, cp_cell)
    srt = np.argsort(cp_cell, kind="stable")
    cs = cp_cell[srt]
    Rc = int(np.ceil(float(spec.R)))
    a_all, c_all, e_all = [], [], []
    for o in gs._offsets(D, -Rc - 1, Rc + 1):
        G = gs.encode(spec, b, F + o)
        lo = np.searchsorted(cs, G, side="left")
        hi = np.searchsorted(cs, G, side="right")
        n = np.where(G >= 0, hi - lo, 0)
        if n.sum() == 0:
            continue
        ai = np.repeat(np.arange(P), n)
        within = np.arange(n.sum()) - np.repeat(np.cumsum(n) - n, n)
        cj = srt[np.repeat(lo, n) + within]
        ee = gs.disp(spec, np.broadcast_to(o, (len(ai), D)), 0.0, cp_off[ai], cp_off[cj])
        keep_g = (gs.norm(spec, ee) <= spec.R) & ((ebits[ai] & ebits[cj]) != 0)
        a_all.append(ai[keep_g])
        c_all.append(cj[keep_g])
        e_all.append(ee[keep_g])
    ga = np.concatenate(a_all) if a_all else np.zeros(0, np.int64)
    gc = np.concatenate(c_all) if c_all else np.zeros(0, np.int64)
    ge = np.concatenate(e_all) if e_all else np.zeros((0, D))
    fstart, ford = _csr(ga, P)
    sw = trace["sw"]
    inv = np.zeros_like(sw)
    np.divide(1.0, sw, out=inv, where=sw > 0)
    binst, _ = gs.decode(spec, st.cell)
    inst_start = np.searchsorted(binst, np.arange(len(spec.instances) + 1), side="left")
    thin_cell = trace["comp_cell"].reshape(M, Q).astype(np.int64)
    tape = {
        "counts": {"M": M, "P": P, "refine": int(keep.sum()), "resample": len(ci2), "gapfill": len(ga)},
        "in_cell": st.cell.astype(np.int64), "in_off": st.off.astype(np.float64), "in_f": st.f.astype(np.float64),
        "fstar": fstar, "thin_cell": np.where(thin_cell < 0, NONE, thin_cell),
        "cp_thin": cells[order], "cp_count": cnt[order], "cp_cen": cen[order].astype(np.float64),
        "cp_moved": moved_thin[order].astype(np.int64), "out_cell": cp_cell, "out_off": cp_off.astype(np.float64),
        "empty": ebits, "inv_sw": inv.reshape(M, Q),
        "ref_start": rstart, "ref_item": ci[keep][rord], "ref_e": e[keep][rord].astype(np.float64),
        "res_start": gstart, "res_item": ci2[gord], "res_e": e2[gord].astype(np.float64),
        "gap_start": fstart, "gap_item": gc[ford], "gap_bits": (ebits[ga] & ebits[gc])[ford],
        "gap_e": ge[ford].astype(np.float64), "inst_start": inst_start,
    }
    return tape, nxt


# ---- the fixed-structure step in torch -----------------------------------------------------------

def collide(f, tau_m, lattice):
    """BGK collision without a vacuum guard (direbm/warp/physics.py:45-62), torch float64."""
    C = torch.as_tensor(lattice.C, dtype=f.dtype)
    W = torch.as_tensor(lattice.W, dtype=f.dtype)
    inv = 1.0 / lattice.cs2
    rho = f.sum(1)
    u = (f @ C) / rho[:, None]
    cu = u @ C.T
    usq = (u * u).sum(1, keepdim=True)
    feq = rho[:, None] * W[None, :] * (1 + inv * cu + 0.5 * inv * inv * cu * cu - 0.5 * inv * usq)
    return f + (feq - f) / tau_m[:, None]


def safe_norm(e):
    """|e| with the subgradient 0 at zero."""
    d2 = (e * e).sum(1)
    pos = d2 > 0
    return torch.where(pos, torch.sqrt(torch.where(pos, d2, torch.ones_like(d2))), torch.zeros_like(d2))


def _rows(start):
    start = np.asarray(start, dtype=np.int64)
    return np.repeat(np.arange(len(start) - 1), np.diff(start))


def step_fixed(T: dict, lattice, R: float, base, rho_rest, off_in, f_in, tau):
    """One step for the structure of tape T.  off_in (M, D) offsets in cell units, f_in (M, Q),
    tau (n_inst,) float64 torch tensors; base (n_inst+1,) first global cell of each instance;
    rho_rest (n_inst,).  Returns (out offsets (P, D), out f (P, Q))."""
    Q, D = lattice.Q, lattice.D
    M, P = T["counts"]["M"], T["counts"]["P"]
    Rt = float(R)
    W = torch.as_tensor(lattice.W, dtype=torch.float64)
    in_cell = np.asarray(T["in_cell"])
    inst_m = torch.as_tensor(np.searchsorted(np.asarray(base), in_cell, side="right") - 1)
    fs = collide(f_in, tau[inst_m], lattice)
    fs_rec = torch.as_tensor(T["fstar"])
    dX = off_in - torch.as_tensor(T["in_off"])
    # thinning: components -> sorted CP j through the thin cell
    cp_thin = np.asarray(T["cp_thin"])
    thin = np.asarray(T["thin_cell"]).reshape(-1)
    srt = np.argsort(cp_thin)
    loc = np.searchsorted(cp_thin[srt], thin)
    loc = np.minimum(loc, max(len(cp_thin) - 1, 0))
    hit = (thin >= 0) & (len(cp_thin) > 0)
    if len(cp_thin):
        hit &= cp_thin[srt][loc] == thin
    comp = np.flatnonzero(hit)
    jt = srt[loc[comp]]
    dcen = torch.zeros((P, D), dtype=torch.float64).index_add_(0, torch.as_tensor(jt), dX[torch.as_tensor(comp // Q)])
    dcen = dcen / torch.as_tensor(np.asarray(T["cp_count"]), dtype=torch.float64).clamp(min=1)[:, None]
    # refine: p = cen + sum w e / sum w for the moved CPs (rows are CP x direction)
    rrow = torch.as_tensor(_rows(T["ref_start"]) // Q)
    ritem = np.asarray(T["ref_item"])
    rm, rk = torch.as_tensor(ritem // Q), torch.as_tensor(ritem % Q)
    e_r = torch.as_tensor(T["ref_e"]) + dX[rm] - dcen[rrow]
    w = torch.exp(fs[rm, rk])
    w0 = torch.exp(fs_rec[rm, rk])
    Wt = torch.zeros(P, dtype=torch.float64).index_add_(0, rrow, w)
    W0 = torch.zeros(P, dtype=torch.float64).index_add_(0, rrow, w0)
    sx = torch.zeros((P, D), dtype=torch.float64).index_add_(0, rrow, w[:, None] * e_r)
    sx0 = torch.zeros((P, D), dtype=torch.float64).index_add_(0, rrow, w0[:, None] * torch.as_tensor(T["ref_e"]))
    moved = torch.as_tensor(np.asarray(T["cp_moved"]) > 0)
    Ws = torch.where(moved, Wt, torch.ones_like(Wt))
    W0s = torch.where(moved, W0, torch.ones_like(W0))
    ds = torch.where(moved[:, None], sx / Ws[:, None] - sx0 / W0s[:, None], torch.zeros_like(sx))
    dP = dcen + ds
    out_off = torch.as_tensor(T["out_off"]) + dP
    # resampling: F_jk = sum (R - d)/sw_i f*_i
    grow = _rows(T["res_start"])
    gj = torch.as_tensor(grow // Q)
    gitem = np.asarray(T["res_item"])
    gi = torch.as_tensor(gitem)
    gm, gk = torch.as_tensor(gitem // Q), torch.as_tensor(gitem % Q)
    e_g = torch.as_tensor(T["res_e"]) + dX[gm] - dP[gj]
    wg = Rt - safe_norm(e_g)
    sw = torch.zeros(M * Q, dtype=torch.float64).index_add_(0, gi, wg)
    live = torch.as_tensor(np.asarray(T["inv_sw"]).reshape(-1)[gitem] > 0)
    sws = torch.where(live, sw[gi], torch.ones_like(wg))
    contrib = torch.where(live, wg / sws * fs[gm, gk], torch.zeros_like(wg))
    F = torch.zeros(P * Q, dtype=torch.float64).index_add_(0, torch.as_tensor(grow), contrib).reshape(P, Q)
    # gap fill
    frow = torch.as_tensor(_rows(T["gap_start"]))
    fl = torch.as_tensor(np.asarray(T["gap_item"]))
    fbits = np.asarray(T["gap_bits"])
    e_f = torch.as_tensor(T["gap_e"]) + dP[fl] - dP[frow]
    wf = Rt - safe_norm(e_f)
    em = np.asarray(T["empty"])
    out_cell = np.asarray(T["out_cell"])
    inst_p = np.searchsorted(np.asarray(base), out_cell, side="right") - 1
    rr = torch.as_tensor(np.asarray(rho_rest, dtype=np.float64)[inst_p])
    cols = []
    for k in range(Q):
        sel = torch.as_tensor(((fbits >> k) & 1) > 0)
        s = torch.zeros(P, dtype=torch.float64).index_add_(0, frow[sel], wf[sel])
        fill = torch.as_tensor(((em >> k) & 1) > 0) & (s > 0)
        ss = torch.where(fill, s, torch.ones_like(s))
        cols.append(torch.where(fill, (Rt / ss) * rr * W[k], F[:, k]))
    return out_off, torch.stack(cols, dim=1)
