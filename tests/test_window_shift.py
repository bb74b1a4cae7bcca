"""Host-side check of the shifted-window argument behind the tiled kernels' whole-cell form
(csrc/sim_tiled.cuh: win_rows, gather_cp_shift, refine_shift): with whole-cell displacements
(D2Q9, dx = cell), the per-direction window of a reference point and the cd = 0 window shifted by
-cd_k visit the same hits in the same order.  Evaluated in float32 with the kernels' rounding
order on random and near-boundary reference points (no GPU)."""

import numpy as np

f32 = np.float32
R = f32(1.5)
TINY = f32(1e-4)
CD = [(0, 0), (1, 0), (0, 1), (-1, 0), (0, -1), (1, 1), (-1, 1), (-1, -1), (1, -1)]


def _r2(r):
    """Largest float32 d2 whose correctly rounded square root is <= r."""
    d2 = f32(r * r)
    while np.sqrt(np.nextafter(d2, f32(np.inf))) <= r:
        d2 = np.nextafter(d2, f32(np.inf))
    while np.sqrt(d2) > r:
        d2 = np.nextafter(d2, f32(0))
    return d2


R2 = _r2(R)


def _axis_lower(c):
    hi = f32(c + f32(1))
    return c if c > 0 else (-hi if hi < 0 else f32(0))


def _halfwidth(lb):
    rem = f32(R2 - f32(lb * lb))
    if rem < -R2 * f32(1e-6):
        return f32(-1)
    x = f32(max(rem, f32(0)) + R2 * f32(9.5367431640625e-07))
    return f32(f32(np.sqrt(x)) * f32(1.0001) + f32(1e-6))


def _hits(p, off, rows):
    """Hits of one direction: rows = [(sy, cy, lo, hi)] in moment-cell coordinates relative to p's
    cell; off[(sx, sy)] is the moment offset there; candidate x uses c = (float(sx) + cd) - p."""
    out = []
    for sy, cy, lo, hi, cdx in rows:
        for sx in range(lo, hi + 1):
            o = off.get((sx, sy))
            if o is None:
                continue
            cx = f32(f32(f32(sx) + f32(cdx)) - p[0])
            ex, ey = f32(o[0] + cx), f32(o[1] + cy)
            if f32(f32(ex * ex) + f32(ey * ey)) <= R2:
                out.append((sx, sy))
    return out


def _per_direction(p, off, cdx, cdy):
    bxr, byr = f32(p[0] - f32(cdx)), f32(p[1] - f32(cdy))
    rows = []
    for sy in range(int(np.floor(f32(f32(byr - R) - TINY))), int(np.floor(f32(f32(byr + R) + TINY))) + 1):
        cy = f32(f32(f32(sy) + f32(cdy)) - p[1])
        hw = _halfwidth(_axis_lower(cy))
        if hw < 0:
            continue
        rows.append((sy, cy, int(np.floor(f32(f32(bxr - hw) - TINY))), int(np.floor(f32(f32(bxr + hw) + TINY))), cdx))
    return _hits(p, off, rows)


def _shifted(p, off, cdx, cdy):
    jlo = int(np.floor(f32(f32(p[1] - R) - TINY)))
    jhi = int(np.floor(f32(f32(p[1] + R) + TINY)))
    assert jhi - jlo + 1 <= 5  # the kernels' table height for R < 2 cells
    rows = []
    for jy in range(jlo, jhi + 1):
        cy = f32(f32(jy) - p[1])
        hw = _halfwidth(_axis_lower(cy))
        if hw < 0:
            continue
        a, b = int(np.floor(f32(f32(p[0] - hw) - TINY))), int(np.floor(f32(f32(p[0] + hw) + TINY)))
        rows.append((jy - cdy, cy, a - cdx, b - cdx, cdx))
    return _hits(p, off, rows)


def test_shifted_windows_visit_the_same_hits_in_the_same_order():
    rng = np.random.default_rng(11)
    edges = np.array([0.0, 0.5, 1 - 2 ** -24, 2 ** -24, 0.5 - 2 ** -25, 0.5 + 2 ** -24, 0.25, 0.75], dtype=np.float32)
    points = [rng.random(2).astype(np.float32) for _ in range(400)]
    points += [np.array([a, b], dtype=np.float32) for a in edges for b in edges]
    for t, p in enumerate(points):
        off = {(sx, sy): (f32(u), f32(v)) for sx in range(-4, 5) for sy in range(-4, 5)
               for u, v in [rng.random(2).astype(np.float32)]}
        if t % 3 == 0:  # offsets on the cell faces too
            for key in list(off)[::5]:
                off[key] = (f32(0), f32(edges[t % len(edges)]))
        for cdx, cdy in CD:
            assert _per_direction(p, off, cdx, cdy) == _shifted(p, off, cdx, cdy), (p, cdx, cdy)


def _lb_row(o_y, basey):
    ely, ehy = f32(o_y + f32(basey - f32(1))), f32(o_y + basey)
    return ely if ely > 0 else (-ehy if ehy < 0 else f32(0))


def _cp_hits(o, cps, rows):
    """Weights-side hits of component (moment offset o, direction cd): rows = [(gy, basey, lo, hi,
    cdx)] in control-point cell coordinates relative to the moment's cell; e = o + (base - p)."""
    out = []
    for gy, basey, lo, hi, cdx in rows:
        for gx in range(lo, hi + 1):
            p = cps.get((gx, gy))
            if p is None:
                continue
            basex = f32(f32(-gx) + f32(cdx))
            ex, ey = f32(o[0] + f32(basex - p[0])), f32(o[1] + f32(basey - p[1]))
            if f32(f32(ex * ex) + f32(ey * ey)) <= R2:
                out.append((gx, gy))
    return out


def test_shifted_weights_windows_visit_the_same_control_points():
    """The weights kernel's form: a component's control-point window rows depend on its moment's
    offset alone, shifted by cd_k (weights_rows_shift against weights_rows)."""
    rng = np.random.default_rng(12)
    edges = np.array([0.0, 0.5, 1 - 2 ** -24, 2 ** -24, 0.25], dtype=np.float32)
    offsets = [rng.random(2).astype(np.float32) for _ in range(300)]
    offsets += [np.array([a, b], dtype=np.float32) for a in edges for b in edges]
    for o in offsets:
        cps = {(gx, gy): rng.random(2).astype(np.float32) for gx in range(-4, 5) for gy in range(-4, 5)}
        for cdx, cdy in CD:
            tx, ty = f32(o[0] + f32(cdx)), f32(o[1] + f32(cdy))
            rows_a = []
            for gy in range(int(np.floor(f32(f32(ty - R) - TINY))), int(np.floor(f32(f32(ty + R) + TINY))) + 1):
                basey = f32(f32(-gy) + f32(cdy))
                hw = _halfwidth(_lb_row(o[1], basey))
                if hw >= 0:
                    rows_a.append((gy, basey, int(np.floor(f32(f32(tx - hw) - TINY))),
                                   int(np.floor(f32(f32(tx + hw) + TINY))), cdx))
            rows_b = []
            ulo, uhi = int(np.floor(f32(f32(o[1] - R) - TINY))), int(np.floor(f32(f32(o[1] + R) + TINY)))
            assert uhi - ulo + 1 <= 5
            for u in range(ulo, uhi + 1):
                basey = f32(-u)
                hw = _halfwidth(_lb_row(o[1], basey))
                if hw >= 0:
                    a, b = int(np.floor(f32(f32(o[0] - hw) - TINY))), int(np.floor(f32(f32(o[0] + hw) + TINY)))
                    rows_b.append((u + cdy, basey, a + cdx, b + cdx, cdx))
            assert _cp_hits(o, cps, rows_a) == _cp_hits(o, cps, rows_b), (o, cdx, cdy)
