// Shared-memory tiled variants of the three window-loop kernels of the fused step (2D).
//
// A block owns a tile of tx x ty cells of one instance.  It stages everything its window loops
// can touch -- the moments (or control points) of the tile plus a halo -- from the sorted cell
// ranges into shared memory once, with coalesced row-segment copies, and then every thread runs
// its loops out of shared memory.  The per-thread loop order is the same as in the untiled
// kernels, so results are bit-identical to them and the FP64 path stays bit-compatible with the
// oracle.  With the FP32 store (kFirstItemsFirst), a window sum takes per direction the first item
// of every window cell (window rows ascending, columns ascending), then, if a window cell holds
// more, a second pass takes the other items in the same cell order; with FP64 the items of each
// cell in order.  Two-item cells are rare (refine moves that cross a cell face), so the second
// pass is rare too.
//
// Regions hold a data-dependent number of items.  When a region holds more than the shared-memory
// capacity, the block keeps global indices in its range table and reads the items from global
// memory instead (same code, same order): correctness never depends on the capacity.
#pragma once

#include "sim.cuh"

namespace dbm {

struct Tile2 {
  int inst;
  int x0, y0;
};

// Halo of a region around a tile: region cells x in [x0 + xl, x0 + tx - 1 + xh] (same for y).
struct Halo {
  int xl, xh, yl, yh;
};

struct TileGeo {
  int tx, ty;
  Halo mom;  // moments around a cell / control-point tile (thin+refine, gather)
  Halo cp;   // control points around a moment tile (weights)
  int cap_refine, cap_gather, cap_weights;  // staged region items per block
  int cap_tile;                             // tile item list entries per block
};

__device__ __forceinline__ int warp_sum(int v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ int warp_incl_scan(int v) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    int y = __shfl_up_sync(0xffffffffu, v, o);
    if (lane >= o) v += y;
  }
  return v;
}

// Global cell of unwrapped 2D coordinates for region staging.  A region may be wider than a small
// periodic box (it then holds some cells twice, which is harmless: one window never spans a box),
// so periodic coordinates are wrapped as often as needed (a region coordinate lies within a few
// halo widths of the box, so this is at most a few steps and usually none, cheaper than a modulo).
__device__ __forceinline__ bool region_cell(const InstK& I, int x, int y, uint32_t* g) {
  const int nx = I.dims[0], ny = I.dims[1];
  if (I.periodic) {
    while (x < 0) x += nx;
    while (x >= nx) x -= nx;
    while (y < 0) y += ny;
    while (y >= ny) y -= ny;
  } else if (x < 0 || x >= nx || y < 0 || y >= ny) {
    return false;
  }
  *g = I.base + (uint32_t)x + (uint32_t)nx * (uint32_t)y;
  return true;
}

// Stage the items of region cells [xr0, xr0 + rw) x [yr0, yr0 + rh) (unwrapped coordinates).
// On return (after a barrier) s_beg/s_end[ry * rw + rx] is each cell's half-open item range:
// local indices into the staged arrays when *s_local != 0, global indices otherwise.
// copy(global, local, region column) is called once per staged item.  Needs rh + 2 ints at s_row.
template <class Copy>
__device__ __forceinline__ void stage_region(const InstK& I, int xr0, int yr0, int rw, int rh,
                                             const uint32_t* __restrict__ start, int cap, int* s_beg, int* s_end,
                                             int* s_row, Copy&& copy) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int ry = warp; ry < rh; ry += nw) {
    int cnt = 0;
    for (int rx = lane; rx < rw; rx += 32) {
      uint32_t g;
      if (region_cell(I, xr0 + rx, yr0 + ry, &g)) cnt += (int)(start[g + 1] - start[g]);
    }
    cnt = warp_sum(cnt);
    if (lane == 0) s_row[ry] = cnt;
  }
  __syncthreads();
  if (warp == 0) {  // exclusive prefix over the region rows, 32 at a time
    int acc = 0;
    for (int r0 = 0; r0 < rh; r0 += 32) {
      const int ry = r0 + lane;
      const int c = ry < rh ? s_row[ry] : 0;
      const int incl = warp_incl_scan(c);
      if (ry < rh) s_row[ry] = acc + incl - c;
      acc += __shfl_sync(0xffffffffu, incl, 31);
    }
    if (lane == 0) {
      s_row[rh] = acc;
      s_row[rh + 1] = acc <= cap ? 1 : 0;
    }
  }
  __syncthreads();
  const bool local = s_row[rh + 1] != 0;
  for (int ry = warp; ry < rh; ry += nw) {
    int base = s_row[ry];
    for (int rx0 = 0; rx0 < rw; rx0 += 32) {
      const int rx = rx0 + lane;
      uint32_t g;
      int b = 0, e = 0;
      if (rx < rw && region_cell(I, xr0 + rx, yr0 + ry, &g)) {
        b = (int)start[g];
        e = (int)start[g + 1];
      }
      const int cnt = e - b;
      const int incl = warp_incl_scan(cnt);
      const int lb = base + incl - cnt;
      if (rx < rw) {
        const int ci = ry * rw + rx;
        s_beg[ci] = local ? lb : b;
        s_end[ci] = local ? lb + cnt : e;
      }
      if (local)
        for (int i = 0; i < cnt; ++i) copy(b + i, lb + i, rx);
      base += __shfl_sync(0xffffffffu, incl, 31);
    }
  }
  __syncthreads();
}

template <class T>
__device__ __forceinline__ T* carve(unsigned char*& p, int n) {
  uintptr_t a = ((uintptr_t)p + 15) & ~(uintptr_t)15;
  T* r = (T*)a;
  p = (unsigned char*)(a + (size_t)n * sizeof(T));
  return r;
}

template <class real>
struct alignas(2 * sizeof(real)) Pair {
  real x, y;
};

// A staged item for the row-segment loops: its offsets and the region column of its cell as an
// exact small integer in floating point (so float(dS_x) = rx - bx without a conversion).
template <class real>
struct alignas(4 * sizeof(real)) Item {
  real ox, oy, rx, pad;
};

// Lower bound of |e| on one axis over a window row/column whose candidates have e in
// [fl(c), fl(c + 1)] (offsets in [0, 1), rounding monotonic).
template <class real>
__device__ __forceinline__ real axis_lower(real c) {
  const real hi = rn_add(c, (real)1);
  return c > (real)0 ? c : (hi < (real)0 ? -hi : (real)0);
}

// Half-width bound on |e_x| for a window row whose |e_y| >= lby: any hit has fl(e_x^2) + lb_y^2 <=
// R2 up to one rounding of the sum, so |e_x| <= sqrt(R2 - lby^2 + R2 * 2^-20).  Returns < 0 if
// the row cannot hold a hit.
template <class real>
__device__ __forceinline__ real row_halfwidth(real R2, real lby) {
  const float rem = (float)(R2 - lby * lby);
  if (rem < -(float)R2 * 1e-6f) return (real)-1;
  // a fast square root is enough for a bound: inflate it well past its error
  const float x = fmaxf(rem, 0.f) + (float)R2 * 9.5367431640625e-07f;
  return (real)(bound_sqrt(x) * 1.0001f + 1e-6f);
}

// ---- thinning + refine ------------------------------------------------------------------------
//
// One thread per cell of the tile.  Thinning needs only moment offsets; refine runs one direction
// at a time so that only exp(f*) of that direction is staged.  LOCAL selects shared-memory or
// global-memory operands at compile time (the block decides at run time which one it needs).

template <int Q, class P, bool LOCAL>
__device__ __forceinline__ void thin_refine_body(const Args<Q, 2, P>& A, const InstK& I, const Tile2& T,
                                                 const TileGeo& G, int rw, int rh, const int* s_beg, const int* s_end,
                                                 const int* s_gi, const Pair<typename P::real>* s_pos,
                                                 typename P::real* s_w, int nstaged) {
  using real = typename P::real;
  constexpr bool F64 = std::is_same<P, PF64>::value;
  const int lx = threadIdx.x % G.tx, ly = threadIdx.x / G.tx;
  const int Fx = T.x0 + lx, Fy = T.y0 + ly;
  const bool valid = ly < G.ty && Fx < I.dims[0] && Fy < I.dims[1];
  const uint32_t F = valid ? I.base + (uint32_t)Fx + (uint32_t)I.dims[0] * (uint32_t)Fy : 0u;
  const real* gox = A.a.off;
  const real* goy = A.a.off + A.mcap;
  auto pos = [&](int m) -> Pair<real> {
    if constexpr (LOCAL) return s_pos[m];
    else return Pair<real>{gox[m], goy[m]};
  };
  const int bx = lx - G.mom.xl, by = ly - G.mom.yl;  // region coordinates of F

  // thinning: component (m, k) lands in F iff floor(off + cd) == -so on both axes
  uint32_t cnt = 0;
  real cen[3] = {0, 0, 0};
  if (valid) {
    real sum[2] = {0, 0};
    CSum csum[2];
#pragma unroll 1
    for (int k = 0; k < Q; ++k) {
      const real cdx = A.L.template cd_as<real>(k, 0), cdy = A.L.template cd_as<real>(k, 1);
      int lox, nx, loy, ny;
      thin_sources<real>(cdx, &lox, &nx);
      thin_sources<real>(cdy, &loy, &ny);
#pragma unroll 1
      for (int oy = 0; oy < ny; ++oy)
#pragma unroll 1
        for (int ox = 0; ox < nx; ++ox) {
          const int sox = lox + ox, soy = loy + oy;
          const real fx0 = (real)(-sox), fy0 = (real)(-soy);
          const int ci = (by + soy) * rw + (bx + sox);
          const int m1 = s_end[ci];
          for (int m = s_beg[ci]; m < m1; ++m) {
            const Pair<real> o = pos(m);
            const real tx = rn_add(o.x, cdx), ty = rn_add(o.y, cdy);
            if (tx >= fx0 && tx < fx0 + (real)1 && ty >= fy0 && ty < fy0 + (real)1) {
              ++cnt;
              const real rx = rn_add((real)sox, tx), ry = rn_add((real)soy, ty);
              if constexpr (F64) {
                sum[0] += rx;
                sum[1] += ry;
              } else {
                csum[0].add(rx);
                csum[1].add(ry);
              }
            }
          }
        }
    }
    if (cnt) {
      if constexpr (F64) {
        cen[0] = sum[0] / (real)cnt;
        cen[1] = sum[1] / (real)cnt;
      } else {
        cen[0] = csum[0].value() / (real)cnt;
        cen[1] = csum[1].value() / (real)cnt;
      }
    }
  }
  const bool occupied = valid && cnt > 0;

  // refine, one direction at a time; the move is cen + sum(w e) / sum(w)
  uint32_t mask = 0;
  double swd = 0, sxd[2] = {0, 0};
  float swf = 0.f, sxf[2] = {0.f, 0.f};
#pragma unroll 1
  for (int k = 0; k < Q; ++k) {
    if constexpr (LOCAL) {
      __syncthreads();
      for (int l = threadIdx.x; l < nstaged; l += blockDim.x) s_w[l] = exp(fstar_at<Q, 2, P>(A, (uint32_t)s_gi[l], k));
      __syncthreads();
    }
    if (!occupied) continue;
    const real cdx = A.L.template cd_as<real>(k, 0), cdy = A.L.template cd_as<real>(k, 1);
    const real bxr = cen[0] - cdx, byr = cen[1] - cdy;
    const int lox = max((int)floor(bxr - A.R - A.tiny), -bx), hix = min((int)floor(bxr + A.R + A.tiny), rw - 1 - bx);
    const int loy = max((int)floor(byr - A.R - A.tiny), -by), hiy = min((int)floor(byr + A.R + A.tiny), rh - 1 - by);
    bool more = false;  // (2D FP32) a window cell holds a second item: a second pass takes those
#pragma unroll 1
    for (int pass = 0; pass <= (int)(kFirstItemsFirst<P, 2> && more); ++pass)
#pragma unroll 1
    for (int sy = loy; sy <= hiy; ++sy) {
      const real cy = canon_c<real>(sy, cdy, cen[1]);
#pragma unroll 1
      for (int sx = lox; sx <= hix; ++sx) {
        const real c[3] = {canon_c<real>(sx, cdx, cen[0]), cy, 0};
        if (cell_d2_lower<2, real>(c) > A.R2) continue;
        const int ci = (by + sy) * rw + (bx + sx);
        const int mb = s_beg[ci], me = s_end[ci];
        more |= me - mb > 1;
        const int m0 = pass ? mb + 1 : mb, m1 = (pass || !kFirstItemsFirst<P, 2>) ? me : min(me, mb + 1);
        for (int m = m0; m < m1; ++m) {
          const Pair<real> o2 = pos(m);
          const real o[3] = {o2.x, o2.y, 0};
          real e[3];
          if (canon_d2<2, real>(o, c, e) <= A.R2) {
            mask |= 1u << k;
            real w;
            if constexpr (LOCAL) w = s_w[m];
            else w = exp(fstar_at<Q, 2, P>(A, (uint32_t)m, k));
            if constexpr (F64) {
              swd = __dadd_rn(swd, w);
              sxd[0] = __dadd_rn(sxd[0], __dmul_rn(w, e[0]));
              sxd[1] = __dadd_rn(sxd[1], __dmul_rn(w, e[1]));
            } else {
              swf += w;
              sxf[0] = fmaf(w, e[0], sxf[0]);
              sxf[1] = fmaf(w, e[1], sxf[1]);
            }
          }
        }
      }
    }
  }
  if (!valid) return;
  if (!occupied) {
    A.occ[F] = 0u;
    if (A.write_trace) {
      A.tcnt[F] = 0u;
      A.mask[F] = 0u;
    }
    return;
  }
  const int kappa = __popc(mask);
  real np[2];
#pragma unroll
  for (int a = 0; a < 2; ++a) {
    if (kappa <= A.kappa_hard) np[a] = cen[a];
    else if constexpr (F64) np[a] = __dadd_rn(cen[a], __ddiv_rn(sxd[a], swd));
    else np[a] = cen[a] + sxf[a] / swf;
  }
  bool finite = true;
#pragma unroll
  for (int a = 0; a < 2; ++a) finite &= isfinite(np[a]) && fabs(np[a]) < (real)64;
  if (!finite) {
    atomicOr(A.status, ST_NONFINITE);
    np[0] = cen[0];
    np[1] = cen[1];
  }
  int sh[2];
  real off[2];
#pragma unroll
  for (int a = 0; a < 2; ++a) {
    const real fl = floor(np[a]);
    sh[a] = (int)fl;
    off[a] = np[a] - fl;
    if (off[a] >= (real)1) {
      off[a] = 0;
      sh[a] += 1;
    }
  }
  uint32_t Gc;
  const bool inside = cell_at<2>(I, Fx + sh[0], Fy + sh[1], 0, &Gc);
  if (!inside) atomicOr(A.status, ST_OUT_OF_BOX);
  A.occ[F] = inside ? 1u : 0u;
  A.fkey[F] = inside ? Gc : 0xffffffffu;
  A.foff[F] = off[0];
  A.foff[(int64_t)A.ncells + F] = off[1];
  if (A.write_trace) {
    A.tcnt[F] = cnt;
    A.mask[F] = mask;
    A.cen[F] = cen[0];
    A.cen[(int64_t)A.ncells + F] = cen[1];
  }
}

// ---- whole-cell displacements: one window-row table per reference point ------------------------
//
// When every displacement cd_k is a whole number of cells (D2Q9 with dx = cell), the canonical
// c = (float(dS) + cd_k) - p of a window cell is rn_sub(float(j), p) with j = dS + cd_k exact, so
// direction k's window around a reference point p is the window of cd = 0 shifted by -cd_k:
// component row j (relative to p's cell) has the same c_y, the same half-width bound and the
// same column range [a_j, b_j] for every direction; only the moment row j - cd_k,y and the moment
// columns [a_j - cd_k,x, b_j - cd_k,x] move.  The table of rows is built once per reference point
// instead of once per (point, direction).  The window bounds keep their 1e-4 cell margin, which
// is far above the rounding of p - cd, so every hit lies inside the shifted window and the hits
// are visited in the same order (rows ascending, then the row's items, first items before the
// others): sums are bit-identical to
// the per-direction windows.

// Rows of the whole-cell window tables: NR >= floor(2R + 2 tiny) + 2 (R < 2 cells).
constexpr int kShiftRows = 5;

template <int NR>
struct WinRows {
  int jlo, nr;
  float cy[NR];
  int a[NR], b[NR];
};

template <int NR, class ArgsT>
__device__ __forceinline__ void win_rows(const ArgsT& A, Pair<float> p, WinRows<NR>& w) {
  w.jlo = (int)floorf(p.y - A.R - A.tiny);
  const int n = (int)floorf(p.y + A.R + A.tiny) - w.jlo + 1;
  if (n > NR) atomicOr(A.status, ST_INTERNAL);  // the host sizes NR for R; never expected
  w.nr = min(n, NR);
#pragma unroll
  for (int t = 0; t < NR; ++t) {
    const float cy = rn_sub((float)(w.jlo + t), p.y);
    const float hw = row_halfwidth<float>(A.R2, axis_lower<float>(cy));
    w.cy[t] = cy;
    const bool on = t < w.nr && hw >= 0.f;
    w.a[t] = on ? (int)floorf(p.x - hw - A.tiny) : 1;
    w.b[t] = on ? (int)floorf(p.x + hw + A.tiny) : 0;
  }
}

// The refine sums of one centroid over the shifted windows of every direction (FP32 store): the
// loop of thin_refine_rows with the row table built once.
template <int Q, int NR>
__device__ __forceinline__ void refine_shift(const Args<Q, 2, PF32>& A, int rw, int rh, const int* s_beg,
                                             const int* s_end, const Item<float>* s_it, const float* s_w, int cap,
                                             int bx, int by, Pair<float> c, uint32_t& mask, float& swf,
                                             float (&sxf)[2]) {
  WinRows<NR> w;
  win_rows<NR>(A, c, w);
  float2 sx = make_float2(sxf[0], sxf[1]);
#pragma unroll 1
  for (int k = 0; k < Q; ++k) {
    const int cdx = __float2int_rn(A.L.cdf[k][0]), cdy = __float2int_rn(A.L.cdf[k][1]);
    const float cxo = (float)(cdx - bx);
    const float* wk = s_w + k * cap;
    bool hit = false;
    bool more = false;  // a window cell holds a second item: a second pass takes those
#pragma unroll 1
    for (int pass = 0; pass <= (int)more; ++pass)
#pragma unroll
    for (int t = 0; t < NR; ++t) {
      if (t >= w.nr) break;
      const int ry = by + w.jlo + t - cdy;
      const int lo = max(w.a[t] - cdx, -bx), hi = min(w.b[t] - cdx, rw - 1 - bx);
      if (ry < 0 || ry >= rh || lo > hi) continue;
      const int row = ry * rw + bx;
      const int m1 = s_end[row + hi];
      const float cy = w.cy[t];
      float prev = -1.f;  // column of the previous item of the row
      for (int m = s_beg[row + lo]; m < m1; ++m) {
        const Item<float> it = s_it[m];
        const bool first = it.rx != prev;
        prev = it.rx;
        if (first != (pass == 0)) {
          more = true;
          continue;
        }
        const float cx = rn_sub(rn_add(it.rx, cxo), c.x);
        const float2 e = __fadd2_rn(make_float2(it.ox, it.oy), make_float2(cx, cy));
        const float2 e2 = __fmul2_rn(e, e);
        if (rn_add(e2.x, e2.y) <= A.R2) {
          hit = true;
          const float wt = wk[m];
          swf = __fadd_rn(swf, wt);
          sx = __ffma2_rn(make_float2(wt, wt), e, sx);
        }
      }
    }
    if (hit) mask |= 1u << k;
  }
  sxf[0] = sx.x;
  sxf[1] = sx.y;
}

// Row-segment versions of the three bodies (shared-memory mode).  A window row's cells are
// consecutive columns of one region row, whose items were staged contiguously in column order, so
// the row is one item range [s_beg[first], s_end[last]) with no per-cell bookkeeping.  Each row's
// column range is narrowed to the cells that can hold a hit given the row's smallest |e_y|; the
// narrowing only drops cells with no hit, so sums (and their order) are those of the per-cell
// loops.

// SHIFT (FP32 store, whole-cell displacements): the refine windows come from one row table of
// the centroid, shifted per direction (refine_shift above); bit-identical to the per-direction
// windows.
template <int Q, class P, bool SHIFT = false>
__device__ __forceinline__ void thin_refine_rows(const Args<Q, 2, P>& A, const InstK& I, const Tile2& T,
                                                 const TileGeo& G, int rw, int rh, const int* s_beg, const int* s_end,
                                                 const Item<typename P::real>* s_it, const typename P::real* s_w,
                                                 int cap) {
  using real = typename P::real;
  constexpr bool F64 = std::is_same<P, PF64>::value;
  const int lx = threadIdx.x % G.tx, ly = threadIdx.x / G.tx;
  const int Fx = T.x0 + lx, Fy = T.y0 + ly;
  if (ly >= G.ty || Fx >= I.dims[0] || Fy >= I.dims[1]) return;
  const uint32_t F = I.base + (uint32_t)Fx + (uint32_t)I.dims[0] * (uint32_t)Fy;
  const int bx = lx - G.mom.xl, by = ly - G.mom.yl;
  const real bxf = (real)bx;

  // thinning
  uint32_t cnt = 0;
  real sum[2] = {0, 0};
  CSum csum[2];
#pragma unroll 1
  for (int k = 0; k < Q; ++k) {
    const real cdx = A.L.template cd_as<real>(k, 0), cdy = A.L.template cd_as<real>(k, 1);
    int lox, nx, loy, ny;
    thin_sources<real>(cdx, &lox, &nx);
    thin_sources<real>(cdy, &loy, &ny);
#pragma unroll 1
    for (int oy = 0; oy < ny; ++oy) {
      const int soy = loy + oy;
      const real fy0 = (real)(-soy), sy = (real)soy;
      const int row = (by + soy) * rw + bx;
      const int m1 = s_end[row + lox + nx - 1];
      for (int m = s_beg[row + lox]; m < m1; ++m) {
        const Item<real> it = s_it[m];
        const real tx = rn_add(it.ox, cdx), ty = rn_add(it.oy, cdy);
        const real sxf = it.rx - bxf;  // = float(sox), exact
        if (tx >= -sxf && tx < (real)1 - sxf && ty >= fy0 && ty < fy0 + (real)1) {
          ++cnt;
          const real rx = rn_add(sxf, tx), ry = rn_add(sy, ty);
          if constexpr (F64) {
            sum[0] += rx;
            sum[1] += ry;
          } else {
            csum[0].add(rx);
            csum[1].add(ry);
          }
        }
      }
    }
  }
  if (cnt == 0) {
    A.occ[F] = 0u;
    if (A.write_trace) {
      A.tcnt[F] = 0u;
      A.mask[F] = 0u;
    }
    return;
  }
  real cen[2];
  if constexpr (F64) {
    cen[0] = sum[0] / (real)cnt;
    cen[1] = sum[1] / (real)cnt;
  } else {
    cen[0] = csum[0].value() / (real)cnt;
    cen[1] = csum[1].value() / (real)cnt;
  }

  // refine
  uint32_t mask = 0;
  double swd = 0, sxd[2] = {0, 0};
  float swf = 0.f, sxf[2] = {0.f, 0.f};
  if constexpr (SHIFT) {
    static_assert(!F64, "the shifted windows serve the FP32 store");
    refine_shift<Q, kShiftRows>(A, rw, rh, s_beg, s_end, s_it, s_w, cap, bx, by, Pair<float>{cen[0], cen[1]}, mask, swf, sxf);
  } else {
#pragma unroll 1
  for (int k = 0; k < Q; ++k) {
    const real cdx = A.L.template cd_as<real>(k, 0), cdy = A.L.template cd_as<real>(k, 1);
    const real bxr = cen[0] - cdx, byr = cen[1] - cdy;
    const int loy = max((int)floor(byr - A.R - A.tiny), -by), hiy = min((int)floor(byr + A.R + A.tiny), rh - 1 - by);
    const real* wk = s_w + k * cap;
    bool more = false;  // (2D FP32) a window cell holds a second item: a second pass takes those
#pragma unroll 1
    for (int pass = 0; pass <= (int)(kFirstItemsFirst<P, 2> && more); ++pass)
#pragma unroll 1
    for (int sy = loy; sy <= hiy; ++sy) {
      const real cy = canon_c<real>(sy, cdy, cen[1]);
      const real hw = row_halfwidth<real>(A.R2, axis_lower<real>(cy));
      if (hw < (real)0) continue;
      const int lox = max((int)floor(bxr - hw - A.tiny), -bx), hix = min((int)floor(bxr + hw + A.tiny), rw - 1 - bx);
      if (lox > hix) continue;
      const int row = (by + sy) * rw + bx;
      const int m1 = s_end[row + hix];
      [[maybe_unused]] real prev = (real)-1;  // column of the previous item of the row
      for (int m = s_beg[row + lox]; m < m1; ++m) {
        const Item<real> it = s_it[m];
        if constexpr (kFirstItemsFirst<P, 2>) {
          const bool first = it.rx != prev;
          prev = it.rx;
          if (first != (pass == 0)) {
            more = true;
            continue;
          }
        }
        const real cx = rn_sub(rn_add(it.rx - bxf, cdx), cen[0]);
        const real ex = rn_add(it.ox, cx), ey = rn_add(it.oy, cy);
        const real d2 = rn_add(rn_mul(ex, ex), rn_mul(ey, ey));
        if (d2 <= A.R2) {
          mask |= 1u << k;
          const real w = wk[m];
          if constexpr (F64) {
            swd = __dadd_rn(swd, w);
            sxd[0] = __dadd_rn(sxd[0], __dmul_rn(w, ex));
            sxd[1] = __dadd_rn(sxd[1], __dmul_rn(w, ey));
          } else {
            swf += w;
            sxf[0] = fmaf(w, ex, sxf[0]);
            sxf[1] = fmaf(w, ey, sxf[1]);
          }
        }
      }
    }
  }
  }
  const int kappa = __popc(mask);
  real np[2];
#pragma unroll
  for (int a = 0; a < 2; ++a) {
    if (kappa <= A.kappa_hard) np[a] = cen[a];
    else if constexpr (F64) np[a] = __dadd_rn(cen[a], __ddiv_rn(sxd[a], swd));
    else np[a] = cen[a] + sxf[a] / swf;
  }
  bool finite = true;
#pragma unroll
  for (int a = 0; a < 2; ++a) finite &= isfinite(np[a]) && fabs(np[a]) < (real)64;
  if (!finite) {
    atomicOr(A.status, ST_NONFINITE);
    np[0] = cen[0];
    np[1] = cen[1];
  }
  int sh[2];
  real off[2];
#pragma unroll
  for (int a = 0; a < 2; ++a) {
    const real fl = floor(np[a]);
    sh[a] = (int)fl;
    off[a] = np[a] - fl;
    if (off[a] >= (real)1) {
      off[a] = 0;
      sh[a] += 1;
    }
  }
  uint32_t Gc;
  const bool inside = cell_at<2>(I, Fx + sh[0], Fy + sh[1], 0, &Gc);
  if (!inside) atomicOr(A.status, ST_OUT_OF_BOX);
  A.occ[F] = inside ? 1u : 0u;
  A.fkey[F] = inside ? Gc : 0xffffffffu;
  A.foff[F] = off[0];
  A.foff[(int64_t)A.ncells + F] = off[1];
  if (A.write_trace) {
    A.tcnt[F] = cnt;
    A.mask[F] = mask;
    A.cen[F] = cen[0];
    A.cen[(int64_t)A.ncells + F] = cen[1];
  }
}

// The three tiled kernels take a tile list and loop over it with a fixed stride (tile blockIdx.x,
// blockIdx.x + gridDim.x, ...): launched with one block per tile they are ordinary kernels;
// launched with fewer blocks (a few per SM) they are persistent.  Either way each tile is processed
// by one block with the same per-thread loop order, so results do not depend on the launch.
// One tile of thinning + refine, staged through `smem` (the block's dynamic shared memory).
template <int Q, class P, bool SHIFT>
__device__ __forceinline__ void thin_refine_tile(const Args<Q, 2, P>& A, const Tile2& T, const InstK& I,
                                                 const TileGeo& G, unsigned char* smem) {
  using real = typename P::real;
  const int rw = G.tx + G.mom.xh - G.mom.xl, rh = G.ty + G.mom.yh - G.mom.yl;
  const int cap = G.cap_refine;
  unsigned char* p = smem;
  int* s_beg = carve<int>(p, rw * rh);
  int* s_end = carve<int>(p, rw * rh);
  int* s_row = carve<int>(p, rh + 2);
  Item<real>* s_it = carve<Item<real>>(p, cap);
  real* s_w = carve<real>(p, Q * cap);  // exp(f*) of every direction
  stage_region(I, T.x0 + G.mom.xl, T.y0 + G.mom.yl, rw, rh, A.a.start, cap, s_beg, s_end, s_row,
               [&](int gm, int l, int rx) {
                 s_it[l] = Item<real>{A.a.off[gm], A.a.off[A.mcap + gm], (real)rx, (real)0};
#pragma unroll
                 for (int k = 0; k < Q; ++k) s_w[k * cap + l] = exp(fstar_at<Q, 2, P>(A, (uint32_t)gm, k));
               });
  if (s_row[rh + 1]) {
    thin_refine_rows<Q, P, SHIFT>(A, I, T, G, rw, rh, s_beg, s_end, s_it, s_w, cap);
  } else {
    thin_refine_body<Q, P, false>(A, I, T, G, rw, rh, s_beg, s_end, nullptr, nullptr, nullptr, 0);
  }
}

template <int Q, class P, bool SHIFT = false>
__global__ void __launch_bounds__(256) k_thin_refine_t(const __grid_constant__ Args<Q, 2, P> A,
                                                      const Tile2* __restrict__ tiles, const TileGeo G, int ntiles) {
  extern __shared__ __align__(16) unsigned char smem[];
  for (int tb = blockIdx.x; tb < ntiles; tb += gridDim.x) {
    const Tile2 T = tiles[tb];
    const InstK I = A.inst[T.inst];
    thin_refine_tile<Q, P, SHIFT>(A, T, I, G, smem);
    __syncthreads();  // shared memory is restaged for the next tile
  }
}

// List of the items (moments of state a, or control points of state b) in the tile's cells: the
// tile's rows are contiguous item ranges.  Fills entries [c0, c0 + cap_t) of the tile's list with
// the global index, the region coordinates of the item's cell and the item's offsets.  Returns
// the tile's total item count.
template <class real>
__device__ __forceinline__ int tile_items(const InstK& I, const Tile2& T, const TileGeo& G, const Halo& H,
                                          const uint32_t* __restrict__ start, const uint32_t* __restrict__ cellv,
                                          const real* __restrict__ off, int64_t stride, int c0, int cap_t,
                                          int* s_tr, int* s_ij, short* s_bx, short* s_by, Pair<real>* s_p) {
  if (threadIdx.x < 32) {  // the tile's rows, one lane each (ty <= 32), prefix by a warp scan
    const int txe = min(G.tx, I.dims[0] - T.x0);
    int acc = 0;
    for (int r0 = 0; r0 < G.ty; r0 += 32) {
      const int r = r0 + (int)threadIdx.x;
      const int y = T.y0 + r;
      int b = 0, c = 0;
      if (r < G.ty && y < I.dims[1]) {
        const uint32_t g0 = I.base + (uint32_t)T.x0 + (uint32_t)I.dims[0] * (uint32_t)y;
        b = (int)start[g0];
        c = (int)start[g0 + txe] - b;
      }
      const int incl = warp_incl_scan(c);
      if (r < G.ty) {
        s_tr[2 * r] = b;
        s_tr[2 * r + 1] = acc + incl - c;
      }
      acc += __shfl_sync(0xffffffffu, incl, 31);
    }
    if (threadIdx.x == 0) s_tr[2 * G.ty] = acc;
  }
  __syncthreads();
  const int n = s_tr[2 * G.ty];
  const int nc = min(cap_t, n - c0);
  for (int i = threadIdx.x; i < nc; i += blockDim.x) {
    const int li = c0 + i;
    int r = 0;  // the last tile row whose first list entry is <= li (binary search; rows are sorted)
    for (int step = 16; step > 0; step >>= 1)
      if (r + step < G.ty && s_tr[2 * (r + step) + 1] <= li) r += step;
    const int j = s_tr[2 * r] + (li - s_tr[2 * r + 1]);
    const uint32_t lc = cellv[j] - I.base;
    s_ij[i] = j;
    s_bx[i] = (short)((int)(lc % (uint32_t)I.dims[0]) - T.x0 - H.xl);
    s_by[i] = (short)(r - H.yl);
    s_p[i] = Pair<real>{off[j], off[stride + j]};
  }
  __syncthreads();
  return n;
}

// ---- weights: per component, 1 / (sum over control points within R of (R - d)) -----------------

template <int Q, class P, bool LOCAL>
__device__ __forceinline__ void weights_body(const Args<Q, 2, P>& A, const InstK& I, const Tile2& T,
                                             const TileGeo& G, int rw, int rh, const int* s_beg, const int* s_end,
                                             const Pair<typename P::real>* s_cpos, int* s_tr, int* s_ij, short* s_bx,
                                             short* s_by, Pair<typename P::real>* s_mpos) {
  using real = typename P::real;
  constexpr bool F64 = std::is_same<P, PF64>::value;
  const int cap_t = G.cap_tile;
  const real* gpx = A.b.off;
  const real* gpy = A.b.off + A.ccap;
  auto cpos = [&](int c) -> Pair<real> {
    if constexpr (LOCAL) return s_cpos[c];
    else return Pair<real>{gpx[c], gpy[c]};
  };
  for (int c0 = 0;; c0 += cap_t) {
    const int n = tile_items<real>(I, T, G, G.cp, A.a.start, A.a.cell, A.a.off, A.mcap, c0, cap_t, s_tr, s_ij, s_bx,
                                   s_by, s_mpos);
    const int nc = min(cap_t, n - c0);
#pragma unroll 1
    for (int k = 0; k < Q; ++k) {
      const real cdx = A.L.template cd_as<real>(k, 0), cdy = A.L.template cd_as<real>(k, 1);
      for (int i = threadIdx.x; i < nc; i += blockDim.x) {
        const int bx = s_bx[i], by = s_by[i];
        const Pair<real> mo = s_mpos[i];
        const real o[3] = {mo.x, mo.y, 0};
        const real tx = rn_add(o[0], cdx), ty = rn_add(o[1], cdy);
        const int lox = max((int)floor(tx - A.R - A.tiny), -bx), hix = min((int)floor(tx + A.R + A.tiny), rw - 1 - bx);
        const int loy = max((int)floor(ty - A.R - A.tiny), -by), hiy = min((int)floor(ty + A.R + A.tiny), rh - 1 - by);
        double swd = 0;
        CSum sws;
        bool more = false;  // (2D FP32) a window cell holds a second item: a second pass takes those
#pragma unroll 1
        for (int pass = 0; pass <= (int)(kFirstItemsFirst<P, 2> && more); ++pass)
#pragma unroll 1
        for (int gy = loy; gy <= hiy; ++gy) {
          const real basey = rn_add((real)(-gy), cdy);
          const real ely = rn_add(o[1], rn_sub(basey, (real)1)), ehy = rn_add(o[1], basey);
          const real lby = ely > (real)0 ? ely : (ehy < (real)0 ? -ehy : (real)0);
          const real lby2 = rn_mul(lby, lby);
#pragma unroll 1
          for (int gx = lox; gx <= hix; ++gx) {
            const real basex = rn_add((real)(-gx), cdx);
            const real elx = rn_add(o[0], rn_sub(basex, (real)1)), ehx = rn_add(o[0], basex);
            const real lbx = elx > (real)0 ? elx : (ehx < (real)0 ? -ehx : (real)0);
            if (rn_add(rn_mul(lbx, lbx), lby2) > A.R2) continue;
            const int ci = (by + gy) * rw + (bx + gx);
            const int cb = s_beg[ci], ce = s_end[ci];
            more |= ce - cb > 1;
            const int cs = pass ? cb + 1 : cb, c1 = (pass || !kFirstItemsFirst<P, 2>) ? ce : min(ce, cb + 1);
            for (int c = cs; c < c1; ++c) {
              const Pair<real> pc = cpos(c);
              const real cc[3] = {rn_sub(basex, pc.x), rn_sub(basey, pc.y), 0};
              real e[3];
              const real d2 = canon_d2<2, real>(o, cc, e);
              if (d2 <= A.R2) {
                const real d = rn_sqrt(d2);
                if constexpr (F64) swd += A.R - d;
                else sws.add(A.R - d);
              }
            }
          }
        }
        real sw;
        if constexpr (F64) sw = swd;
        else sw = sws.value();
        A.sw[(int64_t)k * A.mcap + s_ij[i]] = sw > (real)0 ? (real)1 / sw : (real)0;
      }
    }
    if (c0 + cap_t >= n) break;
    __syncthreads();
  }
}

template <int Q, class P>
__device__ __forceinline__ void weights_rows(const Args<Q, 2, P>& A, const InstK& I, const Tile2& T,
                                             const TileGeo& G, int rw, int rh, const int* s_beg, const int* s_end,
                                             const Item<typename P::real>* s_cit, int* s_tr, int* s_ij, short* s_bx,
                                             short* s_by, Pair<typename P::real>* s_mpos) {
  using real = typename P::real;
  constexpr bool F64 = std::is_same<P, PF64>::value;
  const int cap_t = G.cap_tile;
  for (int c0 = 0;; c0 += cap_t) {
    const int n = tile_items<real>(I, T, G, G.cp, A.a.start, A.a.cell, A.a.off, A.mcap, c0, cap_t, s_tr, s_ij, s_bx,
                                   s_by, s_mpos);
    const int nc = min(cap_t, n - c0);
    // one work unit per (item, direction), direction-major: finer than one item's nine directions,
    // so the threads of a block finish together; each unit's sum is still one thread's loop
    for (int wu = threadIdx.x; wu < nc * Q; wu += blockDim.x) {
      const int k = wu / nc, i = wu - k * nc;
      const real cdx = A.L.template cd_as<real>(k, 0), cdy = A.L.template cd_as<real>(k, 1);
      {
        const int bx = s_bx[i], by = s_by[i];
        const real bxf = (real)bx;
        const Pair<real> o = s_mpos[i];
        const real tx = rn_add(o.x, cdx), ty = rn_add(o.y, cdy);
        const int loy = max((int)floor(ty - A.R - A.tiny), -by), hiy = min((int)floor(ty + A.R + A.tiny), rh - 1 - by);
        double swd = 0;
        CSum sws;
        bool more = false;  // (2D FP32) a window cell holds a second item: a second pass takes those
#pragma unroll 1
        for (int pass = 0; pass <= (int)(kFirstItemsFirst<P, 2> && more); ++pass)
#pragma unroll 1
        for (int gy = loy; gy <= hiy; ++gy) {
          const real basey = rn_add((real)(-gy), cdy);
          // candidates have e_y in [fl(o.y + fl(basey - 1)), fl(o.y + basey)]
          const real ely = rn_add(o.y, rn_sub(basey, (real)1)), ehy = rn_add(o.y, basey);
          const real lby = ely > (real)0 ? ely : (ehy < (real)0 ? -ehy : (real)0);
          const real hw = row_halfwidth<real>(A.R2, lby);
          if (hw < (real)0) continue;
          const int lox = max((int)floor(tx - hw - A.tiny), -bx), hix = min((int)floor(tx + hw + A.tiny), rw - 1 - bx);
          if (lox > hix) continue;
          const int row = (by + gy) * rw + bx;
          const int c1 = s_end[row + hix];
          [[maybe_unused]] real prev = (real)-1;  // column of the previous item of the row
          for (int c = s_beg[row + lox]; c < c1; ++c) {
            const Item<real> it = s_cit[c];
            if constexpr (kFirstItemsFirst<P, 2>) {
              const bool first = it.rx != prev;
              prev = it.rx;
              if (first != (pass == 0)) {
                more = true;
                continue;
              }
            }
            const real basex = rn_add(bxf - it.rx, cdx);  // float(-dG) + cd
            const real ex = rn_add(o.x, rn_sub(basex, it.ox)), ey = rn_add(o.y, rn_sub(basey, it.oy));
            const real d2 = rn_add(rn_mul(ex, ex), rn_mul(ey, ey));
            if (d2 <= A.R2) {
              const real d = rn_sqrt(d2);
              if constexpr (F64) swd += A.R - d;
              else sws.add(A.R - d);
            }
          }
        }
        real sw;
        if constexpr (F64) sw = swd;
        else sw = sws.value();
        A.sw[(int64_t)k * A.mcap + s_ij[i]] = sw > (real)0 ? (real)1 / sw : (real)0;
      }
    }
    if (c0 + cap_t >= n) break;
    __syncthreads();
  }
}

// Weights with whole-cell displacements (FP32 store, shared-memory mode): one thread per moment,
// all directions.  Component (m, k) sits at the moment's offset o plus cd_k; its control-point
// window rows, relative to the component's cell, depend on o alone: row u (a control point row
// gy = u + cd_k,y) has base_y = float(-u), the same lower bound on |e_y| and the same half-width,
// and the column range [cd_k,x + a_u, cd_k,x + b_u].  One table per moment serves all
// directions; the window margins are far above the rounding of o + cd, and each direction's
// control points are visited in the same order, so sums are bit-identical to weights_rows.
template <int Q, int NR>
__device__ __forceinline__ void weights_rows_shift(const Args<Q, 2, PF32>& A, const InstK& I, const Tile2& T,
                                                   const TileGeo& G, int rw, int rh, const int* s_beg,
                                                   const int* s_end, const Item<float>* s_cit, int* s_tr, int* s_ij,
                                                   short* s_bx, short* s_by, Pair<float>* s_mpos) {
  const int cap_t = G.cap_tile;
  for (int c0 = 0;; c0 += cap_t) {
    const int n = tile_items<float>(I, T, G, G.cp, A.a.start, A.a.cell, A.a.off, A.mcap, c0, cap_t, s_tr, s_ij,
                                    s_bx, s_by, s_mpos);
    const int nc = min(cap_t, n - c0);
    for (int i = threadIdx.x; i < nc; i += blockDim.x) {
      const int bx = s_bx[i], by = s_by[i];
      const Pair<float> o = s_mpos[i];
      // the row table of the moment: rows u in [ulo, ulo + nr)
      const int ulo = (int)floorf(o.y - A.R - A.tiny);
      const int nrow = (int)floorf(o.y + A.R + A.tiny) - ulo + 1;
      if (nrow > NR) atomicOr(A.status, ST_INTERNAL);  // the host sizes NR for R; never expected
      const int nr = min(nrow, NR);
      float by_[NR];
      int a_[NR], b_[NR];
#pragma unroll
      for (int t = 0; t < NR; ++t) {
        const float basey = (float)(-(ulo + t));
        const float ely = rn_add(o.y, rn_sub(basey, 1.f)), ehy = rn_add(o.y, basey);
        const float lby = ely > 0.f ? ely : (ehy < 0.f ? -ehy : 0.f);
        const float hw = row_halfwidth<float>(A.R2, lby);
        by_[t] = basey;
        const bool on = t < nr && hw >= 0.f;
        a_[t] = on ? (int)floorf(o.x - hw - A.tiny) : 1;
        b_[t] = on ? (int)floorf(o.x + hw + A.tiny) : 0;
      }
      const int j = s_ij[i];
#pragma unroll 1
      for (int k = 0; k < Q; ++k) {
        const int cdx = __float2int_rn(A.L.cdf[k][0]), cdy = __float2int_rn(A.L.cdf[k][1]);
        const float bxc = (float)(bx + cdx);  // base_x of a control point in region column rx = bxc - rx
        CSum sws;
        bool more = false;  // a window cell holds a second item: a second pass takes those
#pragma unroll 1
        for (int pass = 0; pass <= (int)more; ++pass)
#pragma unroll
        for (int t = 0; t < NR; ++t) {
          if (t >= nr) break;
          const int ry = by + ulo + t + cdy;
          const int lo = max(a_[t] + cdx, -bx), hi = min(b_[t] + cdx, rw - 1 - bx);
          if (ry < 0 || ry >= rh || lo > hi) continue;
          const int row = ry * rw + bx;
          const int c1 = s_end[row + hi];
          const float basey = by_[t];
          float prev = -1.f;  // column of the previous item of the row
          for (int c = s_beg[row + lo]; c < c1; ++c) {
            const Item<float> it = s_cit[c];
            const bool first = it.rx != prev;
            prev = it.rx;
            if (first != (pass == 0)) {
              more = true;
              continue;
            }
            const float basex = rn_sub(bxc, it.rx);  // float(cd_x - dG_x), exact
            const float2 q = __fadd2_rn(make_float2(basex, basey), make_float2(-it.ox, -it.oy));
            const float2 e = __fadd2_rn(make_float2(o.x, o.y), q);
            const float2 e2 = __fmul2_rn(e, e);
            const float d2 = rn_add(e2.x, e2.y);
            if (d2 <= A.R2) sws.add(A.R - rn_sqrt(d2));
          }
        }
        const float sw = sws.value();
        A.sw[(int64_t)k * A.mcap + j] = sw > 0.f ? 1.f / sw : 0.f;
      }
    }
    if (c0 + cap_t >= n) break;
    __syncthreads();
  }
}

// One tile of the weights kernel, staged through `smem`.
template <int Q, class P, bool SHIFT>
__device__ __forceinline__ void weights_tile(const Args<Q, 2, P>& A, const Tile2& T, const InstK& I,
                                             const TileGeo& G, unsigned char* smem) {
  using real = typename P::real;
  const int rw = G.tx + G.cp.xh - G.cp.xl, rh = G.ty + G.cp.yh - G.cp.yl;
  const int cap = G.cap_weights, cap_t = G.cap_tile;
  unsigned char* p = smem;
  int* s_beg = carve<int>(p, rw * rh);
  int* s_end = carve<int>(p, rw * rh);
  int* s_row = carve<int>(p, rh + 2);
  Item<real>* s_cit = carve<Item<real>>(p, cap);
  int* s_tr = carve<int>(p, 2 * G.ty + 2);
  int* s_ij = carve<int>(p, cap_t);
  short* s_bx = carve<short>(p, cap_t);
  short* s_by = carve<short>(p, cap_t);
  Pair<real>* s_mpos = carve<Pair<real>>(p, cap_t);
  stage_region(I, T.x0 + G.cp.xl, T.y0 + G.cp.yl, rw, rh, A.b.start, cap, s_beg, s_end, s_row,
               [&](int gc, int l, int rx) {
                 s_cit[l] = Item<real>{A.b.off[gc], A.b.off[A.ccap + gc], (real)rx, (real)0};
               });
  if (s_row[rh + 1]) {
    if constexpr (SHIFT) weights_rows_shift<Q, kShiftRows>(A, I, T, G, rw, rh, s_beg, s_end, s_cit, s_tr, s_ij, s_bx,
                                                           s_by, s_mpos);
    else weights_rows<Q, P>(A, I, T, G, rw, rh, s_beg, s_end, s_cit, s_tr, s_ij, s_bx, s_by, s_mpos);
  }
  else weights_body<Q, P, false>(A, I, T, G, rw, rh, s_beg, s_end, nullptr, s_tr, s_ij, s_bx, s_by, s_mpos);
}

template <int Q, class P, bool SHIFT = false>
__global__ void __launch_bounds__(256) k_weights_t(const __grid_constant__ Args<Q, 2, P> A,
                                                  const Tile2* __restrict__ tiles, const TileGeo G, int ntiles) {
  extern __shared__ __align__(16) unsigned char smem[];
  for (int tb = blockIdx.x; tb < ntiles; tb += gridDim.x) {
    const Tile2 T = tiles[tb];
    const InstK I = A.inst[T.inst];
    weights_tile<Q, P, SHIFT>(A, T, I, G, smem);
    __syncthreads();
  }
}

// ---- gather: per control point and direction ------------------------------------------------------

template <int Q, class P, bool LOCAL>
__device__ __forceinline__ void gather_body(const Args<Q, 2, P>& A, const InstK& I, const Tile2& T,
                                            const TileGeo& G, int rw, int rh, const int* s_beg, const int* s_end,
                                            const int* s_gi, const Pair<typename P::real>* s_pos,
                                            const typename P::real* s_rho, Pair<typename P::real>* s_kv, int nstaged,
                                            int* s_tr, int* s_ij, short* s_bx, short* s_by,
                                            Pair<typename P::real>* s_cpos) {
  using real = typename P::real;
  constexpr bool F64 = std::is_same<P, PF64>::value;
  const int cap_t = G.cap_tile;
  const real* gox = A.a.off;
  const real* goy = A.a.off + A.mcap;
  for (int c0 = 0;; c0 += cap_t) {
    const int n = tile_items<real>(I, T, G, G.mom, A.b.start, A.b.cell, A.b.off, A.ccap, c0, cap_t, s_tr, s_ij, s_bx,
                                   s_by, s_cpos);
    const int nc = min(cap_t, n - c0);
#pragma unroll 1
    for (int k = 0; k < Q; ++k) {
      const real* ginv = A.sw + (int64_t)k * A.mcap;
      const real* gfk = F64 ? (const real*)(A.a.f64 + (int64_t)k * A.mcap) : (const real*)(A.a.dev + (int64_t)k * A.mcap);
      if constexpr (LOCAL) {
        __syncthreads();
        for (int l = threadIdx.x; l < nstaged; l += blockDim.x) {
          const int gm = s_gi[l];
          s_kv[l] = Pair<real>{ginv[gm], gfk[gm]};
        }
        __syncthreads();
      }
      const real cdx = A.L.template cd_as<real>(k, 0), cdy = A.L.template cd_as<real>(k, 1);
      for (int i = threadIdx.x; i < nc; i += blockDim.x) {
        const int bx = s_bx[i], by = s_by[i];
        const Pair<real> pp = s_cpos[i];
        const real bxr = pp.x - cdx, byr = pp.y - cdy;
        const int lox = max((int)floor(bxr - A.R - A.tiny), -bx), hix = min((int)floor(bxr + A.R + A.tiny), rw - 1 - bx);
        const int loy = max((int)floor(byr - A.R - A.tiny), -by), hiy = min((int)floor(byr + A.R + A.tiny), rh - 1 - by);
        double acc = 0;
        CSum sa;
        float sb = 0.f;  // deviation part: small, plain FMA accumulation suffices
        bool more = false;  // (2D FP32) a window cell holds a second item: a second pass takes those
#pragma unroll 1
        for (int pass = 0; pass <= (int)(kFirstItemsFirst<P, 2> && more); ++pass)
#pragma unroll 1
        for (int sy = loy; sy <= hiy; ++sy) {
          const real cy = canon_c<real>(sy, cdy, pp.y);
#pragma unroll 1
          for (int sx = lox; sx <= hix; ++sx) {
            const real c[3] = {canon_c<real>(sx, cdx, pp.x), cy, 0};
            if (cell_d2_lower<2, real>(c) > A.R2) continue;
            const int ci = (by + sy) * rw + (bx + sx);
            const int mb = s_beg[ci], me = s_end[ci];
            more |= me - mb > 1;
            const int m0 = pass ? mb + 1 : mb, m1 = (pass || !kFirstItemsFirst<P, 2>) ? me : min(me, mb + 1);
            for (int m = m0; m < m1; ++m) {
              real o[3];
              if constexpr (LOCAL) {
                const Pair<real> o2 = s_pos[m];
                o[0] = o2.x;
                o[1] = o2.y;
              } else {
                o[0] = gox[m];
                o[1] = goy[m];
              }
              o[2] = 0;
              real e[3];
              const real d2 = canon_d2<2, real>(o, c, e);
              if (d2 <= A.R2) {
                Pair<real> kv;
                if constexpr (LOCAL) kv = s_kv[m];
                else kv = Pair<real>{ginv[m], gfk[m]};
                if (kv.x > (real)0) {
                  const real wgt = (A.R - rn_sqrt(d2)) * kv.x;
                  if constexpr (F64) {
                    acc += wgt * kv.y;
                  } else {
                    real rho;
                    if constexpr (LOCAL) rho = s_rho[m];
                    else rho = A.a.rho[m];
                    sa.add_prod(wgt, rho);
                    sb = __fmaf_rn(wgt, kv.y, sb);
                  }
                }
              }
            }
          }
        }
        const int j = s_ij[i];
        bool empty;
        if constexpr (F64) {
          A.cpf64[(int64_t)k * A.ccap + j] = acc;
          empty = acc < (double)A.eps;
        } else {
          DF Ad = df_norm(sa.hi, sa.lo);
          DF Bd = DF{sb, 0.f};
          DF Fv = df_add(df_mul(DF{A.L.wf[k], A.L.wlo[k]}, Ad), Bd);
          A.cpfhi[(int64_t)k * A.ccap + j] = Fv.hi;
          A.cpflo[(int64_t)k * A.ccap + j] = Fv.lo;
          empty = Fv.hi < A.eps;
        }
        if (empty) atomicOr(A.emask + j, 1u << k);
      }
    }
    if (c0 + cap_t >= n) break;
    __syncthreads();
  }
}

template <int Q, class P>
__device__ __forceinline__ void gather_rows(const Args<Q, 2, P>& A, const InstK& I, const Tile2& T,
                                            const TileGeo& G, int rw, int rh, const int* s_beg, const int* s_end,
                                            const int* s_gi, const Item<typename P::real>* s_it,
                                            const typename P::real* s_rho, Pair<typename P::real>* s_kv, int nstaged,
                                            int* s_tr, int* s_ij, short* s_bx, short* s_by,
                                            Pair<typename P::real>* s_cpos) {
  using real = typename P::real;
  constexpr bool F64 = std::is_same<P, PF64>::value;
  const int cap_t = G.cap_tile;
  for (int c0 = 0;; c0 += cap_t) {
    const int n = tile_items<real>(I, T, G, G.mom, A.b.start, A.b.cell, A.b.off, A.ccap, c0, cap_t, s_tr, s_ij, s_bx,
                                   s_by, s_cpos);
    const int nc = min(cap_t, n - c0);
#pragma unroll 1
    for (int k = 0; k < Q; ++k) {
      const real* ginv = A.sw + (int64_t)k * A.mcap;
      const real* gfk = F64 ? (const real*)(A.a.f64 + (int64_t)k * A.mcap) : (const real*)(A.a.dev + (int64_t)k * A.mcap);
      // stage (1/sw, f_k) of every region item for this direction
      __syncthreads();
      for (int l = threadIdx.x; l < nstaged; l += blockDim.x) {
        const int gm = s_gi[l];
        s_kv[l] = Pair<real>{ginv[gm], gfk[gm]};
      }
      __syncthreads();
      const real cdx = A.L.template cd_as<real>(k, 0), cdy = A.L.template cd_as<real>(k, 1);
      for (int i = threadIdx.x; i < nc; i += blockDim.x) {
        const int bx = s_bx[i], by = s_by[i];
        const real bxf = (real)bx;
        const Pair<real> pp = s_cpos[i];
        const real bxr = pp.x - cdx, byr = pp.y - cdy;
        const int loy = max((int)floor(byr - A.R - A.tiny), -by), hiy = min((int)floor(byr + A.R + A.tiny), rh - 1 - by);
        double acc = 0;
        CSum sa;
        float sb = 0.f;  // deviation part: small, plain FMA accumulation suffices
        bool more = false;  // (2D FP32) a window cell holds a second item: a second pass takes those
#pragma unroll 1
        for (int pass = 0; pass <= (int)(kFirstItemsFirst<P, 2> && more); ++pass)
#pragma unroll 1
        for (int sy = loy; sy <= hiy; ++sy) {
          const real cy = canon_c<real>(sy, cdy, pp.y);
          const real hw = row_halfwidth<real>(A.R2, axis_lower<real>(cy));
          if (hw < (real)0) continue;
          const int lox = max((int)floor(bxr - hw - A.tiny), -bx), hix = min((int)floor(bxr + hw + A.tiny), rw - 1 - bx);
          if (lox > hix) continue;
          const int row = (by + sy) * rw + bx;
          const int m1 = s_end[row + hix];
          [[maybe_unused]] real prev = (real)-1;  // column of the previous item of the row
          for (int m = s_beg[row + lox]; m < m1; ++m) {
            const Item<real> it = s_it[m];
            if constexpr (kFirstItemsFirst<P, 2>) {
              const bool first = it.rx != prev;
              prev = it.rx;
              if (first != (pass == 0)) {
                more = true;
                continue;
              }
            }
            const real cx = rn_sub(rn_add(it.rx - bxf, cdx), pp.x);
            const real ex = rn_add(it.ox, cx), ey = rn_add(it.oy, cy);
            const real d2 = rn_add(rn_mul(ex, ex), rn_mul(ey, ey));
            if (d2 <= A.R2) {
              const Pair<real> kv = s_kv[m];
              if (kv.x > (real)0) {
                const real wgt = (A.R - rn_sqrt(d2)) * kv.x;
                if constexpr (F64) {
                  acc += wgt * kv.y;
                } else {
                  sa.add_prod(wgt, s_rho[m]);
                  sb = __fmaf_rn(wgt, kv.y, sb);
                }
              }
            }
          }
        }
        const int j = s_ij[i];
        bool empty;
        if constexpr (F64) {
          A.cpf64[(int64_t)k * A.ccap + j] = acc;
          empty = acc < (double)A.eps;
        } else {
          DF Ad = df_norm(sa.hi, sa.lo);
          DF Bd = DF{sb, 0.f};
          DF Fv = df_add(df_mul(DF{A.L.wf[k], A.L.wlo[k]}, Ad), Bd);
          A.cpfhi[(int64_t)k * A.ccap + j] = Fv.hi;
          A.cpflo[(int64_t)k * A.ccap + j] = Fv.lo;
          empty = Fv.hi < A.eps;
        }
        if (empty) atomicOr(A.emask + j, 1u << k);
      }
    }
    if (c0 + cap_t >= n) break;
    __syncthreads();
  }
}

// A staged moment for the whole-cell gather: offsets, region column (exact small integer), rho,
// then (1/sw, f*_k) of the kGatherGroup directions staged together, so a hit reads its operands
// at a fixed offset from the candidate it just tested.
constexpr int kGatherGroup = 3;
struct alignas(16) GRec {
  float ox, oy, rx, rho;
  float kv[2 * kGatherGroup];  // (1/sw, f*) of each staged direction
  float pad[(4 - (2 * kGatherGroup) % 4) % 4];
};

// One control point, one direction (FP32 store): the gather_rows sum over the shifted rows.
template <int Q, int NR>
__device__ __forceinline__ void gather_cp_shift(const Args<Q, 2, PF32>& A, int k, int slot, int cdx, int cdy, int rw,
                                                int rh, const int* s_beg, const int* s_end, const GRec* s_rec,
                                                int bx, int by, Pair<float> pp, const WinRows<NR>& w, int j) {
  const float cxo = (float)(cdx - bx);  // region column + cxo = float(dS_x + cd_x), exact
  CSum sa;
  float sb = 0.f;  // deviation part: plain FMA accumulation, as in gather_rows
  bool more = false;  // a window cell holds a second item: a second pass takes those
#pragma unroll 1
  for (int pass = 0; pass <= (int)more; ++pass)
#pragma unroll
  for (int t = 0; t < NR; ++t) {
    if (t >= w.nr) break;
    const int ry = by + w.jlo + t - cdy;
    const int lo = max(w.a[t] - cdx, -bx), hi = min(w.b[t] - cdx, rw - 1 - bx);
    if (ry < 0 || ry >= rh || lo > hi) continue;
    const int row = ry * rw + bx;
    const GRec* it = s_rec + s_beg[row + lo];
    const GRec* const end = s_rec + s_end[row + hi];
    const float cy = w.cy[t];
    float prev = -1.f;  // column of the previous item of the row
    for (; it < end; ++it) {
      const float4 a = *reinterpret_cast<const float4*>(it);
      const bool first = a.z != prev;
      prev = a.z;
      if (first != (pass == 0)) {
        more = true;
        continue;
      }
      const float cx = rn_sub(rn_add(a.z, cxo), pp.x);
      const float2 e = __fadd2_rn(make_float2(a.x, a.y), make_float2(cx, cy));
      const float2 e2 = __fmul2_rn(e, e);
      const float d2 = rn_add(e2.x, e2.y);
      if (d2 <= A.R2) {
        // A dropped component has 1/sw = 0: its weight is +0 and every sum below is unchanged
        // (the sums are >= +0 and f is finite), so it needs no test of its own.
        const float2 kv = *reinterpret_cast<const float2*>(&it->kv[2 * slot]);
        const float wgt = (A.R - rn_sqrt(d2)) * kv.x;
        // CSum::add_prod(wgt, rho) and the deviation FMA, the two FMAs as one paired op
        const float p = __fmul_rn(wgt, a.w);
        const float2 r = __ffma2_rn(make_float2(wgt, wgt), make_float2(a.w, kv.y), make_float2(-p, sb));
        sa.add(p);
        sa.lo = __fadd_rn(sa.lo, r.x);
        sb = r.y;
      }
    }
  }
  const DF Ad = df_norm(sa.hi, sa.lo);
  const DF Fv = df_add(df_mul(DF{A.L.wf[k], A.L.wlo[k]}, Ad), DF{sb, 0.f});
  A.cpfhi[(int64_t)k * A.ccap + j] = Fv.hi;
  A.cpflo[(int64_t)k * A.ccap + j] = Fv.lo;
  if (Fv.hi < A.eps) atomicOr(A.emask + j, 1u << k);
}

// Gather with whole-cell displacements (FP32 store, shared-memory mode).  Each thread keeps the
// row table of its first control point in registers across the nine directions; a tile with more
// control points than threads builds the extra points' tables per direction.
template <int Q, int NR>
__device__ __forceinline__ void gather_rows_shift(const Args<Q, 2, PF32>& A, const InstK& I, const Tile2& T,
                                                  const TileGeo& G, int rw, int rh, const int* s_beg,
                                                  const int* s_end, const int* s_gi, GRec* s_rec, int nstaged,
                                                  int* s_tr, int* s_ij, short* s_bx, short* s_by,
                                                  Pair<float>* s_cpos) {
  const int cap_t = G.cap_tile;
  for (int c0 = 0;; c0 += cap_t) {
    const int n = tile_items<float>(I, T, G, G.mom, A.b.start, A.b.cell, A.b.off, A.ccap, c0, cap_t, s_tr, s_ij,
                                    s_bx, s_by, s_cpos);
    const int nc = min(cap_t, n - c0);
    const int i0 = threadIdx.x;
    const bool has0 = i0 < nc;
    WinRows<NR> w0;
    int bx0 = 0, by0 = 0, j0 = 0;
    Pair<float> p0{0.f, 0.f};
    if (has0) {
      bx0 = s_bx[i0];
      by0 = s_by[i0];
      j0 = s_ij[i0];
      p0 = s_cpos[i0];
      win_rows<NR>(A, p0, w0);
    }
    // directions in groups of kGatherGroup: one staging pass (two barriers) per group
#pragma unroll 1
    for (int k0 = 0; k0 < Q; k0 += kGatherGroup) {
      const int ng = min(kGatherGroup, Q - k0);
      __syncthreads();
      for (int l = threadIdx.x; l < nstaged; l += blockDim.x) {
        const int gm = s_gi[l];
        for (int q = 0; q < ng; ++q)
          *reinterpret_cast<float2*>(&s_rec[l].kv[2 * q]) =
              make_float2(A.sw[(int64_t)(k0 + q) * A.mcap + gm], A.a.dev[(int64_t)(k0 + q) * A.mcap + gm]);
      }
      __syncthreads();
#pragma unroll 1
      for (int q = 0; q < ng; ++q) {
        const int k = k0 + q;
        const int cdx = __float2int_rn(A.L.cdf[k][0]), cdy = __float2int_rn(A.L.cdf[k][1]);
        if (has0) gather_cp_shift<Q, NR>(A, k, q, cdx, cdy, rw, rh, s_beg, s_end, s_rec, bx0, by0, p0, w0, j0);
        for (int i = i0 + blockDim.x; i < nc; i += blockDim.x) {
          WinRows<NR> w;
          const Pair<float> pp = s_cpos[i];
          win_rows<NR>(A, pp, w);
          gather_cp_shift<Q, NR>(A, k, q, cdx, cdy, rw, rh, s_beg, s_end, s_rec, s_bx[i], s_by[i], pp, w, s_ij[i]);
        }
      }
    }
    if (c0 + cap_t >= n) break;
    __syncthreads();
  }
}

// One tile of the whole-cell gather, staged through `smem`.
template <int Q>
__device__ __forceinline__ void gather_ts_tile(const Args<Q, 2, PF32>& A, const Tile2& T, const InstK& I,
                                               const TileGeo& G, unsigned char* smem) {
  const int rw = G.tx + G.mom.xh - G.mom.xl, rh = G.ty + G.mom.yh - G.mom.yl;
  const int cap = G.cap_gather, cap_t = G.cap_tile;
  unsigned char* p = smem;
  int* s_beg = carve<int>(p, rw * rh);
  int* s_end = carve<int>(p, rw * rh);
  int* s_row = carve<int>(p, rh + 2);
  int* s_gi = carve<int>(p, cap);
  GRec* s_rec = carve<GRec>(p, cap);
  int* s_tr = carve<int>(p, 2 * G.ty + 2);
  int* s_ij = carve<int>(p, cap_t);
  short* s_bx = carve<short>(p, cap_t);
  short* s_by = carve<short>(p, cap_t);
  Pair<float>* s_cpos = carve<Pair<float>>(p, cap_t);
  stage_region(I, T.x0 + G.mom.xl, T.y0 + G.mom.yl, rw, rh, A.a.start, cap, s_beg, s_end, s_row,
               [&](int gm, int l, int rx) {
                 s_gi[l] = gm;
                 *reinterpret_cast<float4*>(&s_rec[l]) =
                     make_float4(A.a.off[gm], A.a.off[A.mcap + gm], (float)rx, A.a.rho[gm]);
               });
  if (s_row[rh + 1])
    gather_rows_shift<Q, kShiftRows>(A, I, T, G, rw, rh, s_beg, s_end, s_gi, s_rec, s_row[rh], s_tr, s_ij, s_bx,
                                     s_by, s_cpos);
  else
    gather_body<Q, PF32, false>(A, I, T, G, rw, rh, s_beg, s_end, s_gi, nullptr, nullptr, nullptr, 0, s_tr, s_ij,
                                s_bx, s_by, s_cpos);
}

template <int Q>
__global__ void __launch_bounds__(256) k_gather_ts(const __grid_constant__ Args<Q, 2, PF32> A,
                                                  const Tile2* __restrict__ tiles, const TileGeo G, int ntiles) {
  extern __shared__ __align__(16) unsigned char smem[];
  for (int tb = blockIdx.x; tb < ntiles; tb += gridDim.x) {
    const Tile2 T = tiles[tb];
    const InstK I = A.inst[T.inst];
    gather_ts_tile<Q>(A, T, I, G, smem);
    __syncthreads();
  }
}

template <int Q, class P>
__global__ void __launch_bounds__(256) k_gather_t(const __grid_constant__ Args<Q, 2, P> A,
                                                 const Tile2* __restrict__ tiles, const TileGeo G, int ntiles) {
  using real = typename P::real;
  constexpr bool F64 = std::is_same<P, PF64>::value;
  extern __shared__ __align__(16) unsigned char smem[];
  for (int tb = blockIdx.x; tb < ntiles; tb += gridDim.x) {
  const Tile2 T = tiles[tb];
  const InstK I = A.inst[T.inst];
  const int rw = G.tx + G.mom.xh - G.mom.xl, rh = G.ty + G.mom.yh - G.mom.yl;
  const int cap = G.cap_gather, cap_t = G.cap_tile;
  unsigned char* p = smem;
  int* s_beg = carve<int>(p, rw * rh);
  int* s_end = carve<int>(p, rw * rh);
  int* s_row = carve<int>(p, rh + 2);
  int* s_gi = carve<int>(p, cap);
  Item<real>* s_it = carve<Item<real>>(p, cap);
  real* s_rho = carve<real>(p, cap);
  Pair<real>* s_kv = carve<Pair<real>>(p, cap);
  int* s_tr = carve<int>(p, 2 * G.ty + 2);
  int* s_ij = carve<int>(p, cap_t);
  short* s_bx = carve<short>(p, cap_t);
  short* s_by = carve<short>(p, cap_t);
  Pair<real>* s_cpos = carve<Pair<real>>(p, cap_t);
  stage_region(I, T.x0 + G.mom.xl, T.y0 + G.mom.yl, rw, rh, A.a.start, cap, s_beg, s_end, s_row,
               [&](int gm, int l, int rx) {
                 s_gi[l] = gm;
                 s_it[l] = Item<real>{A.a.off[gm], A.a.off[A.mcap + gm], (real)rx, (real)0};
                 if constexpr (!F64) s_rho[l] = A.a.rho[gm];
               });
  if (s_row[rh + 1])
    gather_rows<Q, P>(A, I, T, G, rw, rh, s_beg, s_end, s_gi, s_it, s_rho, s_kv, s_row[rh], s_tr, s_ij, s_bx, s_by,
                      s_cpos);
  else
    gather_body<Q, P, false>(A, I, T, G, rw, rh, s_beg, s_end, s_gi, nullptr, s_rho, s_kv, 0, s_tr, s_ij, s_bx, s_by,
                             s_cpos);
  __syncthreads();
  }
}

}  // namespace dbm
