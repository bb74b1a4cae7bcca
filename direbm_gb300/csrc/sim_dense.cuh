// Dense-stencil variants of the three whole-cell window kernels (2D, FP32 store).
//
// With whole-cell displacements (every cd_k an integer, D2Q9 with dx = cell) and R < 2 cells, the
// thinning cell holds at most one control point, so in the ensemble and inverse-problem workloads
// almost every cell holds exactly one moment: all of them at first, and after some steps all but
// ~1 % (a refine move occasionally crosses a cell face, leaving a cell with two items and another
// empty).  A tile's region is therefore staged as a dense grid -- one record per region cell, an
// empty cell holding an offset far outside every window, a cell with two items naming the slot of
// its second item in a small per-tile overflow list -- and each reference point's window for
// direction k becomes a fixed 4 x 4 block of cells: the component-cell offsets j with
// e = off + (j - p) in reach of R are floor(p - R - tiny) .. floor(p + R + tiny), four values per
// axis at R = 1.5 except within tiny of p = 1/2 (five).  A point whose range is not four wide takes
// a loop over its exact range, so no access leaves the staged region (its halo covers the exact
// ranges for any R < 2).  Every thread runs the same unrolled stencil, without the per-row
// bookkeeping and the uneven loop trips of the row-segment loops, and the canonical
// c = rn(float(j) - p) of the stencil's four columns and rows is computed once per point.
//
// Results are bit-identical to the row-segment kernels: each sum visits the same hits in the same
// order with the same operations.  The first items of the window's cells come first (window rows
// ascending, then columns ascending), then the second items in the same cell order.  The unrolled
// stencil reads only the records; a record naming a second item sets a bit of a per-thread
// window mask, and a short loop over that mask visits the second items afterwards.  A warp then
// pays for a second item only in the loop, not at every stencil position where some lane's cell
// has one.  A tile whose region holds a cell with three or more items, or more two-item
// cells than the overflow list takes, is handed to the row-segment code (a second, normally empty,
// launch over the deferred tiles).
#pragma once

#include "sim_tiled.cuh"

namespace dbm {

// Offset stored for an empty cell: every displacement from it is ~1e4 cells, far outside R.
constexpr float kEmptyOff = 1.0e4f;
// Second items of a tile's region (cells holding two items): at most this many per tile.  A cell
// with three or more items, or more two-item cells than this, sends the tile to the fallback.
constexpr int kOvf = 32;

// Dynamic shared memory of the dense layouts (region of `cells` cells): per cell a float4 record
// {offset x, offset y, overflow slot of the cell's second item (-1: none), rho or 0} plus per
// direction data, the same for the kOvf overflow items, the region coordinates of each overflow
// item's cell, and the overflow counter.
__host__ __device__ inline size_t dense_off(size_t n) { return (n + 15) & ~(size_t)15; }
// Byte offsets of the cell records, their data, the overflow records and their data; returns the
// total including the overflow cells' coordinates and the counter.
__host__ __device__ inline size_t ds_layout(int cells, size_t per_cell, size_t* offs) {
  const int n[2] = {cells, kOvf};
  size_t o = 0;
  for (int b = 0; b < 2; ++b) {
    offs[2 * b] = o;
    o += dense_off((size_t)n[b] * 16);
    offs[2 * b + 1] = o;
    o += dense_off((size_t)n[b] * per_cell);
  }
  return o + dense_off((size_t)kOvf * 4) + 16;  // + the overflow cells' coordinates, the counter
}
__host__ __device__ inline size_t ds_bytes(int cells, size_t per_cell) {
  size_t offs[4];
  return ds_layout(cells, per_cell, offs);
}
// per-direction bytes per item: thin + refine exp(f*) (4 Q), weights none, gather (1/sw, f*) (8 Q)
__host__ __device__ inline size_t ds_bytes_refine(int Q, int cells) { return ds_bytes(cells, (size_t)4 * Q); }
__host__ __device__ inline size_t ds_bytes_weights(int cells) { return ds_bytes(cells, 0); }
__host__ __device__ inline size_t ds_bytes_gather(int Q, int cells) { return ds_bytes(cells, (size_t)8 * Q); }

struct DenseSmem {
  float4* rec;          // [cells]
  unsigned char* dat;   // per-direction data of the cells' first items
  float4* orec;         // [kOvf]
  unsigned char* odat;  // per-direction data of the overflow items
  int* ocell;           // [kOvf] region row << 16 | region column of each overflow item's cell
  int* novf;            // overflow counter
};
__device__ __forceinline__ DenseSmem dense_smem(unsigned char* smem, int cells, size_t per_cell) {
  size_t offs[4];
  const size_t total = ds_layout(cells, per_cell, offs);
  return DenseSmem{reinterpret_cast<float4*>(smem + offs[0]), smem + offs[1], reinterpret_cast<float4*>(smem + offs[2]),
                   smem + offs[3], reinterpret_cast<int*>(smem + total - 16 - dense_off((size_t)kOvf * 4)),
                   reinterpret_cast<int*>(smem + total - 16)};
}

// Window positions (b * ncol + a, a < ncol columns, b < nrow rows from region cell (row0, col0))
// whose cell holds a second item, from the tile's overflow list: no per-position test in the
// stencil, and nothing to do in a tile without two-item cells.
__device__ __forceinline__ uint32_t second_item_mask(const DenseSmem& S, int no, int row0, int col0, int nrow,
                                                     int ncol) {
  uint32_t ov = 0;
#pragma unroll 1
  for (int q = 0; q < no; ++q) {
    const int rc = S.ocell[q];
    const int b = (rc >> 16) - row0, a = (rc & 0xffff) - col0;
    if ((unsigned)b < (unsigned)nrow && (unsigned)a < (unsigned)ncol) ov |= 1u << (b * ncol + a);
  }
  return ov;
}

// Item range of global cell g: at most two items, else *many is set.
__device__ __forceinline__ void cell_items(const uint32_t* __restrict__ start, uint32_t g, int* b, int* e, int* many) {
  const uint32_t b0 = start[g], e0 = start[g + 1];
  if (e0 - b0 > 2u) {
    *many = 1;
    *b = *e = (int)b0;
  } else {
    *b = (int)b0;
    *e = (int)e0;
  }
}

// Dense staging of region cells [xr0, xr0 + rw) x [yr0, yr0 + rh) of a state's sorted ranges
// `start`: put(record, per-direction data, stride, slot, item, nxt) fills the record of one item
// (its per-direction data goes to data[k * stride + slot]); the record of an empty cell gets the
// empty offset.  A cell's second item goes to the next overflow slot.  Returns false, the same in
// every thread, when the tile must be deferred (`many` from the caller, a cell with three or more
// items, or a full overflow list).
template <class Put>
__device__ __forceinline__ bool stage_dense(const InstK& I, int xr0, int yr0, int rw, int rh,
                                            const uint32_t* __restrict__ start, const DenseSmem& S, int many,
                                            Put&& put) {
  const int cells = rw * rh;
  if (threadIdx.x == 0) *S.novf = 0;
  __syncthreads();
  for (int ci = threadIdx.x; ci < cells; ci += blockDim.x) {
    const int ry = ci / rw, rx = ci - ry * rw;
    uint32_t g;
    int b = 0, e = 0;
    if (region_cell(I, xr0 + rx, yr0 + ry, &g)) cell_items(start, g, &b, &e, &many);
    float nxt = -1.f;
    if (e - b == 2) {
      const int q = atomicAdd(S.novf, 1);
      if (q < kOvf) {
        put(S.orec + q, S.odat, kOvf, q, b + 1, -1.f);
        S.ocell[q] = (ry << 16) | rx;
        nxt = (float)q;
      } else {
        many = 1;
      }
    }
    if (e > b) put(S.rec + ci, S.dat, cells, ci, b, nxt);
    else S.rec[ci] = make_float4(kEmptyOff, kEmptyOff, -1.f, 0.f);
  }
  return !__syncthreads_or(many);
}

// Second items of the tile's own two-item cells (moments in the weights kernel, control points in
// the gather): their (item, direction) units are spread over the block after every thread's first
// item, so a two-item cell adds one direction's work to nine threads instead of nine directions to
// one thread (whose warp, and with it the block, would wait for it).  Each unit's sum is its own:
// no result changes.
struct SecondMoments {
  int n;
  int item[256];
  short bx[256], by[256];
};

// Stencil origin and width along one axis for reference offset p: j in [lo, lo + n).
__device__ __forceinline__ void stencil_axis(float p, float R, float tiny, int* lo, int* n) {
  *lo = (int)floorf(p - R - tiny);
  *n = (int)floorf(p + R + tiny) - *lo + 1;
}

// ---- thinning + refine --------------------------------------------------------------------------
// Per-direction data: exp(f*_k) of each item, direction-major ([k][cells] and [k][kOvf]).

template <int Q>
__device__ __forceinline__ bool thin_refine_ds_tile(const Args<Q, 2, PF32>& A, const Tile2& T, const InstK& I,
                                                    const TileGeo& G, unsigned char* smem) {
  const int rw = G.tx + G.mom.xh - G.mom.xl, rh = G.ty + G.mom.yh - G.mom.yl;
  const int cells = rw * rh;
  const DenseSmem S = dense_smem(smem, cells, (size_t)4 * Q);
  float* s_w = reinterpret_cast<float*>(S.dat);
  float* s_ow = reinterpret_cast<float*>(S.odat);
  const bool dense = stage_dense(I, T.x0 + G.mom.xl, T.y0 + G.mom.yl, rw, rh, A.a.start, S, 0,
                                 [&](float4* r, unsigned char* dat, int stride, int slot, int m, float nxt) {
                                   *r = make_float4(A.a.off[m], A.a.off[A.mcap + m], nxt, 0.f);
                                   float* w = reinterpret_cast<float*>(dat);
#pragma unroll
                                   for (int k = 0; k < Q; ++k)
                                     w[k * stride + slot] = exp(fstar_at<Q, 2, PF32>(A, (uint32_t)m, k));
                                 });
  if (!dense) return false;
  const int no = *S.novf;  // second items in the overflow list (at most kOvf in a dense tile)

  const int lx = threadIdx.x % G.tx, ly = threadIdx.x / G.tx;
  const int Fx = T.x0 + lx, Fy = T.y0 + ly;
  if (ly >= G.ty || Fx >= I.dims[0] || Fy >= I.dims[1]) return true;
  const uint32_t F = I.base + (uint32_t)Fx + (uint32_t)I.dims[0] * (uint32_t)Fy;
  const int bx = lx - G.mom.xl, by = ly - G.mom.yl;  // region coordinates of F

  // thinning: component (m, k) lands in F iff floor(off + cd) == -so on both axes
  uint32_t cnt = 0;
  CSum csum[2];
#pragma unroll 1
  for (int k = 0; k < Q; ++k) {
    const float cdx = A.L.cdf[k][0], cdy = A.L.cdf[k][1];
    int lox, nx, loy, ny;
    thin_sources<float>(cdx, &lox, &nx);
    thin_sources<float>(cdy, &loy, &ny);
#pragma unroll 1
    for (int oy = 0; oy < ny; ++oy) {
      const int soy = loy + oy;
      const float fy0 = (float)(-soy), sy = (float)soy;
#pragma unroll 1
      for (int ox = 0; ox < nx; ++ox) {
        const int sox = lox + ox;
        const float sxf = (float)sox;
        auto land = [&](float4 o) {
          const float tx = rn_add(o.x, cdx), ty = rn_add(o.y, cdy);
          if (tx >= -sxf && tx < 1.f - sxf && ty >= fy0 && ty < fy0 + 1.f) {
            ++cnt;
            csum[0].add(rn_add(sxf, tx));
            csum[1].add(rn_add(sy, ty));
          }
        };
        const float4 o = S.rec[(by + soy) * rw + (bx + sox)];
        land(o);
        if (o.z >= 0.f) land(S.orec[(int)o.z]);
      }
    }
  }
  if (cnt == 0) {
    A.occ[F] = 0u;
    if (A.write_trace) {
      A.tcnt[F] = 0u;
      A.mask[F] = 0u;
    }
    return true;
  }
  const float cen[2] = {csum[0].value() / (float)cnt, csum[1].value() / (float)cnt};

  // refine: the centroid's 4 x 4 stencil, shifted by -cd_k per direction
  int jlx, nxs, jly, nys;
  stencil_axis(cen[0], A.R, A.tiny, &jlx, &nxs);
  stencil_axis(cen[1], A.R, A.tiny, &jly, &nys);
  const bool wide = nxs != 4 || nys != 4;  // exact-range loops otherwise
  float cx[4], cy[4];
#pragma unroll
  for (int a = 0; a < 4; ++a) {
    cx[a] = rn_sub((float)(jlx + a), cen[0]);
    cy[a] = rn_sub((float)(jly + a), cen[1]);
  }
  uint32_t mask = 0;
  float swf = 0.f;
  float2 sx = make_float2(0.f, 0.f);
#pragma unroll 1
  for (int k = 0; k < Q; ++k) {
    const int cdx = __float2int_rn(A.L.cdf[k][0]), cdy = __float2int_rn(A.L.cdf[k][1]);
    const int c0 = (by + jly - cdy) * rw + (bx + jlx - cdx);
    const float* wk = s_w + k * cells;
    const float* owk = s_ow + k * kOvf;
    bool hit = false;
    auto one = [&](float4 o, const float* wp, float ex0, float ey0) {
      const float2 e = __fadd2_rn(make_float2(o.x, o.y), make_float2(ex0, ey0));
      const float2 e2 = __fmul2_rn(e, e);
      if (rn_add(e2.x, e2.y) <= A.R2) {
        hit = true;
        const float wt = *wp;
        swf = __fadd_rn(swf, wt);
        sx = __ffma2_rn(make_float2(wt, wt), e, sx);
      }
    };
    // first items of the window's cells
    auto visit = [&](int ci, float ex0, float ey0) { one(S.rec[ci], wk + ci, ex0, ey0); };
    const int ncol = wide ? nxs : 4;
    if (!wide) {
#pragma unroll
      for (int b = 0; b < 4; ++b)
#pragma unroll
        for (int a = 0; a < 4; ++a) visit(c0 + b * rw + a, cx[a], cy[b]);
    } else {
#pragma unroll 1
      for (int b = 0; b < nys; ++b) {
        const float cyb = rn_sub((float)(jly + b), cen[1]);
#pragma unroll 1
        for (int a = 0; a < nxs; ++a) visit(c0 + b * rw + a, rn_sub((float)(jlx + a), cen[0]), cyb);
      }
    }
    // then the second items, in window order
    uint32_t ov = no ? second_item_mask(S, no, by + jly - cdy, bx + jlx - cdx, wide ? nys : 4, ncol) : 0u;
#pragma unroll 1
    while (ov) {
      const int pos = __ffs(ov) - 1;
      ov &= ov - 1;
      const int b = wide ? pos / ncol : pos >> 2, a = pos - b * ncol;
      const int ci = c0 + b * rw + a;
      const int q = (int)S.rec[ci].z;
      one(S.orec[q], owk + q, rn_sub((float)(jlx + a), cen[0]), rn_sub((float)(jly + b), cen[1]));
    }
    if (hit) mask |= 1u << k;
  }
  const int kappa = __popc(mask);
  float np[2];
  if (kappa <= A.kappa_hard) {
    np[0] = cen[0];
    np[1] = cen[1];
  } else {
    np[0] = cen[0] + sx.x / swf;
    np[1] = cen[1] + sx.y / swf;
  }
  bool finite = true;
#pragma unroll
  for (int a = 0; a < 2; ++a) finite &= isfinite(np[a]) && fabsf(np[a]) < 64.f;
  if (!finite) {
    atomicOr(A.status, ST_NONFINITE);
    np[0] = cen[0];
    np[1] = cen[1];
  }
  int sh[2];
  float off[2];
#pragma unroll
  for (int a = 0; a < 2; ++a) {
    const float fl = floorf(np[a]);
    sh[a] = (int)fl;
    off[a] = np[a] - fl;
    if (off[a] >= 1.f) {
      off[a] = 0.f;
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
  return true;
}

// ---- weights: per component, 1 / (sum over control points within R of (R - d)) -----------------

template <int Q>
__device__ __forceinline__ bool weights_ds_tile(const Args<Q, 2, PF32>& A, const Tile2& T, const InstK& I,
                                                const TileGeo& G, unsigned char* smem) {
  const int rw = G.tx + G.cp.xh - G.cp.xl, rh = G.ty + G.cp.yh - G.cp.yl;
  const int cells = rw * rh;
  const DenseSmem S = dense_smem(smem, cells, 0);
  // the tile's own moments (at most two per cell)
  const int lx = threadIdx.x % G.tx, ly = threadIdx.x / G.tx;
  const int Sx = T.x0 + lx, Sy = T.y0 + ly;
  int m0 = 0, m1 = 0, many = 0;
  if (ly < G.ty && Sx < I.dims[0] && Sy < I.dims[1])
    cell_items(A.a.start, I.base + (uint32_t)Sx + (uint32_t)I.dims[0] * (uint32_t)Sy, &m0, &m1, &many);
  __shared__ SecondMoments L2;
  if (threadIdx.x == 0) L2.n = 0;  // ordered before its use by stage_dense's barriers
  const bool dense = stage_dense(I, T.x0 + G.cp.xl, T.y0 + G.cp.yl, rw, rh, A.b.start, S, many,
                                 [&](float4* r, unsigned char*, int, int, int c, float nxt) {
                                   *r = make_float4(A.b.off[c], A.b.off[A.ccap + c], nxt, 0.f);
                                 });
  if (!dense) return false;
  const int no = *S.novf;  // second items in the overflow list (at most kOvf in a dense tile)

  const int bx0 = lx - G.cp.xl, by0 = ly - G.cp.yl;  // region coordinates of the moments' cell
  if (m1 - m0 == 2) {
    const int q = atomicAdd(&L2.n, 1);  // one entry per thread at most: q < blockDim.x = 256
    L2.item[q] = m0 + 1;
    L2.bx[q] = (short)bx0;
    L2.by[q] = (short)by0;
  }
  // work units: this thread's first moment with all Q directions, then (second moment, direction)
  // units strided over the block; every thread reaches the barrier once, on entering the second
  bool own = m1 > m0, synced = false;
  int u = (int)threadIdx.x;
#pragma unroll 1
  while (true) {
    int m, k0, k1, bx, by;
    if (own) {
      own = false;
      m = m0;
      k0 = 0;
      k1 = Q;
      bx = bx0;
      by = by0;
    } else {
      if (!synced) {
        __syncthreads();
        synced = true;
      }
      if (u >= L2.n * Q) break;
      const int e = u / Q;
      m = L2.item[e];
      k0 = u - e * Q;
      k1 = k0 + 1;
      bx = L2.bx[e];
      by = L2.by[e];
      u += blockDim.x;
    }
    const float2 o = make_float2(A.a.off[m], A.a.off[A.mcap + m]);
    // control-point offsets u (relative to the component's cell) with a possible hit
    int ulx, nxs, uly, nys;
    stencil_axis(o.x, A.R, A.tiny, &ulx, &nxs);
    stencil_axis(o.y, A.R, A.tiny, &uly, &nys);
    const bool wide = nxs != 4 || nys != 4;  // exact-range loops otherwise
    float bxv[4], byv[4];  // base = float(cd - dG) = float(-u), exact
#pragma unroll
    for (int a = 0; a < 4; ++a) {
      bxv[a] = (float)(-(ulx + a));
      byv[a] = (float)(-(uly + a));
    }
#pragma unroll 1
    for (int k = k0; k < k1; ++k) {
      const int cdx = __float2int_rn(A.L.cdf[k][0]), cdy = __float2int_rn(A.L.cdf[k][1]);
      const int c0 = (by + uly + cdy) * rw + (bx + ulx + cdx);
      CSum sws;
      auto one = [&](float4 pc, float basex, float basey) {
        const float2 q = __fadd2_rn(make_float2(basex, basey), make_float2(-pc.x, -pc.y));
        const float2 e = __fadd2_rn(o, q);
        const float2 e2 = __fmul2_rn(e, e);
        const float d2 = rn_add(e2.x, e2.y);
        if (d2 <= A.R2) sws.add(A.R - rn_sqrt(d2));
      };
      // first items of the window's cells
      auto visit = [&](int ci, float basex, float basey) { one(S.rec[ci], basex, basey); };
      const int ncol = wide ? nxs : 4;
      if (!wide) {
#pragma unroll
        for (int b = 0; b < 4; ++b)
#pragma unroll
          for (int a = 0; a < 4; ++a) visit(c0 + b * rw + a, bxv[a], byv[b]);
      } else {
#pragma unroll 1
        for (int b = 0; b < nys; ++b)
#pragma unroll 1
          for (int a = 0; a < nxs; ++a) visit(c0 + b * rw + a, (float)(-(ulx + a)), (float)(-(uly + b)));
      }
      // then the second items, in window order
      uint32_t ov = no ? second_item_mask(S, no, by + uly + cdy, bx + ulx + cdx, wide ? nys : 4, ncol) : 0u;
#pragma unroll 1
      while (ov) {
        const int pos = __ffs(ov) - 1;
        ov &= ov - 1;
        const int b = wide ? pos / ncol : pos >> 2, a = pos - b * ncol;
        one(S.orec[(int)S.rec[c0 + b * rw + a].z], (float)(-(ulx + a)), (float)(-(uly + b)));
      }
      const float sw = sws.value();
      A.sw[(int64_t)k * A.mcap + m] = sw > 0.f ? 1.f / sw : 0.f;
    }
  }
  return true;
}

// ---- gather: per control point and direction ------------------------------------------------------
// Per-direction data: (1/sw, f*_k) of each item, direction-major.

template <int Q>
__device__ __forceinline__ bool gather_ds_tile(const Args<Q, 2, PF32>& A, const Tile2& T, const InstK& I,
                                               const TileGeo& G, unsigned char* smem) {
  const int rw = G.tx + G.mom.xh - G.mom.xl, rh = G.ty + G.mom.yh - G.mom.yl;
  const int cells = rw * rh;
  const DenseSmem S = dense_smem(smem, cells, (size_t)8 * Q);
  const float2* s_kv = reinterpret_cast<const float2*>(S.dat);
  const float2* s_okv = reinterpret_cast<const float2*>(S.odat);
  // the tile's own control points (at most two per cell)
  const int lx = threadIdx.x % G.tx, ly = threadIdx.x / G.tx;
  const int Fx = T.x0 + lx, Fy = T.y0 + ly;
  int j0 = 0, j1 = 0, many = 0;
  if (ly < G.ty && Fx < I.dims[0] && Fy < I.dims[1])
    cell_items(A.b.start, I.base + (uint32_t)Fx + (uint32_t)I.dims[0] * (uint32_t)Fy, &j0, &j1, &many);
  __shared__ SecondMoments L2;
  if (threadIdx.x == 0) L2.n = 0;  // ordered before its use by stage_dense's barriers
  const bool dense = stage_dense(I, T.x0 + G.mom.xl, T.y0 + G.mom.yl, rw, rh, A.a.start, S, many,
                                 [&](float4* r, unsigned char* dat, int stride, int slot, int m, float nxt) {
                                   *r = make_float4(A.a.off[m], A.a.off[A.mcap + m], nxt, A.a.rho[m]);
                                   float2* kv = reinterpret_cast<float2*>(dat);
#pragma unroll
                                   for (int k = 0; k < Q; ++k)
                                     kv[k * stride + slot] = make_float2(A.sw[(int64_t)k * A.mcap + m],
                                                                         A.a.dev[(int64_t)k * A.mcap + m]);
                                 });
  if (!dense) return false;
  const int no = *S.novf;  // second items in the overflow list (at most kOvf in a dense tile)

  const int bx0 = lx - G.mom.xl, by0 = ly - G.mom.yl;  // region coordinates of the control points' cell
  if (j1 - j0 == 2) {
    const int q = atomicAdd(&L2.n, 1);  // one entry per thread at most: q < blockDim.x = 256
    L2.item[q] = j0 + 1;
    L2.bx[q] = (short)bx0;
    L2.by[q] = (short)by0;
  }
  // work units: this thread's first control point with all Q directions, then (second control
  // point, direction) units strided over the block; every thread reaches the barrier once
  bool own = j1 > j0, synced = false;
  int u = (int)threadIdx.x;
#pragma unroll 1
  while (true) {
    int j, k0, k1, bx, by;
    if (own) {
      own = false;
      j = j0;
      k0 = 0;
      k1 = Q;
      bx = bx0;
      by = by0;
    } else {
      if (!synced) {
        __syncthreads();
        synced = true;
      }
      if (u >= L2.n * Q) break;
      const int e = u / Q;
      j = L2.item[e];
      k0 = u - e * Q;
      k1 = k0 + 1;
      bx = L2.bx[e];
      by = L2.by[e];
      u += blockDim.x;
    }
    const float2 pp = make_float2(A.b.off[j], A.b.off[A.ccap + j]);
    int jlx, nxs, jly, nys;
    stencil_axis(pp.x, A.R, A.tiny, &jlx, &nxs);
    stencil_axis(pp.y, A.R, A.tiny, &jly, &nys);
    const bool wide = nxs != 4 || nys != 4;  // exact-range loops otherwise
    float cx[4], cy[4];
#pragma unroll
    for (int a = 0; a < 4; ++a) {
      cx[a] = rn_sub((float)(jlx + a), pp.x);
      cy[a] = rn_sub((float)(jly + a), pp.y);
    }
    uint32_t empty = 0;
#pragma unroll 1
    for (int k = k0; k < k1; ++k) {
      const int cdx = __float2int_rn(A.L.cdf[k][0]), cdy = __float2int_rn(A.L.cdf[k][1]);
      const int c0 = (by + jly - cdy) * rw + (bx + jlx - cdx);
      const float2* kvk = s_kv + k * cells;
      const float2* okvk = s_okv + k * kOvf;
      CSum sa;
      float sb = 0.f;  // deviation part: plain FMA accumulation, as in the row-segment gathers
      auto one = [&](float4 o, const float2* kvp, float ex0, float ey0) {
        const float2 e = __fadd2_rn(make_float2(o.x, o.y), make_float2(ex0, ey0));
        const float2 e2 = __fmul2_rn(e, e);
        const float d2 = rn_add(e2.x, e2.y);
        if (d2 <= A.R2) {
          // a dropped component has 1/sw = 0: its weight is +0 and leaves every sum unchanged
          const float2 kv = *kvp;
          const float rho = o.w;
          const float wgt = (A.R - rn_sqrt(d2)) * kv.x;
          const float p = __fmul_rn(wgt, rho);
          const float2 r = __ffma2_rn(make_float2(wgt, wgt), make_float2(rho, kv.y), make_float2(-p, sb));
          sa.add(p);
          sa.lo = __fadd_rn(sa.lo, r.x);
          sb = r.y;
        }
      };
      // first items of the window's cells
      auto visit = [&](int ci, float ex0, float ey0) { one(S.rec[ci], kvk + ci, ex0, ey0); };
      const int ncol = wide ? nxs : 4;
      if (!wide) {
#pragma unroll
        for (int b = 0; b < 4; ++b)
#pragma unroll
          for (int a = 0; a < 4; ++a) visit(c0 + b * rw + a, cx[a], cy[b]);
      } else {
#pragma unroll 1
        for (int b = 0; b < nys; ++b) {
          const float cyb = rn_sub((float)(jly + b), pp.y);
#pragma unroll 1
          for (int a = 0; a < nxs; ++a) visit(c0 + b * rw + a, rn_sub((float)(jlx + a), pp.x), cyb);
        }
      }
      // then the second items, in window order
      uint32_t ov = no ? second_item_mask(S, no, by + jly - cdy, bx + jlx - cdx, wide ? nys : 4, ncol) : 0u;
#pragma unroll 1
      while (ov) {
        const int pos = __ffs(ov) - 1;
        ov &= ov - 1;
        const int b = wide ? pos / ncol : pos >> 2, a = pos - b * ncol;
        const int q = (int)S.rec[c0 + b * rw + a].z;
        one(S.orec[q], okvk + q, rn_sub((float)(jlx + a), pp.x), rn_sub((float)(jly + b), pp.y));
      }
      const DF Ad = df_norm(sa.hi, sa.lo);
      const DF Fv = df_add(df_mul(DF{A.L.wf[k], A.L.wlo[k]}, Ad), DF{sb, 0.f});
      A.cpfhi[(int64_t)k * A.ccap + j] = Fv.hi;
      A.cpflo[(int64_t)k * A.ccap + j] = Fv.lo;
      if (Fv.hi < A.eps) empty |= 1u << k;
    }
    // the mask is cleared before the launch: a first control point's whole mask has one writer,
    // a second one's directions are spread over threads and combine
    if (empty) {
      if (k1 - k0 == Q) A.emask[j] = empty;
      else atomicOr(A.emask + j, empty);
    }
  }
  return true;
}

// ---- kernels ----------------------------------------------------------------------------------------
//
// The dense kernels take the tile list (one block per tile, or persistent over it).  A tile that
// is not dense is appended to a fallback list (fb_tiles, *fb_count, cleared before the launch);
// the matching k_*_fb kernel then runs the row-segment code on exactly those tiles.  Keeping the
// two paths in separate kernels keeps the dense kernels' register count (and occupancy) their
// own.  The order of the fallback list is arbitrary, which changes no result: tiles write
// disjoint outputs.

// Resident blocks per SM the dense kernels are compiled for (register budgets 48, 40 and 64;
// chosen by timing the ensemble step on GB300).
#ifndef DBM_DS_BLOCKS_THIN
#define DBM_DS_BLOCKS_THIN 5
#endif
#ifndef DBM_DS_BLOCKS_WEIGHTS
#define DBM_DS_BLOCKS_WEIGHTS 6
#endif
#ifndef DBM_DS_BLOCKS_GATHER
#define DBM_DS_BLOCKS_GATHER 4
#endif

__device__ __forceinline__ void defer_tile(int tb, int* fb_tiles, int* fb_count) {
  if (threadIdx.x == 0) fb_tiles[atomicAdd(fb_count, 1)] = tb;
}

template <int Q>
__global__ void __launch_bounds__(256, DBM_DS_BLOCKS_THIN) k_thin_refine_ds(const __grid_constant__ Args<Q, 2, PF32> A,
                                                          const Tile2* __restrict__ tiles, const TileGeo G, int ntiles,
                                                          int* fb_tiles, int* fb_count) {
  extern __shared__ __align__(16) unsigned char smem[];
  for (int tb = blockIdx.x; tb < ntiles; tb += gridDim.x) {
    const Tile2 T = tiles[tb];
    const InstK I = A.inst[T.inst];
    if (!thin_refine_ds_tile<Q>(A, T, I, G, smem)) defer_tile(tb, fb_tiles, fb_count);
    __syncthreads();
  }
}

template <int Q>
__global__ void __launch_bounds__(256, DBM_DS_BLOCKS_WEIGHTS) k_weights_ds(const __grid_constant__ Args<Q, 2, PF32> A,
                                                      const Tile2* __restrict__ tiles, const TileGeo G, int ntiles,
                                                      int* fb_tiles, int* fb_count) {
  extern __shared__ __align__(16) unsigned char smem[];
  for (int tb = blockIdx.x; tb < ntiles; tb += gridDim.x) {
    const Tile2 T = tiles[tb];
    const InstK I = A.inst[T.inst];
    if (!weights_ds_tile<Q>(A, T, I, G, smem)) defer_tile(tb, fb_tiles, fb_count);
    __syncthreads();
  }
}

template <int Q>
__global__ void __launch_bounds__(256, DBM_DS_BLOCKS_GATHER) k_gather_ds(const __grid_constant__ Args<Q, 2, PF32> A,
                                                     const Tile2* __restrict__ tiles, const TileGeo G, int ntiles,
                                                     int* fb_tiles, int* fb_count) {
  extern __shared__ __align__(16) unsigned char smem[];
  for (int tb = blockIdx.x; tb < ntiles; tb += gridDim.x) {
    const Tile2 T = tiles[tb];
    const InstK I = A.inst[T.inst];
    if (!gather_ds_tile<Q>(A, T, I, G, smem)) defer_tile(tb, fb_tiles, fb_count);
    __syncthreads();
  }
}

// Row-segment passes over the deferred tiles (persistent grid; nothing to do when the list is
// empty).  STAGE: 0 thin + refine, 1 weights, 2 gather.
template <int Q, int STAGE>
__global__ void __launch_bounds__(256) k_dense_fallback(const __grid_constant__ Args<Q, 2, PF32> A,
                                                       const Tile2* __restrict__ tiles, const TileGeo G,
                                                       const int* __restrict__ fb_tiles,
                                                       const int* __restrict__ fb_count) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int n = *fb_count;
  for (int i = blockIdx.x; i < n; i += gridDim.x) {
    const Tile2 T = tiles[fb_tiles[i]];
    const InstK I = A.inst[T.inst];
    if constexpr (STAGE == 0) thin_refine_tile<Q, PF32, true>(A, T, I, G, smem);
    else if constexpr (STAGE == 1) weights_tile<Q, PF32, true>(A, T, I, G, smem);
    else gather_ts_tile<Q>(A, T, I, G, smem);
    __syncthreads();
  }
}

}  // namespace dbm
