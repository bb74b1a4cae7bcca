// Dense-stencil variants of the three whole-cell window kernels (2D, FP32 store).
//
// With whole-cell displacements (every cd_k an integer, D2Q9 with dx = cell) and R < 2 cells, the
// thinning cell holds at most one control point, and in the ensemble and inverse-problem
// workloads every cell of the grid holds exactly one moment at every step (the refine move stays
// inside its cell).  A tile whose region satisfies "at most one item per cell" is staged as a
// dense grid -- one slot per region cell, an empty cell holding an offset far outside every
// window -- and each reference point's window for direction k becomes a fixed 4 x 4 block of
// cells: the component-cell offsets j with e = off + (j - p) in reach of R are
// floor(p - R - tiny) .. floor(p + R + tiny), four values per axis at R = 1.5 except within tiny
// of p = 1/2 (five).  A point whose range is not four wide takes a loop over its exact range, so
// no access leaves the cells the region stages (its halo covers the exact ranges for any R < 2).  Every thread then runs the same
// unrolled stencil, without the per-row bookkeeping and the uneven loop trips of the row-segment
// loops, and the canonical c = rn(float(j) - p) of the stencil's four columns and rows is
// computed once per point.
//
// Results are bit-identical to the row-segment kernels: each sum visits the same hits in the same
// order (window rows ascending, then columns ascending, one item per cell) with the same
// operations.  A tile whose region (or own cells) holds a cell with two or more items is handed to
// the row-segment code (a second, normally empty, launch over the deferred tiles).
#pragma once

#include "sim_tiled.cuh"

namespace dbm {

// Offset stored for an empty cell: every displacement from it is ~1e4 cells, far outside R.
constexpr float kEmptyOff = 1.0e4f;

// Bytes of dynamic shared memory of the dense layouts (region of rw x rh cells).
__host__ __device__ inline size_t dense_off(size_t n) { return (n + 15) & ~(size_t)15; }
__host__ __device__ inline size_t ds_bytes_refine(int Q, int cells) {
  return dense_off((size_t)cells * 8) + dense_off((size_t)Q * cells * 4);
}
__host__ __device__ inline size_t ds_bytes_weights(int cells) { return dense_off((size_t)cells * 8); }
__host__ __device__ inline size_t ds_bytes_gather(int Q, int cells) {
  return dense_off((size_t)cells * 8) + dense_off((size_t)cells * 4) + dense_off((size_t)Q * cells * 8);
}

// The single item of global cell g in a state's sorted ranges: its index, -1 if the cell is
// empty; sets *many if the cell holds two or more items.
__device__ __forceinline__ int single_item(const uint32_t* __restrict__ start, uint32_t g, int* many) {
  const uint32_t b = start[g], e = start[g + 1];
  if (e - b == 1u) return (int)b;
  if (e != b) *many = 1;
  return -1;
}

// Stencil origin and width along one axis for reference offset p: j in [lo, lo + n).
__device__ __forceinline__ void stencil_axis(float p, float R, float tiny, int* lo, int* n) {
  *lo = (int)floorf(p - R - tiny);
  *n = (int)floorf(p + R + tiny) - *lo + 1;
}

// ---- thinning + refine --------------------------------------------------------------------------

template <int Q>
__device__ __forceinline__ bool thin_refine_ds_tile(const Args<Q, 2, PF32>& A, const Tile2& T, const InstK& I,
                                                    const TileGeo& G, unsigned char* smem) {
  const int rw = G.tx + G.mom.xh - G.mom.xl, rh = G.ty + G.mom.yh - G.mom.yl;
  const int cells = rw * rh;
  float2* s_off = reinterpret_cast<float2*>(smem);
  float* s_w = reinterpret_cast<float*>(smem + dense_off((size_t)cells * 8));  // exp(f*) [Q][cells]
  int many = 0;
  const int xr0 = T.x0 + G.mom.xl, yr0 = T.y0 + G.mom.yl;
  for (int ci = threadIdx.x; ci < cells; ci += blockDim.x) {
    const int ry = ci / rw, rx = ci - ry * rw;
    uint32_t g;
    const int m = region_cell(I, xr0 + rx, yr0 + ry, &g) ? single_item(A.a.start, g, &many) : -1;
    if (m >= 0) {
      s_off[ci] = make_float2(A.a.off[m], A.a.off[A.mcap + m]);
#pragma unroll
      for (int k = 0; k < Q; ++k) s_w[k * cells + ci] = exp(fstar_at<Q, 2, PF32>(A, (uint32_t)m, k));
    } else {
      s_off[ci] = make_float2(kEmptyOff, kEmptyOff);
    }
  }
  if (__syncthreads_or(many)) return false;

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
        const float2 o = s_off[(by + soy) * rw + (bx + sox)];
        const float tx = rn_add(o.x, cdx), ty = rn_add(o.y, cdy);
        const float sxf = (float)sox;
        if (tx >= -sxf && tx < 1.f - sxf && ty >= fy0 && ty < fy0 + 1.f) {
          ++cnt;
          csum[0].add(rn_add(sxf, tx));
          csum[1].add(rn_add(sy, ty));
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
    bool hit = false;
    auto visit = [&](int ci, float ex0, float ey0) {
      const float2 o = s_off[ci];
      const float2 e = __fadd2_rn(o, make_float2(ex0, ey0));
      const float2 e2 = __fmul2_rn(e, e);
      if (rn_add(e2.x, e2.y) <= A.R2) {
        hit = true;
        const float wt = wk[ci];
        swf = __fadd_rn(swf, wt);
        sx = __ffma2_rn(make_float2(wt, wt), e, sx);
      }
    };
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
  float2* s_cp = reinterpret_cast<float2*>(smem);  // control-point offsets
  int many = 0;
  const int xr0 = T.x0 + G.cp.xl, yr0 = T.y0 + G.cp.yl;
  for (int ci = threadIdx.x; ci < cells; ci += blockDim.x) {
    const int ry = ci / rw, rx = ci - ry * rw;
    uint32_t g;
    const int c = region_cell(I, xr0 + rx, yr0 + ry, &g) ? single_item(A.b.start, g, &many) : -1;
    s_cp[ci] = c >= 0 ? make_float2(A.b.off[c], A.b.off[A.ccap + c]) : make_float2(kEmptyOff, kEmptyOff);
  }
  // the tile's own moment (one per cell at most)
  const int lx = threadIdx.x % G.tx, ly = threadIdx.x / G.tx;
  const int Sx = T.x0 + lx, Sy = T.y0 + ly;
  int m = -1;
  if (ly < G.ty && Sx < I.dims[0] && Sy < I.dims[1])
    m = single_item(A.a.start, I.base + (uint32_t)Sx + (uint32_t)I.dims[0] * (uint32_t)Sy, &many);
  if (__syncthreads_or(many)) return false;
  if (m < 0) return true;

  const float2 o = make_float2(A.a.off[m], A.a.off[A.mcap + m]);
  const int bx = lx - G.cp.xl, by = ly - G.cp.yl;  // region coordinates of the moment's cell
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
  for (int k = 0; k < Q; ++k) {
    const int cdx = __float2int_rn(A.L.cdf[k][0]), cdy = __float2int_rn(A.L.cdf[k][1]);
    const int c0 = (by + uly + cdy) * rw + (bx + ulx + cdx);
    CSum sws;
    auto visit = [&](int ci, float basex, float basey) {
      const float2 pc = s_cp[ci];
      const float2 q = __fadd2_rn(make_float2(basex, basey), make_float2(-pc.x, -pc.y));
      const float2 e = __fadd2_rn(o, q);
      const float2 e2 = __fmul2_rn(e, e);
      const float d2 = rn_add(e2.x, e2.y);
      if (d2 <= A.R2) sws.add(A.R - rn_sqrt(d2));
    };
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
    const float sw = sws.value();
    A.sw[(int64_t)k * A.mcap + m] = sw > 0.f ? 1.f / sw : 0.f;
  }
  return true;
}

// ---- gather: per control point and direction ------------------------------------------------------

template <int Q>
__device__ __forceinline__ bool gather_ds_tile(const Args<Q, 2, PF32>& A, const Tile2& T, const InstK& I,
                                               const TileGeo& G, unsigned char* smem) {
  const int rw = G.tx + G.mom.xh - G.mom.xl, rh = G.ty + G.mom.yh - G.mom.yl;
  const int cells = rw * rh;
  float2* s_off = reinterpret_cast<float2*>(smem);
  float* s_rho = reinterpret_cast<float*>(smem + dense_off((size_t)cells * 8));
  float2* s_kv = reinterpret_cast<float2*>(smem + dense_off((size_t)cells * 8) + dense_off((size_t)cells * 4));
  int many = 0;
  const int xr0 = T.x0 + G.mom.xl, yr0 = T.y0 + G.mom.yl;
  for (int ci = threadIdx.x; ci < cells; ci += blockDim.x) {
    const int ry = ci / rw, rx = ci - ry * rw;
    uint32_t g;
    const int m = region_cell(I, xr0 + rx, yr0 + ry, &g) ? single_item(A.a.start, g, &many) : -1;
    if (m >= 0) {
      s_off[ci] = make_float2(A.a.off[m], A.a.off[A.mcap + m]);
      s_rho[ci] = A.a.rho[m];
#pragma unroll
      for (int k = 0; k < Q; ++k)
        s_kv[k * cells + ci] = make_float2(A.sw[(int64_t)k * A.mcap + m], A.a.dev[(int64_t)k * A.mcap + m]);
    } else {
      s_off[ci] = make_float2(kEmptyOff, kEmptyOff);
    }
  }
  // the tile's own control point (one per cell at most)
  const int lx = threadIdx.x % G.tx, ly = threadIdx.x / G.tx;
  const int Fx = T.x0 + lx, Fy = T.y0 + ly;
  int j = -1;
  if (ly < G.ty && Fx < I.dims[0] && Fy < I.dims[1])
    j = single_item(A.b.start, I.base + (uint32_t)Fx + (uint32_t)I.dims[0] * (uint32_t)Fy, &many);
  if (__syncthreads_or(many)) return false;
  if (j < 0) return true;

  const float2 pp = make_float2(A.b.off[j], A.b.off[A.ccap + j]);
  const int bx = lx - G.mom.xl, by = ly - G.mom.yl;  // region coordinates of the CP's cell
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
  for (int k = 0; k < Q; ++k) {
    const int cdx = __float2int_rn(A.L.cdf[k][0]), cdy = __float2int_rn(A.L.cdf[k][1]);
    const int c0 = (by + jly - cdy) * rw + (bx + jlx - cdx);
    const float2* kvk = s_kv + k * cells;
    CSum sa;
    float sb = 0.f;  // deviation part: plain FMA accumulation, as in the row-segment gathers
    auto visit = [&](int ci, float ex0, float ey0) {
      const float2 o = s_off[ci];
      const float2 e = __fadd2_rn(o, make_float2(ex0, ey0));
      const float2 e2 = __fmul2_rn(e, e);
      const float d2 = rn_add(e2.x, e2.y);
      if (d2 <= A.R2) {
        // a dropped component has 1/sw = 0: its weight is +0 and leaves every sum unchanged
        const float2 kv = kvk[ci];
        const float rho = s_rho[ci];
        const float wgt = (A.R - rn_sqrt(d2)) * kv.x;
        const float p = __fmul_rn(wgt, rho);
        const float2 r = __ffma2_rn(make_float2(wgt, wgt), make_float2(rho, kv.y), make_float2(-p, sb));
        sa.add(p);
        sa.lo = __fadd_rn(sa.lo, r.x);
        sb = r.y;
      }
    };
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
    const DF Ad = df_norm(sa.hi, sa.lo);
    const DF Fv = df_add(df_mul(DF{A.L.wf[k], A.L.wlo[k]}, Ad), DF{sb, 0.f});
    A.cpfhi[(int64_t)k * A.ccap + j] = Fv.hi;
    A.cpflo[(int64_t)k * A.ccap + j] = Fv.lo;
    if (Fv.hi < A.eps) empty |= 1u << k;
  }
  // this thread is the only writer of its control point's mask (cleared before the launch)
  if (empty) A.emask[j] = empty;
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

// Resident blocks per SM the dense kernels are compiled for (register budgets 48, 36 and 64;
// chosen by timing the ensemble step on GB300).
#ifndef DBM_DS_BLOCKS_THIN
#define DBM_DS_BLOCKS_THIN 5
#endif
#ifndef DBM_DS_BLOCKS_WEIGHTS
#define DBM_DS_BLOCKS_WEIGHTS 7
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
