// The fused DiReBM step (replaces direbm/warp/simulator.py:50-73 and the propagation pipeline it
// drives, direbm/warp/propagation.py:21-275).
//
// One step, all on the device, no host synchronisation:
//   k_collide       BGK relaxation of every moment in place        (warp/physics.py:45-62)
//   k_thin_refine   per cell: gather the components landing in it (cell thinning, centroid;
//                   propagation.py:39-68,130-153), then refine the control point with the
//                   components within r (kappa mask, exp(f)-weighted move; propagation.py:77-112)
//   compaction      occupied cells -> (refined cell, origin cell) pairs, P on the device
//   radix sort      stable sort of the pairs by refined cell (the next step's moment order)
//   k_finalize      sorted control points -> next state's cells/offsets, + cell ranges
//   k_weights       per component: sw = sum over control points within r of (r - d)
//                   (propagation.py:166-178; the drop rule sw <= 0 is kept)
//   k_gather        per control point and direction: sum (r - d)/sw * f over components within r
//                   (propagation.py:179-186 as a gather: no float atomics, fixed order)
//   k_emit          gap fill of empty directions + emit the next moments (propagation.py:189-218)
//
// Every sum runs in a fixed order inside one thread, so results are bitwise reproducible run to
// run.  FP32DEV stores f as rho (FP32) + dev_k = f_k - rho*W_k (FP32), sums with compensated
// (TwoSum/TwoProd) FP32 accumulators and forms the emitted rho and dev in double-float.
#include <algorithm>
#include <cmath>
#include <limits>
#include <vector>

#include "sim.cuh"
#include "sortscan.cuh"

namespace dbm {

// ---- kernels ------------------------------------------------------------------------------------

template <int Q, int D, class P>
__global__ void __launch_bounds__(256) k_collide(const __grid_constant__ Args<Q, D, P> A) {
  using real = typename P::real;
  const uint32_t M = *A.a.count;
  for (uint32_t m = blockIdx.x * blockDim.x + threadIdx.x; m < M; m += gridDim.x * blockDim.x) {
    const uint32_t g = A.a.cell[m];
    const int b = find_instance(A.inst_base, A.n_inst, g);
    const InstK I = A.inst[b];
    int c[3] = {0, 0, 0};
    if (!I.periodic || I.has_obs || I.inflow_w > 0) decode_cell<D>(I, g, c);
    const bool inflow = I.inflow_w > 0 && c[0] < I.inflow_w;  // reset to the inflow equilibrium
    if constexpr (std::is_same<P, PF64>::value) {
      double f[Q];
#pragma unroll
      for (int k = 0; k < Q; ++k) f[k] = A.a.f64[(int64_t)k * A.mcap + m];
      if (inflow) {
        double rho = 0, u[D];
#pragma unroll
        for (int k = 0; k < Q; ++k) rho += f[k];
#pragma unroll
        for (int a = 0; a < D; ++a) u[a] = I.u_in[a];
        equilibrium_all<Q, D, double>(rho, u, A.L, f);
      } else {
        collide_moment<Q, D, double>(f, I.tau, A.L);
      }
#pragma unroll
      for (int k = 0; k < Q; ++k) A.a.f64[(int64_t)k * A.mcap + m] = f[k];
      if (A.want_wexp) {  // the refine weight exp(f*) once per component (its window kernel reads it)
#pragma unroll
        for (int k = 0; k < Q; ++k) A.wexp[(int64_t)k * A.mcap + m] = exp(f[k]);
      }
    } else {
      float dv[Q];
#pragma unroll
      for (int k = 0; k < Q; ++k) dv[k] = A.a.dev[(int64_t)k * A.mcap + m];
      if (inflow) {
        float u[D];
#pragma unroll
        for (int a = 0; a < D; ++a) u[a] = (float)I.u_in[a];
        eq_deviation_f32<Q, D>(A.a.rho[m], u, A.L, dv);
      } else {
        collide_moment_dev<Q, D>(A.a.rho[m], dv, (float)I.tau, A.L);
      }
#pragma unroll
      for (int k = 0; k < Q; ++k) A.a.dev[(int64_t)k * A.mcap + m] = dv[k];
      if (A.want_wexp) {
        const float rho = A.a.rho[m];
#pragma unroll
        for (int k = 0; k < Q; ++k) A.wexp[(int64_t)k * A.mcap + m] = exp(__fmaf_rn(rho, A.L.wf[k], dv[k]));
      }
    }
    uint32_t bm = 0;
    real om[3] = {0, 0, 0};
    if (I.has_obs) {
#pragma unroll
      for (int a = 0; a < D; ++a) om[a] = A.a.off[(int64_t)a * A.mcap + m];
    }
    if (I.has_obs && sphere_dist2<D, real>(I, c, om) < I.near2) {
      // bounce-back: a direction whose end point lies inside the solid is blocked
#pragma unroll 1
      for (int k = 1; k < Q; ++k) {
        double o[3] = {0, 0, 0};
#pragma unroll
        for (int a = 0; a < D; ++a) o[a] = __dadd_rn((double)A.a.off[(int64_t)a * A.mcap + m], A.L.cd[k][a]);
        if (inside_sphere<D>(I, c, o)) bm |= 1u << k;
      }
    }
    if (A.any_obstacle) A.bmask[m] = bm;
    if (!I.periodic) {  // every component must land inside a bounded box (bounced ones stay put)
      bool out = false;
#pragma unroll
      for (int k = 0; k < Q; ++k) {
        if ((bm >> k) & 1u) continue;
#pragma unroll
        for (int a = 0; a < D; ++a) {
          real t = rn_add(A.a.off[(int64_t)a * A.mcap + m], A.L.template cd_as<real>(k, a));
          int x = c[a] + (int)floor(t);
          out |= (x < 0) | (x >= I.dims[a]);
        }
      }
      if (out) atomicOr(A.status, ST_OUT_OF_BOX);
    }
  }
}

template <int Q, int D, class P>
__device__ __forceinline__ typename P::real fstar_at(const Args<Q, D, P>& A, uint32_t m, int k) {
  if constexpr (std::is_same<P, PF64>::value) {
    return A.a.f64[(int64_t)k * A.mcap + m];
  } else {
    return __fmaf_rn(A.a.rho[m], A.L.wf[k], A.a.dev[(int64_t)k * A.mcap + m]);
  }
}

template <class P>
constexpr int thin_min_blocks() { return std::is_same<P, PF64>::value ? 1 : 6; }

// Thinning + refine of one cell F of instance I (the untiled window kernels).
template <int Q, int D, class P>
__device__ __forceinline__ void thin_refine_cell(const Args<Q, D, P>& A, const uint32_t F, const InstK& I) {
  using real = typename P::real;
  int Fc[3];
  decode_cell<D>(I, F, Fc);

  // ---- thinning: components landing in F (2 candidate source cells per axis per direction) ----
  uint32_t cnt = 0;
  real sum[3] = {0, 0, 0};
  CSum csum[3];
#pragma unroll 1
  for (int k = 0; k < Q; ++k) {
    int lo[3] = {0, 0, 0}, nn[3] = {1, 1, 1};
#pragma unroll
    for (int a = 0; a < D; ++a) thin_sources<real>(A.L.template cd_as<real>(k, a), &lo[a], &nn[a]);
#pragma unroll 1
    for (int oz = 0; oz < nn[2]; ++oz)
#pragma unroll 1
      for (int oy = 0; oy < nn[1]; ++oy)
#pragma unroll 1
        for (int ox = 0; ox < nn[0]; ++ox) {
          const int so[3] = {lo[0] + ox, lo[1] + oy, D == 3 ? lo[2] + oz : 0};
          uint32_t Sg;
          if (!cell_at<D>(I, Fc[0] + so[0], Fc[1] + so[1], Fc[2] + so[2], &Sg)) continue;
          const uint32_t m0 = A.a.start[Sg], m1 = A.a.start[Sg + 1];
          for (uint32_t m = m0; m < m1; ++m) {
            if (A.any_obstacle && ((A.bmask[m] >> k) & 1u)) continue;  // bounced: stays in its cell
            const PackItem<real> it = A.a.pk[m];  // the offsets in one load
            const real om[3] = {it.x, it.y, it.z};
            real t[3];
            bool land = true;
#pragma unroll
            for (int a = 0; a < D; ++a) {
              t[a] = rn_add(om[a], A.L.template cd_as<real>(k, a));
              land &= (so[a] + (int)floor(t[a])) == 0;
            }
            if (land) {
              ++cnt;
#pragma unroll
              for (int a = 0; a < D; ++a) {
                real rel = rn_add((real)so[a], t[a]);
                if constexpr (std::is_same<P, PF64>::value) sum[a] += rel; else csum[a].add(rel);
              }
            }
          }
        }
  }
  if (A.any_obstacle) {  // bounced components land in their own cell, at their moment's offset
    for (uint32_t m = A.a.start[F], m1 = A.a.start[F + 1]; m < m1; ++m) {
      const uint32_t bits = A.bmask[m];
#pragma unroll 1
      for (int k = 1; k < Q; ++k) {
        if (!((bits >> k) & 1u)) continue;
        ++cnt;
#pragma unroll
        for (int a = 0; a < D; ++a) {
          const real rel = A.a.off[(int64_t)a * A.mcap + m];
          if constexpr (std::is_same<P, PF64>::value) sum[a] += rel; else csum[a].add(rel);
        }
      }
    }
  }
  if (cnt == 0) {
    A.occ[F] = 0u;
    if (A.kappa_soft > 0) A.occ[A.ncells + F] = 0u;
    if (A.write_trace) { A.tcnt[F] = 0u; A.mask[F] = 0u; }
    return;
  }
  real cen[3] = {0, 0, 0};
#pragma unroll
  for (int a = 0; a < D; ++a) {
    real s;
    if constexpr (std::is_same<P, PF64>::value) s = sum[a]; else s = csum[a].value();
    cen[a] = s / (real)cnt;
  }

  // ---- refine: components within R of the centroid ---------------------------------------------
  // The move is accumulated as displacements e from the centroid: new = cen + sum(w e) / sum(w).
  uint32_t mask = 0;
  double swd = 0, sxd[3] = {0, 0, 0};
  float swf = 0.f, sxf[3] = {0.f, 0.f, 0.f};
  // soft spawn: sum of the components' direction vectors, FP64 (regular ones as count * c_k)
  double csr[3] = {0, 0, 0}, csb[3] = {0, 0, 0};
#pragma unroll 1
  for (int k = 0; k < Q; ++k) {
    int nk = 0;
    int lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};
    real cdk[3] = {0, 0, 0};
#pragma unroll
    for (int a = 0; a < D; ++a) {
      cdk[a] = A.L.template cd_as<real>(k, a);
      const real base = cen[a] - cdk[a];
      lo[a] = (int)floor(base - A.R - A.tiny);
      hi[a] = (int)floor(base + A.R + A.tiny);
    }
    const real bxr = cen[0] - cdk[0];
    // window rows (sz, sy) in order, each one x range as runs of consecutive cells (see k_gather);
    // 2D FP32: the first item of each cell, then (when a window cell holds more) the others
    bool more = false;
#pragma unroll 1
    for (int pass = 0; pass <= (int)(kFirstItemsFirst<P, D> && more); ++pass)
#pragma unroll 1
    for (int sz = lo[2]; sz <= hi[2]; ++sz)
#pragma unroll 1
      for (int sy = lo[1]; sy <= hi[1]; ++sy) {
        const real cy = canon_c<real>(sy, cdk[1], cen[1]);
        const real cz = D == 3 ? canon_c<real>(sz, cdk[2], cen[2]) : (real)0;
        const real ly = axis_lb<real>(cy);
        real lb2 = rn_mul(ly, ly);
        if (D == 3) {
          const real lz = axis_lb<real>(cz);
          lb2 = rn_add(lb2, rn_mul(lz, lz));
        }
        if (lb2 > A.R2) continue;
        const real hw = row_halfwidth2<real>(A.R2, lb2);
        if (hw < (real)0) continue;
        const int lox = max((int)floor(bxr - hw - A.tiny), lo[0]), hix = min((int)floor(bxr + hw + A.tiny), hi[0]);
        if (lox > hix) continue;
        row_runs<D>(I, Fc[0], Fc[1] + sy, Fc[2] + sz, lox, hix, [&](uint32_t g0, uint32_t g1, int shift) {
          const uint32_t m1 = A.a.start[g1 + 1];
          [[maybe_unused]] real prev = (real)-1;  // cell column of the previous item of the run
          for (uint32_t m = A.a.start[g0]; m < m1; ++m) {
            if (!kFirstItemsFirst<P, D> && A.any_obstacle && ((A.bmask[m] >> k) & 1u)) continue;
            const PackItem<real> it = A.a.pk[m];
            if constexpr (kFirstItemsFirst<P, D>) {
              const bool first = it.cx != prev;
              prev = it.cx;
              if (first != (pass == 0)) {
                more = true;
                continue;
              }
              if (A.any_obstacle && ((A.bmask[m] >> k) & 1u)) continue;  // bounced: visited below
            }
            const int sx = (int)it.cx + shift - Fc[0];
            const real c[3] = {canon_c<real>(sx, cdk[0], cen[0]), cy, cz};
            const real o[3] = {it.x, it.y, it.z};
            real e[3];
            if (canon_d2<D, real>(o, c, e) <= A.R2) {
              mask |= 1u << k;
              ++nk;
              const real w = A.want_wexp ? A.wexp[(int64_t)k * A.mcap + m] : exp(fstar_at<Q, D, P>(A, m, k));
              if constexpr (std::is_same<P, PF64>::value) {
                // separate rounding of product and sum (no FMA), in loop order: the oracle
                // reproduces this sum bit for bit
                swd = __dadd_rn(swd, w);
#pragma unroll
                for (int a = 0; a < D; ++a) sxd[a] = __dadd_rn(sxd[a], __dmul_rn(w, e[a]));
              } else {
                swf += w;
#pragma unroll
                for (int a = 0; a < D; ++a) sxf[a] = fmaf(w, e[a], sxf[a]);
              }
            }
          }
        });
      }
    if (A.kappa_soft > 0 && nk > 0) {
#pragma unroll
      for (int a = 0; a < D; ++a) csr[a] = __dadd_rn(csr[a], __dmul_rn((double)nk, A.L.c[k][a]));
    }
  }
  if (A.any_obstacle && I.has_obs && sphere_dist2<D, real>(I, Fc, cen) < I.reach2) {
    // bounced components (displacement 0, opposite label): window order, then moment, then slot
    int lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};
#pragma unroll
    for (int a = 0; a < D; ++a) {
      lo[a] = (int)floor(cen[a] - A.R - A.tiny);
      hi[a] = (int)floor(cen[a] + A.R + A.tiny);
    }
#pragma unroll 1
    for (int sz = lo[2]; sz <= hi[2]; ++sz)
#pragma unroll 1
      for (int sy = lo[1]; sy <= hi[1]; ++sy)
#pragma unroll 1
        for (int sx = lo[0]; sx <= hi[0]; ++sx) {
          const int dS[3] = {sx, sy, sz};
          real c[3] = {0, 0, 0};
#pragma unroll
          for (int a = 0; a < D; ++a) c[a] = canon_c<real>(dS[a], (real)0, cen[a]);
          if (cell_d2_lower<D, real>(c) > A.R2) continue;
          uint32_t Sg;
          if (!cell_at<D>(I, Fc[0] + sx, Fc[1] + sy, Fc[2] + sz, &Sg)) continue;
          for (uint32_t m = A.a.start[Sg], m1 = A.a.start[Sg + 1]; m < m1; ++m) {
            const uint32_t bits = A.bmask[m];
            if (!bits) continue;
            real o[3] = {0, 0, 0}, e[3];
#pragma unroll
            for (int a = 0; a < D; ++a) o[a] = A.a.off[(int64_t)a * A.mcap + m];
            if (canon_d2<D, real>(o, c, e) > A.R2) continue;
#pragma unroll 1
            for (int k = 1; k < Q; ++k) {
              if (!((bits >> k) & 1u)) continue;
              mask |= 1u << A.L.opp[k];
              if (A.kappa_soft > 0) {
#pragma unroll
                for (int a = 0; a < D; ++a) csb[a] = __dadd_rn(csb[a], A.L.c[A.L.opp[k]][a]);
              }
              const real w = A.want_wexp ? A.wexp[(int64_t)k * A.mcap + m] : exp(fstar_at<Q, D, P>(A, m, k));
              if constexpr (std::is_same<P, PF64>::value) {
                swd = __dadd_rn(swd, w);
#pragma unroll
                for (int a = 0; a < D; ++a) sxd[a] = __dadd_rn(sxd[a], __dmul_rn(w, e[a]));
              } else {
                swf += w;
#pragma unroll
                for (int a = 0; a < D; ++a) sxf[a] = fmaf(w, e[a], sxf[a]);
              }
            }
          }
        }
  }
  const int kappa = __popc(mask);
  real np[3] = {0, 0, 0};
#pragma unroll
  for (int a = 0; a < D; ++a) {
    if (kappa <= A.kappa_hard) {
      np[a] = cen[a];
    } else if constexpr (std::is_same<P, PF64>::value) {
      np[a] = __dadd_rn(cen[a], __ddiv_rn(sxd[a], swd));
    } else {
      np[a] = cen[a] + sxf[a] / swf;
    }
  }
  bool finite = true;
#pragma unroll
  for (int a = 0; a < D; ++a) finite &= isfinite(np[a]) && fabs(np[a]) < (real)64;
  if (!finite) {  // exp(f) underflowed to zero weight: keep the centroid and report it
    atomicOr(A.status, ST_NONFINITE);
#pragma unroll
    for (int a = 0; a < D; ++a) np[a] = cen[a];
  }
  int sh[3] = {0, 0, 0};
  real off[3] = {0, 0, 0};
#pragma unroll
  for (int a = 0; a < D; ++a) {
    real fl = floor(np[a]);
    sh[a] = (int)fl;
    off[a] = np[a] - fl;
    if (off[a] >= (real)1) {
      off[a] = 0;
      sh[a] += 1;
    }
  }
  uint32_t G;
  bool inside = cell_at<D>(I, Fc[0] + sh[0], Fc[1] + sh[1], Fc[2] + sh[2], &G);
  if (!inside) atomicOr(A.status, ST_OUT_OF_BOX);
  if (inside && I.has_obs) {  // a point inside the solid is removed
    int Gc[3];
    decode_cell<D>(I, G, Gc);
    double o[3] = {0, 0, 0};
#pragma unroll
    for (int a = 0; a < D; ++a) o[a] = (double)off[a];
    if (inside_sphere<D>(I, Gc, o)) inside = false;
  }
  A.occ[F] = inside ? 1u : 0u;
  A.fkey[F] = inside ? G : 0xffffffffu;
#pragma unroll
  for (int a = 0; a < D; ++a) A.foff[(int64_t)a * A.ncells + F] = off[a];
  if (A.kappa_soft > 0) {
    // soft-outer spawn (direbm/reference/simulator.py:126-166): the new CP sits soft_off cells from
    // the centroid (the CP before its move) along the normalised direction sum; every operation
    // in FP64 with one rounding each, the offset then rounded to the working precision
    bool spawned = false;
    uint32_t G2 = 0xffffffffu;
    real off2[3] = {0, 0, 0};
    if (kappa > A.kappa_hard && kappa <= A.kappa_soft) {
      double cs[3] = {0, 0, 0};
#pragma unroll
      for (int a = 0; a < D; ++a) cs[a] = __dadd_rn(csr[a], csb[a]);
      double n2 = __dmul_rn(cs[0], cs[0]);
#pragma unroll
      for (int a = 1; a < D; ++a) n2 = __dadd_rn(n2, __dmul_rn(cs[a], cs[a]));
      const double nrm = __dsqrt_rn(n2);
      if (nrm > 1e-8) {
        int sh2[3] = {0, 0, 0};
#pragma unroll
        for (int a = 0; a < D; ++a) {
          const double sp = __dadd_rn((double)cen[a], __dmul_rn(__ddiv_rn(cs[a], nrm), A.soft_off));
          const double fl = floor(sp);
          real o = (real)(sp - fl);
          sh2[a] = (int)fl;
          if (o >= (real)1) {
            o = 0;
            sh2[a] += 1;
          }
          off2[a] = o;
        }
        spawned = cell_at<D>(I, Fc[0] + sh2[0], Fc[1] + sh2[1], Fc[2] + sh2[2], &G2);
        if (!spawned) atomicOr(A.status, ST_OUT_OF_BOX);
        if (spawned && I.has_obs) {
          int Gc[3];
          decode_cell<D>(I, G2, Gc);
          double o[3] = {0, 0, 0};
#pragma unroll
          for (int a = 0; a < D; ++a) o[a] = (double)off2[a];
          if (inside_sphere<D>(I, Gc, o)) spawned = false;
        }
      }
    }
    A.occ[A.ncells + F] = spawned ? 1u : 0u;
    A.fkey[A.ncells + F] = spawned ? G2 : 0xffffffffu;
#pragma unroll
    for (int a = 0; a < D; ++a) A.foff2[(int64_t)a * A.ncells + F] = off2[a];
  }
  if (A.write_trace) {
    A.tcnt[F] = cnt;
    A.mask[F] = mask;
#pragma unroll
    for (int a = 0; a < D; ++a) A.cen[(int64_t)a * A.ncells + F] = cen[a];
  }
}

// The untiled window kernels take one brick of cells per block (thread t <-> cell t of the brick):
// a block's windows then cover a compact region that stays in L1, where consecutive points in cell
// order would span a long strip of rows.
template <int Q, int D, class P>
__global__ void __launch_bounds__(256, thin_min_blocks<P>()) k_thin_refine(const __grid_constant__ Args<Q, D, P> A,
                                                                           const Brick* __restrict__ bricks,
                                                                           int nbricks, BrickGeo bg) {
  for (int bi = blockIdx.x; bi < nbricks; bi += gridDim.x) {
    const Brick B = bricks[bi];
    const InstK I = A.inst[B.inst];
    uint32_t F;
    if (brick_cell<D>(B, I, bg, threadIdx.x, &F)) thin_refine_cell<Q, D, P>(A, F, I);
  }
}

// Packed copy (offsets + cell x coordinate) of a state for the untiled window kernels.
template <int Q, int D, class P>
__global__ void __launch_bounds__(256) k_pack(const __grid_constant__ Args<Q, D, P> A, StateP<P> S, int64_t stride,
                                              const uint32_t* __restrict__ d_n) {
  using real = typename P::real;
  const uint32_t n = *d_n;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const uint32_t g = S.cell[i];
    const InstK I = A.inst[find_instance(A.inst_base, A.n_inst, g)];
    PackItem<real> it;
    it.x = S.off[i];
    it.y = D > 1 ? S.off[stride + i] : (real)0;
    it.z = D > 2 ? S.off[2 * stride + i] : (real)0;
    it.cx = (real)((g - I.base) % (uint32_t)I.dims[0]);
    S.pk[i] = it;
  }
}

// Copy one device word to a mapped host word (and optionally clear it).
__global__ void k_read_word(uint32_t* __restrict__ src, int clear, uint32_t* __restrict__ dst) {
  if (threadIdx.x == 0) {
    *dst = *src;
    if (clear) *src = 0u;
  }
}

// Sorted pairs -> next state's cells and offsets.
template <int Q, int D, class P>
__global__ void __launch_bounds__(256) k_finalize(const __grid_constant__ Args<Q, D, P> A) {
  const uint32_t Pn = *A.d_P;
  for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < Pn; j += gridDim.x * blockDim.x) {
    const uint32_t src = A.svals[j];
    A.b.cell[j] = A.skeys[j];
#pragma unroll
    for (int a = 0; a < D; ++a)
      A.b.off[(int64_t)a * A.ccap + j] = src < A.ncells ? A.foff[(int64_t)a * A.ncells + src]
                                                        : A.foff2[(int64_t)a * A.ncells + (src - A.ncells)];
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) *A.b.count = Pn;
}

// ---- control points in cell order without a sort (2D, small move bound) ---------------------------
// A refined control point lands within +-H cells of its thinning cell on each axis (H = floor(R) + 1:
// centroid in [0, 1], move at most R).  So the stable order by (final cell, thinning cell) that a
// sort would give follows from per-cell counts and, for each point, the number of earlier thinning
// cells of its final cell's (2H+1)^2 neighbourhood that land in the same cell.

// count[G] += 1 per control point (integer atomics: order-independent).
template <int Q, int D, class P>
__global__ void __launch_bounds__(256) k_place_count(const __grid_constant__ Args<Q, D, P> A, uint32_t* __restrict__ cnt) {
  for (uint32_t F = blockIdx.x * blockDim.x + threadIdx.x; F < A.ncells; F += gridDim.x * blockDim.x)
    if (A.occ[F]) atomicAdd(cnt + A.fkey[F], 1u);
}

// Slot of each control point = start[G] + its rank among the thinning cells F' < F that land in G;
// writes the next state's cell and offsets and the (key, thinning cell) pairs a sort would leave.
template <int Q, int D, class P>
__global__ void __launch_bounds__(256) k_place(const __grid_constant__ Args<Q, D, P> A, int H,
                                               uint32_t* __restrict__ keys, uint32_t* __restrict__ vals) {
  for (uint32_t F = blockIdx.x * blockDim.x + threadIdx.x; F < A.ncells; F += gridDim.x * blockDim.x) {
    if (!A.occ[F]) continue;
    const uint32_t G = A.fkey[F];
    const uint32_t g0 = A.b.start[G], ng = A.b.start[G + 1] - g0;
    uint32_t rank = 0;
    if (ng != 1u) {  // a cell with one control point needs no rank (the common case: one per cell)
      const InstK I = A.inst[find_instance(A.inst_base, A.n_inst, G)];
      int Gc[3];
      decode_cell<D>(I, G, Gc);
      uint32_t all = 0;
      for (int dy = -H; dy <= H; ++dy)
        for (int dx = -H; dx <= H; ++dx) {
          uint32_t Fp;
          if (!cell_at<D>(I, Gc[0] + dx, Gc[1] + dy, 0, &Fp)) continue;
          const uint32_t hit = A.fkey[Fp] == G ? 1u : 0u;  // fkey is all ones where no control point was made
          all += hit;
          rank += Fp < F ? hit : 0u;
        }
      // every control point of G comes from this neighbourhood (the move bound): check it
      if (all != ng) atomicOr(A.status, ST_INTERNAL);
    }
    const uint32_t j = g0 + rank;
    keys[j] = G;
    vals[j] = F;
    A.b.cell[j] = G;
#pragma unroll
    for (int a = 0; a < D; ++a) A.b.off[(int64_t)a * A.ccap + j] = A.foff[(int64_t)a * A.ncells + F];
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) *A.b.count = A.b.start[A.ncells];
}

// start[c] = number of sorted keys < c, for c in [0, ncells].  Each thread takes 8 consecutive cells:
// one binary search for the first, then a walk along the sorted keys (8x fewer dependent-load
// searches; a thread's walk covers only the keys of its own cells).
constexpr int kCellStartChunk = 8;
__global__ void __launch_bounds__(256) k_cell_start(const uint32_t* __restrict__ keys, const uint32_t* d_n,
                                                    uint32_t ncells, uint32_t* __restrict__ start) {
  const uint32_t n = *d_n;
  const uint64_t nchunks = ((uint64_t)ncells + kCellStartChunk) / kCellStartChunk;  // cells 0..ncells
  for (uint64_t ch = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; ch < nchunks;
       ch += (uint64_t)gridDim.x * blockDim.x) {
    const uint32_t c0 = (uint32_t)(ch * kCellStartChunk);
    uint32_t lo = 0, hi = n;
    while (lo < hi) {
      const uint32_t mid = (lo + hi) >> 1;
      if (keys[mid] < c0) lo = mid + 1; else hi = mid;
    }
    uint32_t v[kCellStartChunk];
#pragma unroll
    for (int i = 0; i < kCellStartChunk; ++i) {
      v[i] = lo;  // = number of keys < c0 + i
      while (lo < n && keys[lo] == c0 + (uint32_t)i) ++lo;
    }
    if ((uint64_t)c0 + kCellStartChunk <= (uint64_t)ncells + 1) {
      uint4* dst = reinterpret_cast<uint4*>(start + c0);  // 32-byte aligned: c0 is a multiple of 8
      dst[0] = make_uint4(v[0], v[1], v[2], v[3]);
      dst[1] = make_uint4(v[4], v[5], v[6], v[7]);
    } else {
      for (int i = 0; (uint64_t)c0 + i <= ncells; ++i) start[c0 + i] = v[i];
    }
  }
}

static void launch_cell_start(const uint32_t* keys, const uint32_t* d_n, uint32_t ncells, uint32_t* start,
                              cudaStream_t s) {
  const int64_t nchunks = ((int64_t)ncells + kCellStartChunk) / kCellStartChunk;
  k_cell_start<<<std::min<unsigned>(div_up(nchunks, 256), (unsigned)sm_count() * 16), 256, 0, s>>>(keys, d_n, ncells,
                                                                                                  start);
}

// sw of component (m, k), m a moment in cell g of instance I.
template <int Q, int D, class P>
__device__ __forceinline__ void weights_one(const Args<Q, D, P>& A, const uint32_t m, const int k, const uint32_t g,
                                            const InstK& I) {
  using real = typename P::real;
  int Sc[3];
  decode_cell<D>(I, g, Sc);
  real o[3] = {0, 0, 0}, cdk[3] = {0, 0, 0};
  int lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};
  const bool bounced = A.any_obstacle && ((A.bmask[m] >> k) & 1u);  // stays at the moment
#pragma unroll
  for (int a = 0; a < D; ++a) {
    o[a] = A.a.off[(int64_t)a * A.mcap + m];
    cdk[a] = bounced ? (real)0 : A.L.template cd_as<real>(k, a);
    const real t = rn_add(o[a], cdk[a]);
    lo[a] = (int)floor(t - A.R - A.tiny);
    hi[a] = (int)floor(t + A.R + A.tiny);
  }
  double swd = 0;
  CSum sws;
  // window rows (gz, gy) in order; per row one x range narrowed by the row's smallest |e_y|, |e_z|,
  // visited as runs of consecutive cells (the items of a run are contiguous, in cell order); the
  // first item of each cell, then (when a window cell holds more) the others
  const real tx = rn_add(o[0], cdk[0]);
  bool more = false;
#pragma unroll 1
  for (int pass = 0; pass <= (int)(kFirstItemsFirst<P, D> && more); ++pass)
#pragma unroll 1
  for (int gz = lo[2]; gz <= hi[2]; ++gz)
#pragma unroll 1
    for (int gy = lo[1]; gy <= hi[1]; ++gy) {
      // per axis: base = float(dS) + cd with dS = -dG; candidates have e in [fl(o + fl(base - 1)),
      // fl(o + base)] (control-point offsets lie in [0, 1))
      real base[3] = {0, 0, 0};
      const int dG[3] = {0, gy, gz};
      real lb2 = 0;
#pragma unroll
      for (int a = 1; a < D; ++a) {
        base[a] = rn_add((real)(-dG[a]), cdk[a]);
        const real elo = rn_add(o[a], rn_sub(base[a], (real)1)), ehi = rn_add(o[a], base[a]);
        const real lb = elo > (real)0 ? elo : (ehi < (real)0 ? -ehi : (real)0);
        lb2 = a == 1 ? rn_mul(lb, lb) : rn_add(lb2, rn_mul(lb, lb));
      }
      if (lb2 > A.R2) continue;
      const real hw = row_halfwidth2<real>(A.R2, lb2);
      if (hw < (real)0) continue;
      const int lox = max((int)floor(tx - hw - A.tiny), lo[0]), hix = min((int)floor(tx + hw + A.tiny), hi[0]);
      if (lox > hix) continue;
      row_runs<D>(I, Sc[0], Sc[1] + gy, Sc[2] + gz, lox, hix, [&](uint32_t g0, uint32_t g1, int shift) {
        const uint32_t c1 = A.b.start[g1 + 1];
        [[maybe_unused]] real prev = (real)-1;  // cell column of the previous item of the run
        for (uint32_t c = A.b.start[g0]; c < c1; ++c) {
          const PackItem<real> it = A.b.pk[c];
          if constexpr (kFirstItemsFirst<P, D>) {
            const bool first = it.cx != prev;
            prev = it.cx;
            if (first != (pass == 0)) {
              more = true;
              continue;
            }
          }
          const int gx = (int)it.cx + shift - Sc[0];
          const real cc[3] = {rn_sub(rn_add((real)(-gx), cdk[0]), it.x), rn_sub(base[1], it.y),
                              D == 3 ? rn_sub(base[2], it.z) : (real)0};
          real e[3];
          const real d2 = canon_d2<D, real>(o, cc, e);
          if (d2 <= A.R2) {
            const real d = rn_sqrt(d2);
            if constexpr (std::is_same<P, PF64>::value) swd += A.R - d; else sws.add(A.R - d);
          }
        }
      });
    }
  real sw;
  if constexpr (std::is_same<P, PF64>::value) sw = swd; else sw = sws.value();
  const real inv = sw > (real)0 ? (real)1 / sw : (real)0;  // stored inverted
  const int64_t i = (int64_t)k * A.mcap + m;
  A.sw[i] = inv;
  if constexpr (std::is_same<P, PF64>::value) A.kv[i] = KV<real>{inv, A.a.f64[i]};
  else A.kv[i] = KV<real>{inv, A.a.dev[i]};
}

// FP32: six resident blocks per SM (the gather waits on loads and needs the warps); FP64 keeps its
// registers (forcing the same bound spills the double accumulators).
template <class P>
constexpr int gather_min_blocks() { return std::is_same<P, PF64>::value ? 1 : 6; }

// Resampled f_k of control point j, in cell G of instance I.
template <int Q, int D, class P>
__device__ __forceinline__ void gather_one(const Args<Q, D, P>& A, const uint32_t j, const int k, const uint32_t G,
                                           const InstK& I) {
  using real = typename P::real;
  int Gc[3];
  decode_cell<D>(I, G, Gc);
  real p[3] = {0, 0, 0}, cdk[3] = {0, 0, 0};
  int lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};
#pragma unroll
  for (int a = 0; a < D; ++a) {
    p[a] = A.b.off[(int64_t)a * A.ccap + j];
    cdk[a] = A.L.template cd_as<real>(k, a);
    const real base = p[a] - cdk[a];
    lo[a] = (int)floor(base - A.R - A.tiny);
    hi[a] = (int)floor(base + A.R + A.tiny);
  }
  double acc = 0;
  CSum sa;
  float sb = 0.f;  // deviation part: small, plain FMA accumulation suffices
  const real bxr = p[0] - cdk[0];
  // window rows (sz, sy) in order; per row one x range narrowed by the row's smallest |e_y|, |e_z|,
  // visited as runs of consecutive cells (the items of a run are contiguous, in cell order); the
  // first item of each cell, then (when a window cell holds more) the others (2D FP32)
  bool more = false;
#pragma unroll 1
  for (int pass = 0; pass <= (int)(kFirstItemsFirst<P, D> && more); ++pass)
#pragma unroll 1
  for (int sz = lo[2]; sz <= hi[2]; ++sz)
#pragma unroll 1
    for (int sy = lo[1]; sy <= hi[1]; ++sy) {
      const real cy = canon_c<real>(sy, cdk[1], p[1]);
      const real cz = D == 3 ? canon_c<real>(sz, cdk[2], p[2]) : (real)0;
      const real ly = axis_lb<real>(cy);
      real lb2 = rn_mul(ly, ly);
      if (D == 3) {
        const real lz = axis_lb<real>(cz);
        lb2 = rn_add(lb2, rn_mul(lz, lz));
      }
      if (lb2 > A.R2) continue;
      const real hw = row_halfwidth2<real>(A.R2, lb2);
      if (hw < (real)0) continue;
      const int lox = max((int)floor(bxr - hw - A.tiny), lo[0]), hix = min((int)floor(bxr + hw + A.tiny), hi[0]);
      if (lox > hix) continue;
      row_runs<D>(I, Gc[0], Gc[1] + sy, Gc[2] + sz, lox, hix, [&](uint32_t g0, uint32_t g1, int shift) {
        const uint32_t m1 = A.a.start[g1 + 1];
        [[maybe_unused]] real prev = (real)-1;  // cell column of the previous item of the run
        for (uint32_t m = A.a.start[g0]; m < m1; ++m) {
          if (!kFirstItemsFirst<P, D> && A.any_obstacle && ((A.bmask[m] >> k) & 1u)) continue;
          const PackItem<real> it = A.a.pk[m];
          if constexpr (kFirstItemsFirst<P, D>) {
            const bool first = it.cx != prev;
            prev = it.cx;
            if (first != (pass == 0)) {
              more = true;
              continue;
            }
            if (A.any_obstacle && ((A.bmask[m] >> k) & 1u)) continue;  // bounced: label opp[k]
          }
          const int sx = (int)it.cx + shift - Gc[0];
          const real c[3] = {canon_c<real>(sx, cdk[0], p[0]), cy, cz};
          const real o[3] = {it.x, it.y, it.z};
          real e[3];
          const real d2 = canon_d2<D, real>(o, c, e);
          if (d2 <= A.R2) {
            const KV<real> kv = A.kv[(int64_t)k * A.mcap + m];
            if (kv.inv > (real)0) {
              const real wgt = (A.R - rn_sqrt(d2)) * kv.inv;
              if constexpr (std::is_same<P, PF64>::value) {
                acc += wgt * kv.f;
              } else {
                sa.add_prod(wgt, A.a.rho[m]);
                sb = __fmaf_rn(wgt, kv.f, sb);
              }
            }
          }
        }
      });
    }
  if (A.any_obstacle && k > 0 && I.has_obs && sphere_dist2<D, real>(I, Gc, p) < I.reach2) {
    // components of slot kb = opp[k] that bounced carry label k and sit at their moment's offset
    const int kb = A.L.opp[k];
    int blo[3] = {0, 0, 0}, bhi[3] = {0, 0, 0};
#pragma unroll
    for (int a = 0; a < D; ++a) {
      blo[a] = (int)floor(p[a] - A.R - A.tiny);
      bhi[a] = (int)floor(p[a] + A.R + A.tiny);
    }
#pragma unroll 1
    for (int sz = blo[2]; sz <= bhi[2]; ++sz)
#pragma unroll 1
      for (int sy = blo[1]; sy <= bhi[1]; ++sy)
#pragma unroll 1
        for (int sx = blo[0]; sx <= bhi[0]; ++sx) {
          const int dS[3] = {sx, sy, sz};
          real c[3] = {0, 0, 0};
#pragma unroll
          for (int a = 0; a < D; ++a) c[a] = canon_c<real>(dS[a], (real)0, p[a]);
          if (cell_d2_lower<D, real>(c) > A.R2) continue;
          uint32_t Sg;
          if (!cell_at<D>(I, Gc[0] + sx, Gc[1] + sy, Gc[2] + sz, &Sg)) continue;
          for (uint32_t m = A.a.start[Sg], m1 = A.a.start[Sg + 1]; m < m1; ++m) {
            if (!((A.bmask[m] >> kb) & 1u)) continue;
            real o[3] = {0, 0, 0}, e[3];
#pragma unroll
            for (int a = 0; a < D; ++a) o[a] = A.a.off[(int64_t)a * A.mcap + m];
            const real d2 = canon_d2<D, real>(o, c, e);
            if (d2 > A.R2) continue;
            const KV<real> kv = A.kv[(int64_t)kb * A.mcap + m];
            if (kv.inv > (real)0) {
              const real wgt = (A.R - rn_sqrt(d2)) * kv.inv;
              if constexpr (std::is_same<P, PF64>::value) {
                acc += wgt * kv.f;
              } else {
                sa.add_prod(wgt, A.a.rho[m]);
                sb = __fmaf_rn(wgt, kv.f, sb);
              }
            }
          }
        }
  }
  bool empty;
  if constexpr (std::is_same<P, PF64>::value) {
    A.cpf64[(int64_t)k * A.ccap + j] = acc;
    empty = acc < (double)A.eps;
  } else {
    // F = W_k * A + B in double-float
    DF Ad = df_norm(sa.hi, sa.lo);
    DF Bd = DF{sb, 0.f};
    DF Fv = df_add(df_mul(DF{A.L.wf[k], A.L.wlo[k]}, Ad), Bd);
    A.cpfhi[(int64_t)k * A.ccap + j] = Fv.hi;
    A.cpflo[(int64_t)k * A.ccap + j] = Fv.lo;
    empty = Fv.hi < A.eps;
  }
  if (empty) atomicOr(A.emask + j, 1u << k);
}

template <int Q, int D, class P>
__global__ void __launch_bounds__(256, gather_min_blocks<P>()) k_weights(const __grid_constant__ Args<Q, D, P> A,
                                                                         const Brick* __restrict__ bricks, int nbricks,
                                                                         BrickGeo bg) {
  const int k = blockIdx.y;
  for (int bi = blockIdx.x; bi < nbricks; bi += gridDim.x) {
    const Brick B = bricks[bi];
    const InstK I = A.inst[B.inst];
    uint32_t F;
    if (!brick_cell<D>(B, I, bg, threadIdx.x, &F)) continue;
    for (uint32_t m = A.a.start[F], m1 = A.a.start[F + 1]; m < m1; ++m) weights_one<Q, D, P>(A, m, k, F, I);
  }
}

template <int Q, int D, class P>
__global__ void __launch_bounds__(256, gather_min_blocks<P>()) k_gather(const __grid_constant__ Args<Q, D, P> A,
                                                                        const Brick* __restrict__ bricks, int nbricks,
                                                                        BrickGeo bg) {
  const int k = blockIdx.y;
  for (int bi = blockIdx.x; bi < nbricks; bi += gridDim.x) {
    const Brick B = bricks[bi];
    const InstK I = A.inst[B.inst];
    uint32_t F;
    if (!brick_cell<D>(B, I, bg, threadIdx.x, &F)) continue;
    for (uint32_t j = A.b.start[F], j1 = A.b.start[F + 1]; j < j1; ++j) gather_one<Q, D, P>(A, j, k, F, I);
  }
}

template <int Q, int D, class P>
__global__ void __launch_bounds__(256) k_emit(const __grid_constant__ Args<Q, D, P> A) {
  using real = typename P::real;
  const uint32_t Pn = *A.d_P;
  for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < Pn; j += gridDim.x * blockDim.x) {
    const uint32_t em = A.emask[j];
    const uint32_t G = A.b.cell[j];
    const int b = find_instance(A.inst_base, A.n_inst, G);
    const InstK I = A.inst[b];
    double swd[Q];
    float swf[Q];
#pragma unroll
    for (int k = 0; k < Q; ++k) { swd[k] = 0; swf[k] = 0.f; }
    if (em) {
      int Gc[3];
      decode_cell<D>(I, G, Gc);
      real p[3] = {0, 0, 0};
      int lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};
#pragma unroll
      for (int a = 0; a < D; ++a) {
        p[a] = A.b.off[(int64_t)a * A.ccap + j];
        lo[a] = (int)floor(p[a] - A.R - A.tiny);
        hi[a] = (int)floor(p[a] + A.R + A.tiny);
      }
      CSum sws[Q];
#pragma unroll 1
      for (int gz = lo[2]; gz <= hi[2]; ++gz)
#pragma unroll 1
        for (int gy = lo[1]; gy <= hi[1]; ++gy)
#pragma unroll 1
          for (int gx = lo[0]; gx <= hi[0]; ++gx) {
            const int dS[3] = {gx, gy, gz};
            real cc[3] = {0, 0, 0};
#pragma unroll
            for (int a = 0; a < D; ++a) cc[a] = canon_c<real>(dS[a], (real)0, p[a]);
            if (cell_d2_lower<D, real>(cc) > A.R2) continue;
            uint32_t Hg;
            if (!cell_at<D>(I, Gc[0] + gx, Gc[1] + gy, Gc[2] + gz, &Hg)) continue;
            const uint32_t c0 = A.b.start[Hg], c1 = A.b.start[Hg + 1];
            for (uint32_t c = c0; c < c1; ++c) {
              const uint32_t both = A.emask[c] & em;
              if (!both) continue;
              real o[3] = {0, 0, 0}, e[3];
#pragma unroll
              for (int a = 0; a < D; ++a) o[a] = A.b.off[(int64_t)a * A.ccap + c];
              const real d2 = canon_d2<D, real>(o, cc, e);
              if (d2 <= A.R2) {
                const real w = A.R - rn_sqrt(d2);
#pragma unroll
                for (int k = 0; k < Q; ++k) {
                  if ((both >> k) & 1u) {
                    if constexpr (std::is_same<P, PF64>::value) swd[k] += w; else sws[k].add(w);
                  }
                }
              }
            }
          }
      if constexpr (!std::is_same<P, PF64>::value) {
#pragma unroll
        for (int k = 0; k < Q; ++k) swf[k] = sws[k].value();
      }
    }
    if constexpr (std::is_same<P, PF64>::value) {
#pragma unroll
      for (int k = 0; k < Q; ++k) {
        double v = A.cpf64[(int64_t)k * A.ccap + j];
        if (((em >> k) & 1u) && swd[k] > 0.0) v = ((double)A.R / swd[k]) * (I.rho_rest * A.L.w[k]);
        A.b.f64[(int64_t)k * A.ccap + j] = v;
      }
    } else {
      DF Fk[Q];
      DF rho = {0.f, 0.f};
#pragma unroll
      for (int k = 0; k < Q; ++k) {
        if (((em >> k) & 1u) && swf[k] > 0.f) {
          const float s = (A.R / swf[k]) * (float)I.rho_rest;
          Fk[k] = df_mul(DF{A.L.wf[k], A.L.wlo[k]}, DF{s, 0.f});
        } else {
          Fk[k] = DF{A.cpfhi[(int64_t)k * A.ccap + j], A.cpflo[(int64_t)k * A.ccap + j]};
        }
        rho = df_add(rho, Fk[k]);
      }
      A.b.rho[j] = df_float(rho);
#pragma unroll
      for (int k = 0; k < Q; ++k) {
        DF dv = df_add(Fk[k], df_neg(df_mul(DF{A.L.wf[k], A.L.wlo[k]}, rho)));
        A.b.dev[(int64_t)k * A.ccap + j] = df_float(dv);
      }
    }
  }
}

// ---- import / export ------------------------------------------------------------------------

// T: the caller's element type of positions and f (double, or float for the float32 interface).
// GB300 issues FP64 arithmetic (and double<->float conversions) at a small fraction of the FP32
// rate, so the float32 interface runs in float arithmetic where that gives the same bits or, for
// the FP32DEV split of f, a stated rounding:
//   - positions, cell a power of two (cell_f != 0): s = x * (1/cell) and its fraction are exact
//     in float, so cell and offset are bitwise those of the float64 path;
//   - FP32DEV f: rho = compensated float sum of f (TwoSum per term), dev_k = f_k - rho W_k with
//     rho wf_k split exactly by fmaf and W_k = wf_k + wlo_k (double-float); the float64 path
//     rounds the same residual from a float64 sum, so the two agree to about an ulp of dev.
// Cell key (0xffffffff when the moment lies outside its box, with ST_BAD_INPUT raised) and
// in-cell offsets of input moment i.
template <int Q, int D, class P, class T>
__device__ __forceinline__ uint32_t import_key(const Args<Q, D, P>& A, const int32_t* __restrict__ inst_of,
                                               const T* __restrict__ pos, int64_t i, double cell, float inv_cell_f,
                                               typename P::real (&o)[D]) {
  using real = typename P::real;
  constexpr bool kFloatIn = std::is_same<T, float>::value;
  const int b = inst_of[i];
  uint32_t key = 0xffffffffu;
#pragma unroll
  for (int a = 0; a < D; ++a) o[a] = 0;
  if (b >= 0 && b < A.n_inst) {
    const InstK I = A.inst[b];
    int c[3] = {0, 0, 0};
    bool ok = true;
#pragma unroll
    for (int a = 0; a < D; ++a) {
      real oa;
      long long fl_i;
      if (kFloatIn && std::is_same<real, float>::value && inv_cell_f != 0.f) {
        // exact: power-of-two scaling; a float minus its floor is the correctly rounded
        // difference, which the float64 path also rounds once (the difference of two floats
        // within 2^29 of each other is exact in double, and below that both round to 1)
        const float sf = __fmul_rn((float)pos[i * D + a], inv_cell_f);
        const float flf = floorf(sf);
        oa = (real)__fsub_rn(sf, flf);
        fl_i = (long long)flf;
      } else {
        const double sd = (double)pos[i * D + a] / cell;
        const double fl = floor(sd);
        oa = (real)(sd - fl);
        fl_i = (long long)fl;
      }
      const real one_below = std::is_same<real, float>::value ? (real)0.99999994f : (real)0.99999999999999989;
      o[a] = oa > one_below ? one_below : oa;
      long long x = fl_i - I.origin[a];
      const long long n = I.dims[a];
      if (I.periodic) {
        if (x < 0 || x >= n) {
          x %= n;
          if (x < 0) x += n;
        }
      } else {
        ok &= (x >= 0 && x < n);
      }
      c[a] = (int)x;
    }
    uint32_t g;
    if (ok && cell_at<D>(I, c[0], c[1], c[2], &g)) key = g;
  }
  if (key == 0xffffffffu) atomicOr(A.status, ST_BAD_INPUT);
  return key;
}

// State slot j <- distributions of input moment i (FP64: f; FP32DEV: rho and dev).
template <int Q, int D, class P, class T>
__device__ __forceinline__ void import_f(const Args<Q, D, P>& A, const T* __restrict__ fin, int64_t i, int64_t j) {
  if constexpr (std::is_same<P, PF64>::value) {
#pragma unroll
    for (int k = 0; k < Q; ++k) A.a.f64[(int64_t)k * A.mcap + j] = (double)fin[i * Q + k];
  } else if constexpr (std::is_same<T, float>::value) {
    float fk[Q];
#pragma unroll
    for (int k = 0; k < Q; ++k) fk[k] = fin[i * Q + k];
    float s = fk[0], err = 0.f;
#pragma unroll
    for (int k = 1; k < Q; ++k) {
      const DF t = df_two_sum(s, fk[k]);
      s = t.hi;
      err = __fadd_rn(err, t.lo);
    }
    const float rho = __fadd_rn(s, err);
    A.a.rho[j] = rho;
#pragma unroll
    for (int k = 0; k < Q; ++k) {
      const float p = __fmul_rn(rho, A.L.wf[k]);
      const float e = __fmaf_rn(rho, A.L.wf[k], -p);  // rho wf_k = p + e exactly
      const DF d = df_two_sum(fk[k], -p);             // f_k - p exactly
      A.a.dev[(int64_t)k * A.mcap + j] = __fadd_rn(d.hi, __fsub_rn(d.lo, __fmaf_rn(rho, A.L.wlo[k], e)));
    }
  } else {
    double rho = 0;
#pragma unroll
    for (int k = 0; k < Q; ++k) rho += (double)fin[i * Q + k];
    A.a.rho[j] = (float)rho;
#pragma unroll
    for (int k = 0; k < Q; ++k) A.a.dev[(int64_t)k * A.mcap + j] = (float)((double)fin[i * Q + k] - rho * A.L.w[k]);
  }
}

template <int Q, int D, class P, class T>
__global__ void __launch_bounds__(256) k_import_keys(const __grid_constant__ Args<Q, D, P> A, const int32_t* __restrict__ inst_of,
                                                     const T* __restrict__ pos, int64_t m, double cell, float inv_cell_f,
                                                     uint32_t* __restrict__ keys, uint32_t* __restrict__ vals,
                                                     typename P::real* __restrict__ toff) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < m; i += (int64_t)gridDim.x * blockDim.x) {
    typename P::real o[D];
    keys[i] = import_key<Q, D, P, T>(A, inst_of, pos, i, cell, inv_cell_f, o);
    vals[i] = (uint32_t)i;
#pragma unroll
    for (int a = 0; a < D; ++a) toff[(int64_t)a * m + i] = o[a];
  }
}

template <int Q, int D, class P, class T>
__global__ void __launch_bounds__(256) k_import_gather(const __grid_constant__ Args<Q, D, P> A, const T* __restrict__ fin, int64_t m,
                                                       const uint32_t* __restrict__ keys,
                                                       const uint32_t* __restrict__ vals,
                                                       const typename P::real* __restrict__ toff) {
  for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < m; j += (int64_t)gridDim.x * blockDim.x) {
    const uint32_t i = vals[j];
    A.a.cell[j] = keys[j];
#pragma unroll
    for (int a = 0; a < D; ++a) A.a.off[(int64_t)a * A.mcap + j] = toff[(int64_t)a * m + i];
    import_f<Q, D, P, T>(A, fin, i, j);
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) *A.a.count = (uint32_t)m;
}

// A load given in cell order, in one pass: key, offsets and f of moment j go straight to state
// slot j (order[j] = j records the identity import order); k_check_sorted then checks the order.
template <int Q, int D, class P, class T>
__global__ void __launch_bounds__(256) k_import_presorted(const __grid_constant__ Args<Q, D, P> A,
                                                          const int32_t* __restrict__ inst_of,
                                                          const T* __restrict__ pos, const T* __restrict__ fin,
                                                          int64_t m, double cell, float inv_cell_f,
                                                          uint32_t* __restrict__ order) {
  for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < m; j += (int64_t)gridDim.x * blockDim.x) {
    typename P::real o[D];
    A.a.cell[j] = import_key<Q, D, P, T>(A, inst_of, pos, j, cell, inv_cell_f, o);
    order[j] = (uint32_t)j;
#pragma unroll
    for (int a = 0; a < D; ++a) A.a.off[(int64_t)a * A.mcap + j] = o[a];
    import_f<Q, D, P, T>(A, fin, j, j);
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) *A.a.count = (uint32_t)m;
}

// ST_BAD_INPUT where a key is smaller than its predecessor (a presorted load out of cell order).
__global__ void k_check_sorted(const uint32_t* __restrict__ keys, int64_t m, uint32_t* __restrict__ status) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x + 1; i < m; i += (int64_t)gridDim.x * blockDim.x)
    if (keys[i] < keys[i - 1]) atomicOr(status, ST_BAD_INPUT);
}

// T = float (the float32 interface) in float arithmetic: positions, cell a power of two (cell_f != 0)
// and |cell index| < 2^24, are fl32(index + offset) * cell, the same bits as rounding the float64
// position; FP32DEV f_k = rho W_k + dev_k as double-float (rho wf_k split by fmaf), rounded once to
// float, within an ulp of the rounded float64 value.
// Tiles of kExportTile consecutive moments: every load of a moment is issued before the instance
// search that needs its cell, one search per tile bounds the instances of the whole tile (cells are
// sorted, so the first and last moment bound the rest), and the AoS rows (positions (D), f (Q)) are
// staged in shared memory and stored as contiguous, coalesced runs.
constexpr int kExportTile = 256;

template <int Q, int D, class P, class T>
__global__ void __launch_bounds__(kExportTile) k_export(const __grid_constant__ Args<Q, D, P> A, double cell, float cell_f,
                                                        int32_t* __restrict__ inst_out, T* __restrict__ pos,
                                                        T* __restrict__ fout) {
  using real = typename P::real;
  constexpr bool kFloatOut = std::is_same<T, float>::value;
  constexpr bool kDev = !std::is_same<P, PF64>::value;
  __shared__ T s_pos[kExportTile * D];
  __shared__ T s_f[kExportTile * Q];
  __shared__ int s_b[2];
  const uint32_t M = *A.a.count;
  const int t = threadIdx.x;
  for (uint32_t j0 = blockIdx.x * kExportTile; j0 < M; j0 += gridDim.x * kExportTile) {
    const int n = (int)min((uint32_t)kExportTile, M - j0);
    const uint32_t j = j0 + t;
    const bool act = t < n;
    uint32_t g = 0;
    real o[D];
    float rho = 0.f;
    real fv[Q];  // dev (FP32DEV) or f (FP64)
    if (act) {
      g = A.a.cell[j];
#pragma unroll
      for (int a = 0; a < D; ++a) o[a] = A.a.off[(int64_t)a * A.mcap + j];
      if constexpr (kDev) {
        rho = A.a.rho[j];
#pragma unroll
        for (int k = 0; k < Q; ++k) fv[k] = A.a.dev[(int64_t)k * A.mcap + j];
      } else {
#pragma unroll
        for (int k = 0; k < Q; ++k) fv[k] = A.a.f64[(int64_t)k * A.mcap + j];
      }
    }
    if (t == 0) s_b[0] = find_instance(A.inst_base, A.n_inst, g);
    if (t == n - 1) s_b[1] = find_instance(A.inst_base, A.n_inst, g);
    __syncthreads();
    if (act) {
      int b = s_b[0];
      if (s_b[1] != b) {  // the tile spans instances: search between the two
        int lo = s_b[0], hi = s_b[1] + 1;
        while (hi - lo > 1) {
          const int mid = (lo + hi) >> 1;
          if (__ldg(A.inst_base + mid) <= g) lo = mid; else hi = mid;
        }
        b = lo;
      }
      const InstK I = A.inst[b];
      int c[3];
      decode_cell<D>(I, g, c);
      if (inst_out) inst_out[j] = b;
#pragma unroll
      for (int a = 0; a < D; ++a) {
        const long long ci = (long long)I.origin[a] + c[a];
        T v;
        if (kFloatOut && std::is_same<real, float>::value && cell_f != 0.f && ci > -(1ll << 24) && ci < (1ll << 24))
          v = (T)__fmul_rn(__fadd_rn((float)ci, (float)o[a]), cell_f);
        else
          v = (T)(((double)ci + (double)o[a]) * cell);
        s_pos[t * D + a] = v;
      }
#pragma unroll
      for (int k = 0; k < Q; ++k) {
        T v;
        if constexpr (!kDev) {
          v = (T)fv[k];
        } else if constexpr (kFloatOut) {
          // f_k = rho wf_k + dev_k + rho wlo_k: the large pair summed exactly (they cancel where f_k is
          // small), the small terms added to its error before the one rounding
          const float p = __fmul_rn(rho, A.L.wf[k]);
          const float e = __fmaf_rn(rho, A.L.wf[k], -p);
          const DF h = df_two_sum(p, (float)fv[k]);
          v = __fadd_rn(h.hi, __fadd_rn(h.lo, __fmaf_rn(rho, A.L.wlo[k], e)));
        } else {
          v = (T)((double)rho * A.L.w[k] + (double)fv[k]);
        }
        s_f[t * Q + k] = v;
      }
    }
    __syncthreads();
    if (pos)
      for (int e = t; e < n * D; e += kExportTile) pos[(int64_t)j0 * D + e] = s_pos[e];
    if (fout)
      for (int e = t; e < n * Q; e += kExportTile) fout[(int64_t)j0 * Q + e] = s_f[e];
    __syncthreads();  // s_b, s_pos and s_f are rewritten by the next tile
  }
}

// Per-instance FP64 mass and momentum, one block per instance, fixed reduction order.
template <int Q, int D, class P>
__global__ void __launch_bounds__(256) k_conservation(const __grid_constant__ Args<Q, D, P> A, double* __restrict__ out) {
  const int b = blockIdx.x;
  const InstK I = A.inst[b];
  const uint32_t m0 = A.a.start[I.base];
  const uint32_t m1 = A.a.start[A.inst_base[b + 1]];
  double acc[1 + D];
#pragma unroll
  for (int i = 0; i <= D; ++i) acc[i] = 0;
  for (uint32_t m = m0 + threadIdx.x; m < m1; m += blockDim.x) {
#pragma unroll
    for (int k = 0; k < Q; ++k) {
      double f;
      if constexpr (std::is_same<P, PF64>::value) f = A.a.f64[(int64_t)k * A.mcap + m];
      else f = (double)A.a.rho[m] * A.L.w[k] + (double)A.a.dev[(int64_t)k * A.mcap + m];
      acc[0] += f;
#pragma unroll
      for (int a = 0; a < D; ++a) acc[1 + a] += f * A.L.c[k][a];
    }
  }
  __shared__ double red[256];
#pragma unroll 1
  for (int i = 0; i <= D; ++i) {
    red[threadIdx.x] = acc[i];
    __syncthreads();
    for (int s = 128; s > 0; s >>= 1) {
      if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
      __syncthreads();
    }
    if (threadIdx.x == 0) out[(int64_t)b * (1 + D) + i] = red[0];
    __syncthreads();
  }
}

}  // namespace dbm

#include "sim_dense.cuh"

namespace dbm {

// ---- host side ------------------------------------------------------------------------------------

// Largest x with correctly rounded sqrt(x) <= R: the squared-distance test d2 <= R2 then takes
// exactly the decisions of sqrt(d2) <= R (sqrt is monotonic and correctly rounded on host and
// device).
template <class T>
static T sqrt_threshold(T R) {
  T x = R * R;
  for (int i = 0; i < 64; ++i) {
    const T n = std::nextafter(x, std::numeric_limits<T>::infinity());
    if (std::sqrt(n) <= R) x = n; else break;
  }
  for (int i = 0; i < 64 && std::sqrt(x) > R; ++i) x = std::nextafter(x, (T)0);
  return x;
}

// Snapshot blob: this header, then cell u32[M], off real[D][M] and f (FP64: double[Q][M];
// FP32DEV: float rho[M], float dev[Q][M]), each section starting on a 256-byte boundary.
struct SnapHeader {
  uint32_t magic;
  uint32_t m;
  int32_t lattice;
  int32_t precision;
};
constexpr uint32_t kSnapMagic = 0x44424d53u;  // "DBMS"
inline size_t snap_align(size_t x) { return (x + 255) & ~(size_t)255; }

template <int Q, int D, class P>
struct SimImpl : SimBase {
  using real = typename P::real;
  dbm_sim_desc desc{};
  std::vector<InstK> inst_h;
  uint32_t ncells = 0;
  int key_bits = 1;
  int64_t mcap = 0, ccap = 0;
  std::vector<void*> allocs;
  std::vector<size_t> alloc_sizes;  // bytes of allocs[i]
  int64_t bytes = 0;
  Args<Q, D, P> args{};  // args for the current direction (a = current state)
  StateP<P> st[2];
  int cur = 0;
  // sort buffers
  uint32_t *k_in = nullptr, *v_in = nullptr, *k_alt = nullptr, *v_alt = nullptr;
  bool sorted_in_alt = false;
  bool import_in_alt = false;  // where set_state's sort left the import order
  bool pow2_cell = false;      // cell a power of two: the float32 interface scales positions exactly in float
  InstK* dinst = nullptr;
  void* sort_tmp = nullptr;
  void* compact_tmp = nullptr;
  void* place_tmp = nullptr;  // scan scratch of the sort-free control-point placement
  Brick* d_bricks = nullptr;  // bricks of cells for the untiled window kernels (one per block)
  int nbricks = 0;
  BrickGeo bgeo{1, 1, 1};
  int place_h = 0;            // its neighbourhood half-width, 0 if it does not apply
  cudaStream_t own = nullptr;
  cudaEvent_t ev_in = nullptr, ev_out = nullptr;
  cudaGraphExec_t graph[2] = {nullptr, nullptr};
  cudaGraphExec_t graph_tr[2] = {nullptr, nullptr};  // the same step writing every intermediate
  unsigned long long graph_kernels = 0, graph_tr_kernels = 0;
  int trace_on = 0;
  // shared-memory tiling (2D)
  bool tiled = false;
  Tile2* d_tiles = nullptr;
  int ntiles = 0;
  int pgrid[3] = {1, 1, 1};  // persistent grids: thin+refine, weights, gather
  // whole-cell displacements (FP32 store, R < 2 cells): the gather builds one window-row table per
  // control point for all directions (k_gather_ts); geo_s is geo with that kernel's staging capacity
  bool shift_ok = false;
  int pgrid_s = 1, pgrid_rs = 1, pgrid_ws = 1;
  TileGeo geo_s{};
  size_t sm_gather_s = 0;
  // dense-stencil kernels (k_*_ds, shared memory = the dense layout) and the list of tiles they
  // defer to the row-segment code: d_fb[0..2] the per-stage counts, d_fb + 4 the tile indices
  size_t sm_ds[3] = {0, 0, 0};  // thin+refine, weights, gather
  int pgrid_ds[3] = {1, 1, 1};
  int* d_fb = nullptr;
  int use_persistent = 0;
  TileGeo geo{};
  size_t sm_refine = 0, sm_weights = 0, sm_gather = 0;

  ~SimImpl() override {
    for (auto& g : graph)
      if (g) cudaGraphExecDestroy(g);
    for (auto& g : graph_tr)
      if (g) cudaGraphExecDestroy(g);
    if (ev_in) cudaEventDestroy(ev_in);
    if (ev_out) cudaEventDestroy(ev_out);
    if (own) cudaStreamDestroy(own);
    if (hword) cudaFreeHost(hword);
    for (void* p : allocs) cudaFree(p);
  }

  // Host-visible words for status and count reads: a one-thread kernel writes them into mapped
  // pinned memory.  A 4-byte device-to-host copy would queue on the copy engine behind a caller's
  // bulk copies in flight (a pipelined load/export), stalling the read by milliseconds.
  uint32_t* hword = nullptr;
  uint32_t* hword_dev = nullptr;
  int read_word(uint32_t* src, int clear, int slot, cudaStream_t s, uint32_t* out) {
    if (!hword) {
      DBM_CUDA(cudaHostAlloc(&hword, 16, cudaHostAllocMapped));
      DBM_CUDA(cudaHostGetDevicePointer(&hword_dev, hword, 0));
    }
    k_read_word<<<1, 32, 0, s>>>(src, clear, hword_dev + slot);
    DBM_LAUNCH_CHECK();
    DBM_CUDA(cudaStreamSynchronize(s));
    *out = ((volatile uint32_t*)hword)[slot];
    return DBM_OK;
  }

  template <class T>
  int alloc(T** p, int64_t n) {
    size_t b = (size_t)std::max<int64_t>(n, 1) * sizeof(T);
    void* q = nullptr;
    DBM_CUDA(cudaMalloc(&q, b));
    allocs.push_back(q);
    alloc_sizes.push_back(b);
    bytes += (int64_t)b;
    *p = (T*)q;
    return DBM_OK;
  }

  int init(const dbm_sim_desc& d, const dbm_instance_desc* in, int n) {
    desc = d;
    {
      int ex = 0;
      pow2_cell = std::frexp(d.cell, &ex) == 0.5 && ex > -60 && ex < 60;
    }
    const LatHost& LH = *lat_host(d.lattice);
    const double R = d.r_res / d.cell;
    double cmax = 0;
    for (int k = 0; k < Q; ++k) {
      double s = 0;
      for (int a = 0; a < D; ++a) s += LH.c[k][a] * LH.c[k][a];
      cmax = std::max(cmax, std::sqrt(s) * d.dx / d.cell);
    }
    const int need = 2 * (int)std::ceil(R + cmax) + 4;  // periodic boxes must exceed every window
    uint64_t total = 0;
    inst_h.resize(n);
    for (int i = 0; i < n; ++i) {
      InstK& I = inst_h[i];
      I.base = (uint32_t)total;
      uint64_t sz = 1;
      for (int a = 0; a < 3; ++a) {
        I.dims[a] = a < D ? in[i].dims[a] : 1;
        I.origin[a] = a < D ? in[i].origin[a] : 0;
        if (I.dims[a] < 1) { set_last_error("instance %d: dims must be >= 1", i); return DBM_ERR_INVALID; }
        if (a < D && in[i].periodic && I.dims[a] < need) {
          set_last_error("instance %d: periodic box needs >= %d cells per axis (got %d)", i, need, I.dims[a]);
          return DBM_ERR_INVALID;
        }
        sz *= (uint64_t)I.dims[a];
      }
      I.periodic = in[i].periodic ? 1 : 0;
      if (!(in[i].tau > 0.5)) { set_last_error("instance %d: tau must be > 1/2", i); return DBM_ERR_INVALID; }
      I.tau = in[i].tau;
      I.rho_rest = in[i].rho_rest;
      total += sz;
    }
    if (total + 1 >= 0xffffffffull) { set_last_error("too many cells (%llu)", (unsigned long long)total); return DBM_ERR_CAPACITY; }
    ncells = (uint32_t)total;
    lattice = d.lattice;
    precision = d.precision;
    n_inst = n;
    n_cells = ncells;
    key_bits = 1;
    while (((uint64_t)1 << key_bits) <= (uint64_t)ncells) ++key_bits;
    ccap = ncells;
    mcap = std::max<int64_t>(d.moment_capacity, ncells);
    if (mcap >= 0x7fffffffLL) { set_last_error("moment capacity too large"); return DBM_ERR_CAPACITY; }

    uint32_t* dbase;
    DBM_TRY(alloc(&dinst, n));
    DBM_TRY(alloc(&dbase, n + 1));
    std::vector<uint32_t> hb(n + 1);
    for (int i = 0; i < n; ++i) hb[i] = inst_h[i].base;
    hb[n] = ncells;
    DBM_CUDA(cudaMemcpy(dinst, inst_h.data(), sizeof(InstK) * n, cudaMemcpyHostToDevice));
    DBM_CUDA(cudaMemcpy(dbase, hb.data(), sizeof(uint32_t) * (n + 1), cudaMemcpyHostToDevice));

    for (int s = 0; s < 2; ++s) {
      StateP<P>& S = st[s];
      const int64_t cap = std::max(mcap, ccap);
      DBM_TRY(alloc(&S.cell, cap));
      DBM_TRY(alloc(&S.off, (int64_t)D * cap));
      DBM_TRY(alloc(&S.pk, cap));
      if constexpr (std::is_same<P, PF64>::value) {
        DBM_TRY(alloc(&S.f64, (int64_t)Q * cap));
      } else {
        DBM_TRY(alloc(&S.rho, cap));
        DBM_TRY(alloc(&S.dev, (int64_t)Q * cap));
      }
      DBM_TRY(alloc(&S.start, (int64_t)ncells + 1));
      DBM_TRY(alloc(&S.count, 1));
      DBM_CUDA(cudaMemset(S.count, 0, 4));
      DBM_CUDA(cudaMemset(S.start, 0, ((size_t)ncells + 1) * 4));
    }
    // both state buffers share one capacity so they can swap roles
    mcap = ccap = std::max(mcap, ccap);

    Args<Q, D, P>& A = args;
    A.L = make_latk<Q, D>(LH, d.dx, d.cell);
    A.inst = dinst;
    A.inst_base = dbase;
    A.n_inst = n;
    A.ncells = ncells;
    A.R = (real)R;
    A.R2 = sqrt_threshold<real>(A.R);
    A.tiny = (real)1e-4;
    A.kappa_hard = d.kappa_hard;
    A.eps = (real)d.eps;
    A.mcap = mcap;
    A.ccap = ccap;
    DBM_TRY(alloc(&A.occ, ncells));
    DBM_TRY(alloc(&A.tcnt, ncells));
    DBM_TRY(alloc(&A.cen, (int64_t)D * ncells));
    DBM_TRY(alloc(&A.mask, ncells));
    DBM_TRY(alloc(&A.fkey, ncells));
    DBM_TRY(alloc(&A.foff, (int64_t)D * ncells));
    A.kappa_soft = 0;
    A.soft_off = 2.0 * (1.0 - std::sqrt(3.0) / 2.0) * d.dx / d.cell;  // direbm/reference/simulator.py:27
    A.foff2 = nullptr;
    const int64_t sort_cap = std::max<int64_t>(ncells, mcap);  // set_state sorts up to mcap moments
    DBM_TRY(alloc(&k_in, sort_cap));
    DBM_TRY(alloc(&v_in, sort_cap));
    DBM_TRY(alloc(&k_alt, sort_cap));
    DBM_TRY(alloc(&v_alt, sort_cap));
    char* tmp;
    DBM_TRY(alloc(&tmp, (int64_t)radix_tmp_bytes(sort_cap)));
    sort_tmp = tmp;
    DBM_TRY(alloc(&tmp, (int64_t)compact_tmp_bytes(ncells)));
    compact_tmp = tmp;
    DBM_TRY(alloc(&tmp, (int64_t)scan_tmp_bytes((int64_t)ncells + 1)));
    place_tmp = tmp;
    // sort-free placement (2D): move bound H = floor(R) + 1 cells; used while the (2H+1)^2
    // neighbourhood stays small and cannot wrap onto itself in a periodic box
    place_h = 0;
    if constexpr (D == 2) {
      const int H = (int)std::floor(R) + 1;
      bool ok = H <= 3;
      for (const InstK& I : inst_h)
        if (I.periodic && (I.dims[0] < 2 * H + 1 || I.dims[1] < 2 * H + 1)) ok = false;
      if (ok) place_h = H;
    }
    DBM_TRY(alloc(&A.sw, (int64_t)Q * mcap));
    A.kv = nullptr;  // the untiled path's buffers: see ensure_untiled
    A.wexp = nullptr;
    A.want_wexp = 0;
    if constexpr (std::is_same<P, PF64>::value) {
      DBM_TRY(alloc(&A.cpf64, (int64_t)Q * ccap));
    } else {
      DBM_TRY(alloc(&A.cpfhi, (int64_t)Q * ccap));
      DBM_TRY(alloc(&A.cpflo, (int64_t)Q * ccap));
    }
    DBM_TRY(alloc(&A.emask, ccap));
    DBM_TRY(alloc(&A.bmask, mcap));
    A.any_obstacle = 0;
    DBM_TRY(alloc(&A.status, 1));
    DBM_TRY(alloc(&A.d_P, 1));
    DBM_CUDA(cudaMemset(A.status, 0, 4));
    DBM_CUDA(cudaMemset(A.d_P, 0, 4));
    if constexpr (D == 2) DBM_TRY(init_tiles(LH, R));
    DBM_CUDA(cudaStreamCreateWithFlags(&own, cudaStreamNonBlocking));
    DBM_CUDA(cudaEventCreateWithFlags(&ev_in, cudaEventDisableTiming));
    DBM_CUDA(cudaEventCreateWithFlags(&ev_out, cudaEventDisableTiming));
    DBM_TRY(set_brick(D == 3 ? 8 : 16));  // 8 x 8 x 4 in 3D, 16 x 16 in 2D
    if (!tiled) DBM_TRY(ensure_untiled());  // 3D: always the untiled window kernels
    return DBM_OK;
  }

  // Bricks of 256 cells for the untiled window kernels, bx cells along x: 2D bx x (256 / bx); 3D the
  // other 256 / bx cells split between y and z, y taking the larger half.  Results do not depend
  // on the shape (each point's work is the same); only the L1 locality of a block does.
  int set_brick(int bx) override {
    const int minx = D == 3 ? 4 : 8, maxx = D == 3 ? 32 : 64;
    if (bx < minx || bx > maxx || (bx & (bx - 1))) {
      set_last_error("brick width %d: a power of two in %d..%d", bx, minx, maxx);
      return DBM_ERR_INVALID;
    }
    BrickGeo g{bx, 256 / bx, 1};
    if (D == 3) {
      const int rest = 256 / bx;
      int bz = 1;
      while ((2 * bz) * (2 * bz) <= rest) bz *= 2;  // the largest power of two with bz^2 <= rest
      g.bz = bz;
      g.by = rest / bz;
    }
    std::vector<Brick> bl;
    for (int i = 0; i < (int)inst_h.size(); ++i) {
      const int* dm = inst_h[i].dims;
      for (int z0 = 0; z0 < (D == 3 ? dm[2] : 1); z0 += g.bz)
        for (int y0 = 0; y0 < dm[1]; y0 += g.by)
          for (int x0 = 0; x0 < dm[0]; x0 += g.bx) bl.push_back({i, x0, y0, z0});
    }
    if (bl.size() >= 0x7fffffffu) { set_last_error("too many bricks"); return DBM_ERR_CAPACITY; }
    if (d_bricks) {
      if (own) DBM_CUDA(cudaStreamSynchronize(own));  // no step may still read the old list
      release(d_bricks);
      d_bricks = nullptr;
    }
    DBM_TRY(alloc(&d_bricks, (int64_t)bl.size()));
    DBM_CUDA(cudaMemcpy(d_bricks, bl.data(), sizeof(Brick) * bl.size(), cudaMemcpyHostToDevice));
    nbricks = (int)bl.size();
    bgeo = g;
    invalidate_graphs();  // captured launches hold the list and its size
    return DBM_OK;
  }
  int brick_width() const override { return bgeo.bx; }

  // Per-component buffers that only the untiled window kernels use: (1/sw, f*) pairs and exp(f*)
  // ([Q][mcap] each).  Allocated by the calls that make that path possible (creation in 3D, an
  // obstacle, the soft spawn, tiles off), so a tiled 2D simulation never holds them.
  int ensure_untiled() override {
    if (args.kv) return DBM_OK;
    DBM_TRY(alloc(&args.kv, (int64_t)Q * mcap));
    DBM_TRY(alloc(&args.wexp, (int64_t)Q * mcap));
    invalidate_graphs();  // captured launches hold the pointers
    return DBM_OK;
  }

  // Tile table, halos and shared-memory budgets of the tiled kernels (2D only).
  static size_t carve_bytes(const std::vector<std::pair<size_t, size_t>>& parts) {
    size_t off = 0;
    for (auto& pr : parts) off = ((off + 15) & ~(size_t)15) + pr.first * pr.second;
    return off + 16;
  }
  size_t smem_for(int kind, int cap) const {
    const size_t rs = sizeof(real);
    const size_t ct = (size_t)geo.cap_tile;
    const size_t cp = (size_t)cap;
    if (kind == 0) {  // thin+refine
      const size_t cells = (size_t)(geo.tx + geo.mom.xh - geo.mom.xl) * (geo.ty + geo.mom.yh - geo.mom.yl);
      const size_t rh = geo.ty + geo.mom.yh - geo.mom.yl;
      return carve_bytes({{cells, 4}, {cells, 4}, {rh + 2, 4}, {cp, 4 * rs}, {(size_t)Q * cp, rs}});
    } else if (kind == 1) {  // weights
      const size_t cells = (size_t)(geo.tx + geo.cp.xh - geo.cp.xl) * (geo.ty + geo.cp.yh - geo.cp.yl);
      const size_t rh = geo.ty + geo.cp.yh - geo.cp.yl;
      return carve_bytes({{cells, 4}, {cells, 4}, {rh + 2, 4}, {cp, 4 * rs}, {(size_t)2 * geo.ty + 2, 4}, {ct, 4},
                          {ct, 2}, {ct, 2}, {ct, 2 * rs}});
    } else if (kind == 2) {  // gather
      const size_t cells = (size_t)(geo.tx + geo.mom.xh - geo.mom.xl) * (geo.ty + geo.mom.yh - geo.mom.yl);
      const size_t rh = geo.ty + geo.mom.yh - geo.mom.yl;
      return carve_bytes({{cells, 4}, {cells, 4}, {rh + 2, 4}, {cp, 4}, {cp, 4 * rs}, {cp, rs}, {cp, 2 * rs},
                          {(size_t)2 * geo.ty + 2, 4}, {ct, 4}, {ct, 2}, {ct, 2}, {ct, 2 * rs}});
    } else {  // gather with whole-cell displacements (FP32): GRec records
      const size_t cells = (size_t)(geo.tx + geo.mom.xh - geo.mom.xl) * (geo.ty + geo.mom.yh - geo.mom.yl);
      const size_t rh = geo.ty + geo.mom.yh - geo.mom.yl;
      return carve_bytes({{cells, 4}, {cells, 4}, {rh + 2, 4}, {cp, 4}, {cp, sizeof(GRec)}, {(size_t)2 * geo.ty + 2, 4},
                          {ct, 4}, {ct, 2}, {ct, 2}, {ct, 8}});
    }
  }
  int pick_cap(int kind, int cells, size_t budget) const {
    int cap = cells + cells / 2 + 64;  // 1.5 items per region cell; denser regions read global memory
    while (cap > 64 && smem_for(kind, cap) > budget) cap = cap * 7 / 8;
    return cap;
  }

  // Tile geometry for tiles of tx x (256 / tx) cells: halos from the lattice and R, staging
  // capacities from the shared-memory budget, the tile list, and the resident blocks per SM of the
  // three tiled kernels (the grid of their persistent launch).
  int init_tiles(const LatHost& LH, double R, int tx = 32) {
    if (tx < 8 || tx > 128 || 256 % tx) { set_last_error("tile width %d: must divide 256, 8..128", tx); return DBM_ERR_INVALID; }
    geo.tx = tx;
    geo.ty = 256 / tx;
    const double tiny = 2e-4;
    Halo m{0, 0, 0, 0}, c{0, 0, 0, 0};
    for (int k = 0; k < Q; ++k) {
      for (int a = 0; a < 2; ++a) {
        // cover both the FP64 displacement and its FP32 rounding (the FP32 kernels use the latter)
        const double cd64 = LH.c[k][a] * desc.dx / desc.cell;
        const double cd32 = (double)(float)cd64;
        const double cdmin = std::min(cd64, cd32), cdmax = std::max(cd64, cd32);
        int lo = (int)std::floor(-cdmax - R - tiny), hi = (int)std::floor(1.0 - cdmin + R + tiny);
        lo = std::min(lo, -(int)std::floor(cdmax) - 1);
        hi = std::max(hi, -(int)std::floor(cdmin));
        const int clo = (int)std::floor(cdmin - R - tiny), chi = (int)std::floor(cdmax + 1.0 + R + tiny);
        if (a == 0) {
          m.xl = std::min(m.xl, lo); m.xh = std::max(m.xh, hi);
          c.xl = std::min(c.xl, clo); c.xh = std::max(c.xh, chi);
        } else {
          m.yl = std::min(m.yl, lo); m.yh = std::max(m.yh, hi);
          c.yl = std::min(c.yl, clo); c.yh = std::max(c.yh, chi);
        }
      }
    }
    geo.mom = m;
    geo.cp = c;
    const int mcells = (geo.tx + m.xh - m.xl) * (geo.ty + m.yh - m.yl);
    const int ccells = (geo.tx + c.xh - c.xl) * (geo.ty + c.yh - c.yl);
    const size_t budget = std::is_same<P, PF64>::value ? 112 * 1024 : 56 * 1024;
    geo.cap_tile = 2 * geo.tx * geo.ty;
    geo.cap_refine = pick_cap(0, mcells, budget);
    geo.cap_weights = pick_cap(1, ccells, budget);
    geo.cap_gather = pick_cap(2, mcells, budget);
    sm_refine = smem_for(0, geo.cap_refine);
    sm_weights = smem_for(1, geo.cap_weights);
    sm_gather = smem_for(2, geo.cap_gather);
    // whole-cell displacements: every c * dx / cell an integer (in FP64 and in its FP32 rounding)
    shift_ok = std::is_same<P, PF32>::value && R < 1.99;
    for (int k = 0; k < Q && shift_ok; ++k)
      for (int a = 0; a < 2; ++a) {
        const double cd64 = LH.c[k][a] * desc.dx / desc.cell;
        shift_ok = shift_ok && cd64 == std::nearbyint(cd64) && (double)(float)cd64 == cd64 && std::fabs(cd64) <= 8.0;
      }
    geo_s = geo;
    if (shift_ok) {
      geo_s.cap_gather = pick_cap(3, mcells, budget);
      sm_gather_s = smem_for(3, geo_s.cap_gather);
      sm_ds[0] = ds_bytes_refine(Q, mcells);
      sm_ds[1] = ds_bytes_weights(ccells);
      sm_ds[2] = ds_bytes_gather(Q, mcells);
    }
    std::vector<Tile2> tiles;
    for (int i = 0; i < (int)inst_h.size(); ++i)
      for (int y0 = 0; y0 < inst_h[i].dims[1]; y0 += geo.ty)
        for (int x0 = 0; x0 < inst_h[i].dims[0]; x0 += geo.tx) tiles.push_back({i, x0, y0});
    ntiles = (int)tiles.size();
    if (d_tiles) {  // re-tiling: release the previous list
      release(d_tiles);
      d_tiles = nullptr;
    }
    DBM_TRY(alloc(&d_tiles, ntiles));
    DBM_CUDA(cudaMemcpy(d_tiles, tiles.data(), sizeof(Tile2) * ntiles, cudaMemcpyHostToDevice));
    if (d_fb) {
      release(d_fb);
      d_fb = nullptr;
    }
    if (shift_ok) {
      DBM_TRY(alloc(&d_fb, (int64_t)ntiles + 4));
      DBM_CUDA(cudaMemset(d_fb, 0, ((size_t)ntiles + 4) * sizeof(int)));
    }
    if constexpr (D == 2) {
      DBM_CUDA(cudaFuncSetAttribute((const void*)k_thin_refine_t<Q, P>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)sm_refine));
      DBM_CUDA(cudaFuncSetAttribute((const void*)k_weights_t<Q, P>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)sm_weights));
      DBM_CUDA(cudaFuncSetAttribute((const void*)k_gather_t<Q, P>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)sm_gather));
      int nb[3] = {1, 1, 1};
      DBM_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb[0], k_thin_refine_t<Q, P>, 256, sm_refine));
      DBM_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb[1], k_weights_t<Q, P>, 256, sm_weights));
      DBM_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb[2], k_gather_t<Q, P>, 256, sm_gather));
      for (int i = 0; i < 3; ++i) pgrid[i] = std::max(1, std::min(ntiles, std::max(nb[i], 1) * sm_count()));
      if constexpr (std::is_same<P, PF32>::value) {
        if (shift_ok) {
          DBM_CUDA(cudaFuncSetAttribute((const void*)k_gather_ts<Q>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        (int)sm_gather_s));
          int nbs = 1;
          DBM_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nbs, k_gather_ts<Q>, 256, sm_gather_s));
          pgrid_s = std::max(1, std::min(ntiles, std::max(nbs, 1) * sm_count()));
          DBM_CUDA(cudaFuncSetAttribute((const void*)k_thin_refine_t<Q, P, true>,
                                        cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm_refine));
          int nbr = 1;
          DBM_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nbr, k_thin_refine_t<Q, P, true>, 256, sm_refine));
          pgrid_rs = std::max(1, std::min(ntiles, std::max(nbr, 1) * sm_count()));
          DBM_CUDA(cudaFuncSetAttribute((const void*)k_weights_t<Q, P, true>,
                                        cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm_weights));
          int nbw = 1;
          DBM_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nbw, k_weights_t<Q, P, true>, 256, sm_weights));
          pgrid_ws = std::max(1, std::min(ntiles, std::max(nbw, 1) * sm_count()));
          const void* kds[3] = {(const void*)k_thin_refine_ds<Q>, (const void*)k_weights_ds<Q>,
                                (const void*)k_gather_ds<Q>};
          for (int i = 0; i < 3; ++i) {
            DBM_CUDA(cudaFuncSetAttribute(kds[i], cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm_ds[i]));
            int nbd = 1;
            DBM_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nbd, kds[i], 256, sm_ds[i]));
            pgrid_ds[i] = std::max(1, std::min(ntiles, std::max(nbd, 1) * sm_count()));
          }
          DBM_CUDA(cudaFuncSetAttribute((const void*)k_dense_fallback<Q, 0>,
                                        cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm_refine));
          DBM_CUDA(cudaFuncSetAttribute((const void*)k_dense_fallback<Q, 1>,
                                        cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm_weights));
          DBM_CUDA(cudaFuncSetAttribute((const void*)k_dense_fallback<Q, 2>,
                                        cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm_gather_s));
        }
      }
    }
    tiled = true;
    return DBM_OK;
  }

  // Tile width (height 256 / width) and persistent launches of the tiled kernels; results do not
  // depend on either (each tile is one block with the same per-thread loop order).
  int set_tiling(int tx, int persistent) {
    if constexpr (D == 2) {
      if (tx != geo.tx) DBM_TRY(init_tiles(*lat_host(desc.lattice), desc.r_res / desc.cell, tx));
      use_persistent = persistent ? 1 : 0;
      invalidate_graphs();
      return DBM_OK;
    } else {
      set_last_error("tiling options apply to 2D lattices only");
      return DBM_ERR_INVALID;
    }
  }
  int tiling(int* tx, int* persistent) const override {
    *tx = geo.tx;
    *persistent = use_persistent;
    return DBM_OK;
  }
  int set_tiling_v(int tx, int persistent) override { return set_tiling(tx, persistent); }

  // Soft-outer spawn (direbm/reference/simulator.py:126-166) for kappa_hard < kappa <= ks; 0 turns
  // it off.  Up to one extra CP per thinning cell, so the CP capacity must hold 2 ncells.
  int set_soft_spawn(int ks) override {
    if (ks < 0) { set_last_error("soft spawn: kappa_soft must be >= 0"); return DBM_ERR_INVALID; }
    if (ks > 0) {
      if (ccap < 2 * (int64_t)ncells || 2 * (uint64_t)ncells >= 0xffffffffull) {
        set_last_error("soft spawn needs a moment capacity of at least 2 x cells (%lld), have %lld",
                       (long long)(2 * (int64_t)ncells), (long long)ccap);
        return DBM_ERR_CAPACITY;
      }
      if (!spawn_ready) {
        DBM_CUDA(cudaStreamSynchronize(own));  // no step may still use the single-block buffers
        uint32_t *occ2 = nullptr, *fkey2 = nullptr;
        DBM_TRY(alloc(&occ2, 2 * (int64_t)ncells));
        DBM_TRY(alloc(&fkey2, 2 * (int64_t)ncells));
        DBM_TRY(alloc(&args.foff2, (int64_t)D * ncells));
        char* tmp;
        DBM_TRY(alloc(&tmp, (int64_t)compact_tmp_bytes(2 * (int64_t)ncells)));
        release(args.occ);
        release(args.fkey);
        release(compact_tmp);
        args.occ = occ2;
        args.fkey = fkey2;
        compact_tmp = tmp;
        spawn_ready = true;
      }
    }
    if (ks > 0) DBM_TRY(ensure_untiled());
    args.kappa_soft = ks;
    kappa_soft = ks;
    invalidate_graphs();  // captured launches hold the flag and the buffers
    return DBM_OK;
  }
  bool spawn_ready = false;

  // Free one of this handle's allocations (the caller syncs first if a step may still use it).
  void release(void* p) {
    if (!p) return;
    for (size_t i = 0; i < allocs.size(); ++i) {
      if (allocs[i] != p) continue;
      cudaFree(p);
      bytes -= (int64_t)alloc_sizes[i];
      allocs.erase(allocs.begin() + (std::ptrdiff_t)i);
      alloc_sizes.erase(alloc_sizes.begin() + (std::ptrdiff_t)i);
      return;
    }
  }

  void invalidate_graphs() override {
    for (auto* set : {graph, graph_tr})
      for (int i = 0; i < 2; ++i)
        if (set[i]) {
          cudaGraphExecDestroy(set[i]);
          set[i] = nullptr;
        }
  }

  void bind() {
    args.a = st[cur];
    args.b = st[cur ^ 1];
    args.write_trace = trace_on;
  }

  template <class T>
  int import_sorted_states(int64_t m, cudaStream_t s, const int32_t* inst_of, const T* pos, const T* fin,
                           bool presorted) {
    bind();
    const unsigned grid = std::min<unsigned>(div_up(std::max<int64_t>(m, 1), 256), (unsigned)sm_count() * 8);
    const float inv_cell_f = pow2_cell ? (float)(1.0 / desc.cell) : 0.f;
    const uint32_t* ks = args.a.cell;  // the state's cell array holds the sorted keys either way
    if (presorted) {
      // given in cell order: one pass, no sort, then a check of the order
      import_in_alt = false;
      k_import_presorted<Q, D, P, T><<<grid, 256, 0, s>>>(args, inst_of, pos, fin, m, desc.cell, inv_cell_f, v_in);
      DBM_LAUNCH_CHECK();
      if (m > 1) {
        k_check_sorted<<<grid, 256, 0, s>>>(args.a.cell, m, args.status);
        DBM_LAUNCH_CHECK();
      }
    } else {
      // the unsorted offsets [D][m] live in the weight scratch sw ([Q][mcap], Q > D, idle outside a
      // step): an allocation here (and its cudaFree) would wait for every stream of the device,
      // including a caller's copies that overlap the load
      real* toff = args.sw;
      k_import_keys<Q, D, P, T><<<grid, 256, 0, s>>>(args, inst_of, pos, m, desc.cell, inv_cell_f, k_in, v_in, toff);
      DBM_LAUNCH_CHECK();
      // valid keys are < ncells < 2^key_bits; the marker 0xffffffff of a moment outside its box is
      // all ones in those bits too, so it still sorts after every valid key
      bool alt = false;
      DBM_TRY(radix_sort_pairs<uint32_t>(k_in, v_in, k_alt, v_alt, m, nullptr, key_bits, sort_tmp, s, &alt));
      import_in_alt = alt;
      k_import_gather<Q, D, P, T><<<grid, 256, 0, s>>>(args, fin, m, alt ? k_alt : k_in, alt ? v_alt : v_in, toff);
      DBM_LAUNCH_CHECK();
    }
    // count of valid keys = m (invalid ones sort last with key 0xffffffff and raise ST_BAD_INPUT)
    DBM_CUDA(cudaMemcpyAsync(args.d_P, args.a.count, 4, cudaMemcpyDeviceToDevice, s));
    launch_cell_start(ks, args.d_P, ncells, args.a.start, s);
    DBM_LAUNCH_CHECK();
    return DBM_OK;
  }

  int load(const int32_t* inst_of, const void* pos, const void* fin, int64_t m, int flags, cudaStream_t s) override {
    if (m < 0 || m > mcap) { set_last_error("set_state: %lld moments exceed capacity %lld", (long long)m, (long long)mcap); return DBM_ERR_CAPACITY; }
    if (m > 0 && (!inst_of || !pos || !fin)) { set_last_error("set_state: null input"); return DBM_ERR_INVALID; }
    cur = 0;
    ++version;
    const bool presorted = (flags & kLoadPresorted) != 0;
    if (flags & kLoadF32)
      return import_sorted_states<float>(m, s, inst_of, (const float*)pos, (const float*)fin, presorted);
    return import_sorted_states<double>(m, s, inst_of, (const double*)pos, (const double*)fin, presorted);
  }

  // Launch the stages of one step (a = st[cur] -> b = st[cur^1]) on stream s, up to `upto`.
  cudaEvent_t* stage_ev = nullptr;  // when set, an event is recorded after each stage
  void mark(int i, cudaStream_t s) {
    if (stage_ev) cudaEventRecord(stage_ev[i], s);
  }

  // The tiled 2D kernels serve plain periodic/bounded boxes; obstacles and the soft spawn run on
  // the untiled window kernels.
  bool tiled_path() const { return D == 2 && tiled && use_tiles && !args.any_obstacle && args.kappa_soft == 0; }

  int launch_step(cudaStream_t s, int upto) {
    bind();
    Args<Q, D, P>& A = args;
    mark(0, s);
    const unsigned gm = std::min<unsigned>(div_up(mcap, 256), (unsigned)sm_count() * 16);
    // the untiled window kernels (3D, obstacles, the soft spawn, or tiles off) read packed items
    // and the refine weights exp(f*) precomputed by the collision
    const bool untiled = !tiled_path();
    if (untiled && !A.kv) {
      set_last_error("internal: the untiled window kernels' buffers were not allocated");
      return DBM_ERR_STATE;
    }
    A.want_wexp = untiled ? 1 : 0;
    k_collide<Q, D, P><<<gm, 256, 0, s>>>(A);
    DBM_LAUNCH_CHECK();
    if (untiled) {
      k_pack<Q, D, P><<<gm, 256, 0, s>>>(A, A.a, A.mcap, A.a.count);
      DBM_LAUNCH_CHECK();
    }
    mark(1, s);
    if (upto <= 1) return DBM_OK;
    if constexpr (D == 2) {
      if (tiled_path()) {
        bool shifted = false;
        if constexpr (std::is_same<P, PF32>::value) {
          if (shift_ok && use_shift && use_dense) {
            DBM_CUDA(cudaMemsetAsync(d_fb, 0, 3 * sizeof(int), s));  // the three stages' fallback counts
            k_thin_refine_ds<Q><<<use_persistent ? pgrid_ds[0] : ntiles, 256, sm_ds[0], s>>>(A, d_tiles, geo, ntiles,
                                                                                            d_fb + 4, d_fb + 0);
            DBM_LAUNCH_CHECK();
            k_dense_fallback<Q, 0><<<pgrid_rs, 256, sm_refine, s>>>(A, d_tiles, geo, d_fb + 4, d_fb + 0);
            shifted = true;
          } else if (shift_ok && use_shift) {
            k_thin_refine_t<Q, P, true><<<use_persistent ? pgrid_rs : ntiles, 256, sm_refine, s>>>(A, d_tiles, geo,
                                                                                                  ntiles);
            shifted = true;
          }
        }
        if (!shifted)
          k_thin_refine_t<Q, P><<<use_persistent ? pgrid[0] : ntiles, 256, sm_refine, s>>>(A, d_tiles, geo, ntiles);
      } else {
        k_thin_refine<Q, D, P><<<nbricks, 256, 0, s>>>(A, d_bricks, nbricks, bgeo);
      }
    } else {
      k_thin_refine<Q, D, P><<<nbricks, 256, 0, s>>>(A, d_bricks, nbricks, bgeo);
    }
    DBM_LAUNCH_CHECK();
    mark(2, s);
    if (upto <= 2) return DBM_OK;
    // slots: regular CPs [0, ncells), spawned ones [ncells, 2 ncells); the stable sort keeps that
    // order among CPs of one cell
    const unsigned gc = std::min<unsigned>(div_up(ccap, 256), (unsigned)sm_count() * 16);
    if (!untiled && place_h > 0 && A.kappa_soft == 0) {
      // counts per final cell -> cell starts (and P) by one scan -> each point's slot
      const unsigned gf = std::min<unsigned>(div_up(ncells, 256), (unsigned)sm_count() * 16);
      DBM_CUDA(cudaMemsetAsync(A.b.start, 0, ((size_t)ncells + 1) * 4, s));
      k_place_count<Q, D, P><<<gf, 256, 0, s>>>(A, A.b.start);
      DBM_LAUNCH_CHECK();
      DBM_TRY(scan_exclusive_u32(A.b.start, A.b.start, (int64_t)ncells + 1, nullptr, A.d_P, place_tmp, s));
      k_place<Q, D, P><<<gf, 256, 0, s>>>(A, place_h, k_in, v_in);
      DBM_LAUNCH_CHECK();
      sorted_in_alt = false;
      A.skeys = k_in;
      A.svals = v_in;
    } else {
      const int64_t nslots = A.kappa_soft > 0 ? 2 * (int64_t)ncells : (int64_t)ncells;
      DBM_TRY(compact_flags_u32(A.occ, A.fkey, k_in, v_in, nslots, A.d_P, compact_tmp, s));
      bool alt = false;
      DBM_TRY(radix_sort_pairs<uint32_t>(k_in, v_in, k_alt, v_alt, nslots, A.d_P, key_bits, sort_tmp, s, &alt));
      sorted_in_alt = alt;
      A.skeys = alt ? k_alt : k_in;
      A.svals = alt ? v_alt : v_in;
      k_finalize<Q, D, P><<<gc, 256, 0, s>>>(A);
      DBM_LAUNCH_CHECK();
      if (untiled) {
        k_pack<Q, D, P><<<gc, 256, 0, s>>>(A, A.b, A.ccap, A.d_P);
        DBM_LAUNCH_CHECK();
      }
      launch_cell_start(A.skeys, A.d_P, ncells, A.b.start, s);
      DBM_LAUNCH_CHECK();
    }
    mark(3, s);
    if (upto <= 3) return DBM_OK;
    if constexpr (D == 2) {
      if (tiled_path()) {
        bool shifted = false;
        if constexpr (std::is_same<P, PF32>::value) {
          if (shift_ok && use_shift && use_dense) {
            k_weights_ds<Q><<<use_persistent ? pgrid_ds[1] : ntiles, 256, sm_ds[1], s>>>(A, d_tiles, geo, ntiles,
                                                                                        d_fb + 4, d_fb + 1);
            DBM_LAUNCH_CHECK();
            k_dense_fallback<Q, 1><<<pgrid_ws, 256, sm_weights, s>>>(A, d_tiles, geo, d_fb + 4, d_fb + 1);
            shifted = true;
          } else if (shift_ok && use_shift) {
            k_weights_t<Q, P, true><<<use_persistent ? pgrid_ws : ntiles, 256, sm_weights, s>>>(A, d_tiles, geo,
                                                                                               ntiles);
            shifted = true;
          }
        }
        if (!shifted)
          k_weights_t<Q, P><<<use_persistent ? pgrid[1] : ntiles, 256, sm_weights, s>>>(A, d_tiles, geo, ntiles);
      } else {
        k_weights<Q, D, P><<<dim3(nbricks, Q), 256, 0, s>>>(A, d_bricks, nbricks, bgeo);
      }
    } else {
      k_weights<Q, D, P><<<dim3(nbricks, Q), 256, 0, s>>>(A, d_bricks, nbricks, bgeo);
    }
    DBM_LAUNCH_CHECK();
    mark(4, s);
    if (upto <= 4) return DBM_OK;
    DBM_CUDA(cudaMemsetAsync(A.emask, 0, (size_t)ccap * 4, s));
    if constexpr (D == 2) {
      if (tiled_path()) {
        bool shifted = false;
        if constexpr (std::is_same<P, PF32>::value) {
          if (shift_ok && use_shift && use_dense) {
            k_gather_ds<Q><<<use_persistent ? pgrid_ds[2] : ntiles, 256, sm_ds[2], s>>>(A, d_tiles, geo_s, ntiles,
                                                                                       d_fb + 4, d_fb + 2);
            DBM_LAUNCH_CHECK();
            k_dense_fallback<Q, 2><<<pgrid_s, 256, sm_gather_s, s>>>(A, d_tiles, geo_s, d_fb + 4, d_fb + 2);
            shifted = true;
          } else if (shift_ok && use_shift) {
            k_gather_ts<Q><<<use_persistent ? pgrid_s : ntiles, 256, sm_gather_s, s>>>(A, d_tiles, geo_s, ntiles);
            shifted = true;
          }
        }
        if (!shifted)
          k_gather_t<Q, P><<<use_persistent ? pgrid[2] : ntiles, 256, sm_gather, s>>>(A, d_tiles, geo, ntiles);
      } else {
        k_gather<Q, D, P><<<dim3(nbricks, Q), 256, 0, s>>>(A, d_bricks, nbricks, bgeo);
      }
    } else {
      k_gather<Q, D, P><<<dim3(nbricks, Q), 256, 0, s>>>(A, d_bricks, nbricks, bgeo);
    }
    DBM_LAUNCH_CHECK();
    mark(5, s);
    if (upto <= 5) return DBM_OK;
    k_emit<Q, D, P><<<gc, 256, 0, s>>>(A);
    DBM_LAUNCH_CHECK();
    mark(6, s);
    return DBM_OK;
  }

  int step(int n, cudaStream_t s) override {
    if (n <= 0) return DBM_OK;
    ++version;
    DBM_CUDA(cudaEventRecord(ev_in, s));
    DBM_CUDA(cudaStreamWaitEvent(own, ev_in, 0));
    for (int i = 0; i < n; ++i) {
      if (use_graphs && !trace_on) {
        if (!graph[cur]) {
          const unsigned long long before = g_launches;
          cudaGraph_t gr;
          DBM_CUDA(cudaStreamBeginCapture(own, cudaStreamCaptureModeThreadLocal));
          int rc = launch_step(own, 99);
          cudaError_t e = cudaStreamEndCapture(own, &gr);
          if (rc != DBM_OK) return rc;
          if (e != cudaSuccess) { set_last_error("graph capture failed: %s", cudaGetErrorString(e)); return DBM_ERR_CUDA; }
          graph_kernels = g_launches - before;
          g_launches = before;
          DBM_CUDA(cudaGraphInstantiate(&graph[cur], gr, 0));
          cudaGraphDestroy(gr);
        }
        DBM_CUDA(cudaGraphLaunch(graph[cur], own));
        count_launch(graph_kernels);
      } else {
        DBM_TRY(launch_step(own, 99));
      }
      cur ^= 1;
    }
    bind();
    DBM_CUDA(cudaEventRecord(ev_out, own));
    DBM_CUDA(cudaStreamWaitEvent(s, ev_out, 0));
    return DBM_OK;
  }

  // One full step launched stage by stage (no graph) with an event after each stage; stage_ms
  // receives the 6 stage durations (collide, thin+refine, compaction+sort+finalize, weights,
  // gather, emit) measured on the stream the kernels run on.
  int profile_step(float* stage_ms, cudaStream_t s) override {
    ++version;
    cudaEvent_t ev[7];
    for (auto& e : ev) DBM_CUDA(cudaEventCreate(&e));
    DBM_CUDA(cudaEventRecord(ev_in, s));
    DBM_CUDA(cudaStreamWaitEvent(own, ev_in, 0));
    stage_ev = ev;
    int rc = launch_step(own, 99);
    stage_ev = nullptr;
    if (rc == DBM_OK) {
      cur ^= 1;
      bind();
      DBM_CUDA(cudaEventRecord(ev_out, own));
      DBM_CUDA(cudaStreamWaitEvent(s, ev_out, 0));
      DBM_CUDA(cudaEventSynchronize(ev[6]));
      for (int i = 0; i < 6; ++i) cudaEventElapsedTime(&stage_ms[i], ev[i], ev[i + 1]);
    }
    for (auto& e : ev) cudaEventDestroy(e);
    return rc;
  }

  int step_partial(int upto, cudaStream_t s) override {
    trace_on = 1;
    ++version;
    DBM_CUDA(cudaEventRecord(ev_in, s));
    DBM_CUDA(cudaStreamWaitEvent(own, ev_in, 0));
    int rc = launch_step(own, upto);
    DBM_CUDA(cudaEventRecord(ev_out, own));
    DBM_CUDA(cudaStreamWaitEvent(s, ev_out, 0));
    if (rc != DBM_OK) return rc;
    if (upto >= 6) { cur ^= 1; }
    bind();
    return DBM_OK;
  }

  // One full step launched stage by stage with every intermediate kept, and `h` called before the
  // collision and after the emit (the adjoint records its tape there).
  int step_hooked(StepHook* h, cudaStream_t s) override {
    const int keep = trace_on;
    ++version;
    trace_on = 1;
    DBM_CUDA(cudaEventRecord(ev_in, s));
    DBM_CUDA(cudaStreamWaitEvent(own, ev_in, 0));
    bind();
    int rc = h->before(&args, own);
    if (rc == DBM_OK) {
      if (use_graphs) {  // the step with every intermediate kept, captured once per buffer parity
        if (!graph_tr[cur]) {
          const unsigned long long before = g_launches;
          cudaGraph_t gr;
          DBM_CUDA(cudaStreamBeginCapture(own, cudaStreamCaptureModeThreadLocal));
          rc = launch_step(own, 99);
          cudaError_t e = cudaStreamEndCapture(own, &gr);
          if (rc != DBM_OK) { trace_on = keep; return rc; }
          if (e != cudaSuccess) { trace_on = keep; set_last_error("graph capture failed: %s", cudaGetErrorString(e)); return DBM_ERR_CUDA; }
          graph_tr_kernels = g_launches - before;
          g_launches = before;
          DBM_CUDA(cudaGraphInstantiate(&graph_tr[cur], gr, 0));
          cudaGraphDestroy(gr);
        }
        DBM_CUDA(cudaGraphLaunch(graph_tr[cur], own));
        count_launch(graph_tr_kernels);
      } else {
        rc = launch_step(own, 99);
      }
    }
    if (rc == DBM_OK) rc = h->after(&args, own);
    trace_on = keep;
    if (rc != DBM_OK) return rc;
    cur ^= 1;
    bind();
    DBM_CUDA(cudaEventRecord(ev_out, own));
    DBM_CUDA(cudaStreamWaitEvent(s, ev_out, 0));
    return DBM_OK;
  }

  int set_tau(const double* tau, int n) override {
    if (n != (int)inst_h.size()) { set_last_error("set_tau: expected %d values, got %d", (int)inst_h.size(), n); return DBM_ERR_INVALID; }
    for (int i = 0; i < n; ++i)
      if (!(tau[i] > 0.5)) { set_last_error("set_tau: tau must be > 1/2 (instance %d)", i); return DBM_ERR_INVALID; }
    DBM_CUDA(cudaStreamSynchronize(own));  // no step may still read the table
    for (int i = 0; i < n; ++i) inst_h[i].tau = tau[i];
    DBM_CUDA(cudaMemcpy(dinst, inst_h.data(), sizeof(InstK) * n, cudaMemcpyHostToDevice));
    return DBM_OK;
  }

  // A solid sphere (disc in 2D) with bounce-back in instance `b`: center in world units (D values),
  // radius in world units; radius <= 0 removes it.  A sphere in a periodic box must keep a margin
  // of one window from the box faces (the blocked test uses the box's own coordinates, no image).
  int set_obstacle(int b, const double* center, double radius) override {
    if (b < 0 || b >= (int)inst_h.size() || (radius > 0 && !center)) { set_last_error("set_obstacle: bad arguments"); return DBM_ERR_INVALID; }
    InstK& I = inst_h[b];
    if (radius > 0) {
      const double r = radius / desc.cell;
      double cmax = 0;
      const LatHost& LH = *lat_host(desc.lattice);
      for (int k = 0; k < Q; ++k) {
        double s2 = 0;
        for (int a = 0; a < D; ++a) s2 += LH.c[k][a] * LH.c[k][a];
        cmax = std::max(cmax, std::sqrt(s2) * desc.dx / desc.cell);
      }
      const double margin = desc.r_res / desc.cell + cmax + 2;
      for (int a = 0; a < D; ++a) {
        const double c = center[a] / desc.cell - I.origin[a];
        if (I.periodic && (c - r - margin < 0 || c + r + margin > I.dims[a])) {
          set_last_error("set_obstacle: the sphere must stay %.1f cells away from the faces of a periodic box", margin);
          return DBM_ERR_INVALID;
        }
        I.obs_c[a] = c;
      }
      DBM_TRY(ensure_untiled());
      I.obs_r2 = r * r;
      I.has_obs = 1;
      // margins (cell units, generous against FP32 rounding): a blocked direction ends inside the
      // sphere, so its moment lies within r + |cd| of the center; a bounced component within the
      // resampling radius of a point puts that point within r + |cd| + R
      const double near = r + cmax + 1.0, reach = r + cmax + desc.r_res / desc.cell + 2.0;
      I.near2 = (float)(near * near);
      I.reach2 = (float)(reach * reach);
    } else {
      I.has_obs = 0;
    }
    return push_instances();
  }

  // An inflow layer in instance `b`: moments in the first `width` cell columns (x) are set to the
  // equilibrium at velocity u (D values) with their own density instead of colliding.
  int set_inflow(int b, const double* u, int width) override {
    if (b < 0 || b >= (int)inst_h.size() || width < 0 || (width > 0 && !u)) { set_last_error("set_inflow: bad arguments"); return DBM_ERR_INVALID; }
    InstK& I = inst_h[b];
    I.inflow_w = width;
    for (int a = 0; a < 3; ++a) I.u_in[a] = (width > 0 && a < D) ? u[a] : 0.0;
    return push_instances();
  }

  int push_instances() {
    DBM_CUDA(cudaStreamSynchronize(own));  // no step may still read the table
    DBM_CUDA(cudaMemcpy(dinst, inst_h.data(), sizeof(InstK) * inst_h.size(), cudaMemcpyHostToDevice));
    int any = 0;
    for (auto& I : inst_h) any |= I.has_obs;
    if (any != args.any_obstacle) {
      args.any_obstacle = any;
      invalidate_graphs();  // captured launches hold the flag
    }
    return DBM_OK;
  }

  size_t snap_bytes(uint32_t m) const {
    size_t b = snap_align(sizeof(SnapHeader));
    b += snap_align((size_t)m * 4) + snap_align((size_t)D * m * sizeof(real));
    if constexpr (std::is_same<P, PF64>::value) b += snap_align((size_t)Q * m * 8);
    else b += snap_align((size_t)m * 4) + snap_align((size_t)Q * m * 4);
    return b;
  }

  // Copy the current state (count, cells, offsets, f) into a compact device blob.
  int snapshot(void* dst, int64_t nbytes, int64_t* needed, cudaStream_t s) override {
    int64_t m64 = 0;
    DBM_CUDA(cudaEventRecord(ev_in, s));
    DBM_CUDA(cudaStreamWaitEvent(own, ev_in, 0));
    DBM_TRY(count(&m64, own));
    const uint32_t m = (uint32_t)m64;
    const size_t sz = snap_bytes(m);
    if (needed) *needed = (int64_t)sz;
    if (!dst) return DBM_OK;
    if (nbytes < (int64_t)sz) { set_last_error("snapshot: destination too small"); return DBM_ERR_INVALID; }
    SnapHeader hd{kSnapMagic, m, lattice, precision};
    char* p = (char*)dst;
    DBM_CUDA(cudaMemcpyAsync(p, &hd, sizeof(hd), cudaMemcpyHostToDevice, s));
    p += snap_align(sizeof(SnapHeader));
    const StateP<P>& S = st[cur];
    if (m > 0) {
      DBM_CUDA(cudaMemcpyAsync(p, S.cell, (size_t)m * 4, cudaMemcpyDeviceToDevice, s));
      p += snap_align((size_t)m * 4);
      DBM_CUDA(cudaMemcpy2DAsync(p, (size_t)m * sizeof(real), S.off, (size_t)mcap * sizeof(real), (size_t)m * sizeof(real),
                                 D, cudaMemcpyDeviceToDevice, s));
      p += snap_align((size_t)D * m * sizeof(real));
      if constexpr (std::is_same<P, PF64>::value) {
        DBM_CUDA(cudaMemcpy2DAsync(p, (size_t)m * 8, S.f64, (size_t)mcap * 8, (size_t)m * 8, Q, cudaMemcpyDeviceToDevice, s));
      } else {
        DBM_CUDA(cudaMemcpyAsync(p, S.rho, (size_t)m * 4, cudaMemcpyDeviceToDevice, s));
        p += snap_align((size_t)m * 4);
        DBM_CUDA(cudaMemcpy2DAsync(p, (size_t)m * 4, S.dev, (size_t)mcap * 4, (size_t)m * 4, Q, cudaMemcpyDeviceToDevice, s));
      }
    }
    DBM_CUDA(cudaStreamSynchronize(s));  // the header lives on this thread's stack
    return DBM_OK;
  }

  // Make a snapshot the current state again (bit for bit) and rebuild its cell ranges.
  int restore(const void* src, int64_t nbytes, cudaStream_t s) override {
    if (!src || nbytes < (int64_t)snap_align(sizeof(SnapHeader))) { set_last_error("restore: bad blob"); return DBM_ERR_INVALID; }
    SnapHeader hd{};
    DBM_CUDA(cudaMemcpy(&hd, src, sizeof(hd), cudaMemcpyDeviceToHost));
    if (hd.magic != kSnapMagic || hd.lattice != lattice || hd.precision != precision) {
      set_last_error("restore: blob is not a snapshot of this kind of simulator");
      return DBM_ERR_INVALID;
    }
    const uint32_t m = hd.m;
    if ((int64_t)m > mcap || (int64_t)snap_bytes(m) > nbytes) { set_last_error("restore: blob too small or too large"); return DBM_ERR_INVALID; }
    DBM_CUDA(cudaEventRecord(ev_in, s));
    DBM_CUDA(cudaStreamWaitEvent(own, ev_in, 0));
    cur = 0;
    ++version;
    bind();
    StateP<P>& S = st[0];
    const char* p = (const char*)src + snap_align(sizeof(SnapHeader));
    if (m > 0) {
      DBM_CUDA(cudaMemcpyAsync(S.cell, p, (size_t)m * 4, cudaMemcpyDeviceToDevice, own));
      p += snap_align((size_t)m * 4);
      DBM_CUDA(cudaMemcpy2DAsync(S.off, (size_t)mcap * sizeof(real), p, (size_t)m * sizeof(real), (size_t)m * sizeof(real),
                                 D, cudaMemcpyDeviceToDevice, own));
      p += snap_align((size_t)D * m * sizeof(real));
      if constexpr (std::is_same<P, PF64>::value) {
        DBM_CUDA(cudaMemcpy2DAsync(S.f64, (size_t)mcap * 8, p, (size_t)m * 8, (size_t)m * 8, Q, cudaMemcpyDeviceToDevice, own));
      } else {
        DBM_CUDA(cudaMemcpyAsync(S.rho, p, (size_t)m * 4, cudaMemcpyDeviceToDevice, own));
        p += snap_align((size_t)m * 4);
        DBM_CUDA(cudaMemcpy2DAsync(S.dev, (size_t)mcap * 4, p, (size_t)m * 4, (size_t)m * 4, Q, cudaMemcpyDeviceToDevice, own));
      }
    }
    DBM_CUDA(cudaMemcpyAsync(S.count, &m, 4, cudaMemcpyHostToDevice, own));
    DBM_CUDA(cudaMemcpyAsync(args.d_P, &m, 4, cudaMemcpyHostToDevice, own));
    launch_cell_start(S.cell, args.d_P, ncells, S.start, own);
    DBM_LAUNCH_CHECK();
    DBM_CUDA(cudaStreamSynchronize(own));  // `m` lives on this thread's stack
    DBM_CUDA(cudaEventRecord(ev_out, own));
    DBM_CUDA(cudaStreamWaitEvent(s, ev_out, 0));
    return DBM_OK;
  }

  int count(int64_t* m, cudaStream_t s) override {
    uint32_t h = 0;
    DBM_TRY(read_word(st[cur].count, 0, 1, s, &h));
    *m = h;
    return DBM_OK;
  }

  int get_state(int32_t* inst_out, void* pos, void* fout, int f32, cudaStream_t s) override {
    bind();
    const unsigned grid = std::min<unsigned>(div_up(mcap, 256), (unsigned)sm_count() * 8);
    if (f32)
      k_export<Q, D, P, float><<<grid, 256, 0, s>>>(args, desc.cell, pow2_cell ? (float)desc.cell : 0.f, inst_out,
                                                    (float*)pos, (float*)fout);
    else
      k_export<Q, D, P, double><<<grid, 256, 0, s>>>(args, desc.cell, 0.f, inst_out, (double*)pos, (double*)fout);
    DBM_LAUNCH_CHECK();
    return DBM_OK;
  }

  int status(uint32_t* flags, int clear, cudaStream_t s) override {
    uint32_t h = 0;
    DBM_TRY(read_word(args.status, clear, 0, s, &h));
    *flags = h;
    return DBM_OK;
  }

  int conservation(double* out, cudaStream_t s) override {
    bind();
    k_conservation<Q, D, P><<<args.n_inst, 256, 0, s>>>(args, out);
    DBM_LAUNCH_CHECK();
    return DBM_OK;
  }

  int trace(int what, void* dst, int64_t nbytes, int64_t* needed, cudaStream_t s) override {
    const void* src = nullptr;
    int64_t sz = 0;
    const Args<Q, D, P>& A = args;
    switch (what) {
      case DBM_TRACE_OCC: src = A.occ; sz = (int64_t)ncells * 4; break;
      case DBM_TRACE_THIN_CNT: src = A.tcnt; sz = (int64_t)ncells * 4; break;
      case DBM_TRACE_CENTROID: src = A.cen; sz = (int64_t)D * ncells * sizeof(real); break;
      case DBM_TRACE_MASK: src = A.mask; sz = (int64_t)ncells * 4; break;
      case DBM_TRACE_FINAL_CELL: src = A.fkey; sz = (int64_t)ncells * 4; break;
      case DBM_TRACE_FINAL_OFF: src = A.foff; sz = (int64_t)D * ncells * sizeof(real); break;
      case DBM_TRACE_SW: src = A.sw; sz = (int64_t)Q * mcap * sizeof(real); break;
      case DBM_TRACE_EMPTY: src = A.emask; sz = ccap * 4; break;
      case DBM_TRACE_FSTAR:
        if constexpr (std::is_same<P, PF64>::value) { src = A.a.f64; sz = (int64_t)Q * mcap * 8; }
        else { src = A.a.dev; sz = (int64_t)Q * mcap * 4; }
        break;
      case DBM_TRACE_CPF:
        if constexpr (std::is_same<P, PF64>::value) { src = A.cpf64; sz = (int64_t)Q * ccap * 8; }
        else {
          sz = (int64_t)2 * Q * ccap * 4;
          if (needed) *needed = sz;
          if (dst) {
            if (nbytes < sz) { set_last_error("trace: destination too small"); return DBM_ERR_INVALID; }
            DBM_CUDA(cudaMemcpyAsync(dst, A.cpfhi, (size_t)Q * ccap * 4, cudaMemcpyDeviceToDevice, s));
            DBM_CUDA(cudaMemcpyAsync((char*)dst + (size_t)Q * ccap * 4, A.cpflo, (size_t)Q * ccap * 4,
                                     cudaMemcpyDeviceToDevice, s));
          }
          return DBM_OK;
        }
        break;
      case DBM_TRACE_SORTED: {
        sz = (int64_t)2 * ncells * 4;
        if (needed) *needed = sz;
        if (dst) {
          if (nbytes < sz) { set_last_error("trace: destination too small"); return DBM_ERR_INVALID; }
          const uint32_t* ks = sorted_in_alt ? k_alt : k_in;
          const uint32_t* vs = sorted_in_alt ? v_alt : v_in;
          DBM_CUDA(cudaMemcpyAsync(dst, ks, (size_t)ncells * 4, cudaMemcpyDeviceToDevice, s));
          DBM_CUDA(cudaMemcpyAsync((char*)dst + (size_t)ncells * 4, vs, (size_t)ncells * 4, cudaMemcpyDeviceToDevice, s));
        }
        return DBM_OK;
      }
      case DBM_TRACE_IMPORT_ORDER: src = import_in_alt ? v_alt : v_in; sz = mcap * 4; break;
      case DBM_TRACE_STATE_CELL: src = A.a.cell; sz = mcap * 4; break;
      case DBM_TRACE_STATE_OFF: src = A.a.off; sz = (int64_t)D * mcap * sizeof(real); break;
      case DBM_TRACE_COUNTS: {
        sz = 8;
        if (needed) *needed = sz;
        if (dst) {
          if (nbytes < sz) { set_last_error("trace: destination too small"); return DBM_ERR_INVALID; }
          DBM_CUDA(cudaMemcpyAsync(dst, A.a.count, 4, cudaMemcpyDeviceToDevice, s));
          DBM_CUDA(cudaMemcpyAsync((char*)dst + 4, A.d_P, 4, cudaMemcpyDeviceToDevice, s));
        }
        return DBM_OK;
      }
      default: set_last_error("trace: unknown buffer %d", what); return DBM_ERR_INVALID;
    }
    if (needed) *needed = sz;
    if (dst) {
      if (nbytes < sz) { set_last_error("trace: destination too small"); return DBM_ERR_INVALID; }
      DBM_CUDA(cudaMemcpyAsync(dst, src, (size_t)sz, cudaMemcpyDeviceToDevice, s));
    }
    return DBM_OK;
  }

  int64_t device_bytes() const override { return bytes; }
};

}  // namespace dbm

using namespace dbm;

template <class P>
static int make_impl(const dbm_sim_desc& d, const dbm_instance_desc* in, int n, SimBase** out) {
  return dispatch_lattice(d.lattice, [&](auto tag) -> int {
    using LT = decltype(tag);
    auto* s = new SimImpl<LT::Q, LT::D, P>();
    int rc = s->init(d, in, n);
    if (rc != DBM_OK) { delete s; return rc; }
    *out = s;
    return DBM_OK;
  });
}

extern "C" {

int dbm_sim_create(const dbm_sim_desc* desc, const dbm_instance_desc* inst, int32_t n_inst, dbm_sim** out) {
  if (!desc || !inst || n_inst < 1 || !out) { set_last_error("dbm_sim_create: bad arguments"); return DBM_ERR_INVALID; }
  if (!(desc->dx > 0) || !(desc->r_res > 0) || !(desc->cell > 0) || desc->moment_capacity < 0) {
    set_last_error("dbm_sim_create: dx, r_res and cell must be > 0");
    return DBM_ERR_INVALID;
  }
  if (desc->precision != DBM_FP64 && desc->precision != DBM_FP32DEV) {
    set_last_error("dbm_sim_create: unknown precision %d", desc->precision);
    return DBM_ERR_INVALID;
  }
  SimBase* impl = nullptr;
  int rc = desc->precision == DBM_FP64 ? make_impl<PF64>(*desc, inst, n_inst, &impl)
                                       : make_impl<PF32>(*desc, inst, n_inst, &impl);
  if (rc != DBM_OK) return rc;
  *out = new dbm_sim{impl};
  return DBM_OK;
}

int dbm_sim_destroy(dbm_sim* s) {
  if (!s) return DBM_OK;
  delete s->impl;
  delete s;
  return DBM_OK;
}

#define SIM_CHECK(s)                                           \
  if (!(s) || !(s)->impl) {                                    \
    set_last_error("null simulator handle");                   \
    return DBM_ERR_INVALID;                                    \
  }

int dbm_sim_set_state(dbm_sim* s, const int32_t* inst, const double* pos, const double* f, int64_t m, void* stream) {
  SIM_CHECK(s);
  return s->impl->load(inst, pos, f, m, 0, (cudaStream_t)stream);
}
int dbm_sim_set_state_sorted(dbm_sim* s, const int32_t* inst, const double* pos, const double* f, int64_t m,
                             void* stream) {
  SIM_CHECK(s);
  return s->impl->load(inst, pos, f, m, SimBase::kLoadPresorted, (cudaStream_t)stream);
}
int dbm_sim_set_state_f32(dbm_sim* s, const int32_t* inst, const float* pos, const float* f, int64_t m,
                          int32_t presorted, void* stream) {
  SIM_CHECK(s);
  const int flags = SimBase::kLoadF32 | (presorted ? SimBase::kLoadPresorted : 0);
  return s->impl->load(inst, pos, f, m, flags, (cudaStream_t)stream);
}
int dbm_sim_step(dbm_sim* s, int32_t steps, void* stream) {
  SIM_CHECK(s);
  return s->impl->step(steps, (cudaStream_t)stream);
}
int dbm_sim_step_partial(dbm_sim* s, int32_t stage, void* stream) {
  SIM_CHECK(s);
  return s->impl->step_partial(stage, (cudaStream_t)stream);
}
int dbm_sim_profile_step(dbm_sim* s, float* stage_ms, void* stream) {
  SIM_CHECK(s);
  if (!stage_ms) return DBM_ERR_INVALID;
  return s->impl->profile_step(stage_ms, (cudaStream_t)stream);
}
int dbm_sim_count(dbm_sim* s, int64_t* m, void* stream) {
  SIM_CHECK(s);
  if (!m) return DBM_ERR_INVALID;
  return s->impl->count(m, (cudaStream_t)stream);
}
int dbm_sim_get_state(dbm_sim* s, int32_t* inst, double* pos, double* f, void* stream) {
  SIM_CHECK(s);
  return s->impl->get_state(inst, pos, f, 0, (cudaStream_t)stream);
}
int dbm_sim_get_state_f32(dbm_sim* s, int32_t* inst, float* pos, float* f, void* stream) {
  SIM_CHECK(s);
  return s->impl->get_state(inst, pos, f, 1, (cudaStream_t)stream);
}
int dbm_sim_status(dbm_sim* s, uint32_t* flags, int32_t clear, void* stream) {
  SIM_CHECK(s);
  if (!flags) return DBM_ERR_INVALID;
  return s->impl->status(flags, clear, (cudaStream_t)stream);
}
int dbm_sim_conservation(dbm_sim* s, double* out, void* stream) {
  SIM_CHECK(s);
  if (!out) return DBM_ERR_INVALID;
  return s->impl->conservation(out, (cudaStream_t)stream);
}
int dbm_sim_set_option(dbm_sim* s, int32_t option, int32_t value) {
  SIM_CHECK(s);
  if (option == DBM_OPT_GRAPHS) s->impl->use_graphs = value ? 1 : 0;
  else if (option == DBM_OPT_TILES) {
    if (!value) DBM_TRY(s->impl->ensure_untiled());
    s->impl->use_tiles = value ? 1 : 0;
  }
  else if (option == DBM_OPT_TILE_WIDTH || option == DBM_OPT_PERSISTENT) {
    int tx = 0, pers = 0;
    s->impl->tiling(&tx, &pers);
    if (option == DBM_OPT_TILE_WIDTH) tx = value; else pers = value;
    return s->impl->set_tiling_v(tx, pers);
  } else if (option == DBM_OPT_KAPPA_SOFT) {
    return s->impl->set_soft_spawn(value);
  } else if (option == DBM_OPT_BRICK_WIDTH) {
    return s->impl->set_brick(value);
  } else if (option == DBM_OPT_SHIFTED_WINDOWS) {
    s->impl->use_shift = value ? 1 : 0;
  } else if (option == DBM_OPT_DENSE_STENCIL) {
    s->impl->use_dense = value ? 1 : 0;
  } else {
    set_last_error("dbm_sim_set_option: unknown option %d", option);
    return DBM_ERR_INVALID;
  }
  s->impl->invalidate_graphs();
  return DBM_OK;
}
int dbm_sim_use_graphs(dbm_sim* s, int32_t on) {
  SIM_CHECK(s);
  s->impl->use_graphs = on ? 1 : 0;
  return DBM_OK;
}
int dbm_sim_trace(dbm_sim* s, int32_t what, void* dst, int64_t bytes, int64_t* needed, void* stream) {
  SIM_CHECK(s);
  return s->impl->trace(what, dst, bytes, needed, (cudaStream_t)stream);
}
int64_t dbm_sim_device_bytes(dbm_sim* s) {
  if (!s || !s->impl) return -1;
  return s->impl->device_bytes();
}
int dbm_sim_get_brick_width(dbm_sim* s, int32_t* brick_width) {
  SIM_CHECK(s);
  if (!brick_width) return DBM_ERR_INVALID;
  *brick_width = s->impl->brick_width();
  return DBM_OK;
}
int dbm_sim_get_tiling(dbm_sim* s, int32_t* tile_width, int32_t* persistent) {
  SIM_CHECK(s);
  if (!tile_width || !persistent) return DBM_ERR_INVALID;
  int tx = 0, pers = 0;
  DBM_TRY(s->impl->tiling(&tx, &pers));
  *tile_width = tx;
  *persistent = pers;
  return DBM_OK;
}
int dbm_sim_set_tau(dbm_sim* s, const double* tau, int32_t n) {
  SIM_CHECK(s);
  if (!tau) { set_last_error("dbm_sim_set_tau: null tau"); return DBM_ERR_INVALID; }
  return s->impl->set_tau(tau, n);
}
int dbm_sim_set_obstacle(dbm_sim* s, int32_t inst, const double* center, double radius) {
  SIM_CHECK(s);
  return s->impl->set_obstacle(inst, center, radius);
}
int dbm_sim_set_inflow(dbm_sim* s, int32_t inst, const double* u, int32_t width) {
  SIM_CHECK(s);
  return s->impl->set_inflow(inst, u, width);
}
int dbm_sim_snapshot(dbm_sim* s, void* dst, int64_t bytes, int64_t* needed, void* stream) {
  SIM_CHECK(s);
  return s->impl->snapshot(dst, bytes, needed, (cudaStream_t)stream);
}
int dbm_sim_restore(dbm_sim* s, const void* src, int64_t bytes, void* stream) {
  SIM_CHECK(s);
  return s->impl->restore(src, bytes, (cudaStream_t)stream);
}

}  // extern "C"
