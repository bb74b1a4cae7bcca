// Velocity sets and BGK device functions.
//
// D2Q7 and D3Q13 follow the reference tables (direbm/constants.py:15-36, direbm/lattices.py:44-61);
// D2Q9 and D3Q19 are the standard square / cubic sets.  The equilibrium is the reference's
// second-order form with the lattice's cs^2 (direbm/physics.py:29-45, warp/physics.py:31-42).
#pragma once

#include <cmath>

#include "common.cuh"

namespace dbm {

struct LatHost {
  int Q, D;
  double c[19][3];
  double w[19];
  double cs2;
};

// Returns nullptr for an unknown id.
const LatHost* lat_host(int id);

template <int Q_, int D_>
struct Lat {
  static constexpr int Q = Q_;
  static constexpr int D = D_;
};
using LD2Q7 = Lat<7, 2>;
using LD2Q9 = Lat<9, 2>;
using LD3Q13 = Lat<13, 3>;
using LD3Q19 = Lat<19, 3>;

// Kernel-side constants (passed by value in kernel parameter space).
template <int Q, int D>
struct LatK {
  double c[Q][D];
  double w[Q];
  float cf[Q][D];
  float wf[Q];     // W rounded to float
  float wlo[Q];    // W - wf (so W = wf + wlo to double-float accuracy)
  double cd[Q][D]; // c * dx / cell (cell units)
  float cdf[Q][D]; // float(c * dx / cell)
  double inv_cs2;
  float inv_cs2f;  // float(1/cs^2): a double->float conversion runs on the narrow FP64 pipe
  int opp[Q];      // index of -c_k

  // 1/cs^2 in the arithmetic type T, without a per-thread conversion for T = float
  template <class T>
  __host__ __device__ __forceinline__ T inv_cs2_as() const {
    if constexpr (sizeof(T) == sizeof(float)) return inv_cs2f; else return (T)inv_cs2;
  }
  template <class T>
  __host__ __device__ __forceinline__ T c_as(int k, int a) const {
    if constexpr (sizeof(T) == sizeof(float)) return cf[k][a]; else return (T)c[k][a];
  }
  template <class T>
  __host__ __device__ __forceinline__ T cd_as(int k, int a) const {
    if constexpr (sizeof(T) == sizeof(float)) return cdf[k][a]; else return (T)cd[k][a];
  }
  template <class T>
  __host__ __device__ __forceinline__ T w_as(int k) const {
    if constexpr (sizeof(T) == sizeof(float)) return wf[k]; else return (T)w[k];
  }
};

template <int Q, int D>
LatK<Q, D> make_latk(const LatHost& h, double dx, double cell) {
  LatK<Q, D> k{};
  for (int q = 0; q < Q; ++q) {
    k.w[q] = h.w[q];
    k.wf[q] = (float)h.w[q];
    k.wlo[q] = (float)(h.w[q] - (double)k.wf[q]);
    for (int a = 0; a < D; ++a) {
      k.c[q][a] = h.c[q][a];
      k.cf[q][a] = (float)h.c[q][a];
      double v = h.c[q][a] * dx / cell;
      k.cd[q][a] = v;
      k.cdf[q][a] = (float)v;
    }
  }
  k.inv_cs2 = 1.0 / h.cs2;
  k.inv_cs2f = (float)k.inv_cs2;
  for (int q = 0; q < Q; ++q) {
    k.opp[q] = q;
    for (int r = 0; r < Q; ++r) {
      bool neg = true;
      for (int a = 0; a < D; ++a) neg = neg && std::fabs(h.c[r][a] + h.c[q][a]) < 1e-12;
      if (neg) { k.opp[q] = r; break; }
    }
  }
  return k;
}

// f_eq of (rho, u) for all directions, in T arithmetic (reference formula and operation order).
template <int Q, int D, class T>
__device__ __forceinline__ void equilibrium_all(T rho, const T (&u)[D], const LatK<Q, D>& L, T (&feq)[Q]) {
  const T inv = L.template inv_cs2_as<T>();
  T usq = 0;
#pragma unroll
  for (int a = 0; a < D; ++a) usq += u[a] * u[a];
#pragma unroll
  for (int k = 0; k < Q; ++k) {
    T cu = 0;
#pragma unroll
    for (int a = 0; a < D; ++a) cu += L.template c_as<T>(k, a) * u[a];
    T br = (T)1 + inv * cu + (T)0.5 * inv * inv * cu * cu - (T)0.5 * inv * usq;
    feq[k] = rho * L.template w_as<T>(k) * br;
  }
}

// Deviation of f_eq from the rest part rho*W:  rho*W_k*(cu/cs^2 + (cu)^2/(2cs^4) - u^2/(2cs^2)).
template <int Q, int D>
__device__ __forceinline__ void eq_deviation_f32(float rho, const float (&u)[D], const LatK<Q, D>& L,
                                                 float (&deq)[Q]) {
  const float inv = L.inv_cs2f;
  float usq = 0.f;
#pragma unroll
  for (int a = 0; a < D; ++a) usq += u[a] * u[a];
#pragma unroll
  for (int k = 0; k < Q; ++k) {
    float cu = 0.f;
#pragma unroll
    for (int a = 0; a < D; ++a) cu += L.cf[k][a] * u[a];
    float br = inv * cu + 0.5f * inv * inv * cu * cu - 0.5f * inv * usq;
    deq[k] = rho * L.wf[k] * br;
  }
}

// Restore the conserved moments of an FP32 equilibrium vector t: t_k -= W_k (dm + c_k . dj / cs^2)
// with dm = sum t - m0 and dj = sum t c - j0.  With the lattice's FP32-rounded weights, sum W c c
// differs from cs^2 I by a few 1e-8 (12 * float(1/12) = 1 + 3e-8 for D2Q7), so an unprojected
// equilibrium carries that fraction of rho u as extra momentum, and every collision adds
// (1/tau) of it: a steady forcing that a slowly decaying flow integrates (the hex shear wave of
// amplitude 0.01 at 1024^2, tau 0.55, decays 6e-7 per step and would decay ~8 % too slowly).  In
// exact arithmetic dm = dj = 0 and the projection is the identity; computed, it leaves the
// rounding error of the sums, of either sign.
template <int Q, int D>
__device__ __forceinline__ void conserve_moments_f32(float (&t)[Q], float m0, const float (&j0)[D],
                                                     const LatK<Q, D>& L) {
  float dm = -m0, dj[D];
#pragma unroll
  for (int a = 0; a < D; ++a) dj[a] = -j0[a];
#pragma unroll
  for (int k = 0; k < Q; ++k) {
    dm += t[k];
#pragma unroll
    for (int a = 0; a < D; ++a) dj[a] += t[k] * L.cf[k][a];
  }
#pragma unroll
  for (int k = 0; k < Q; ++k) {
    float cj = 0.f;
#pragma unroll
    for (int a = 0; a < D; ++a) cj += L.cf[k][a] * dj[a];
    t[k] -= L.wf[k] * (dm + L.inv_cs2f * cj);
  }
}

// BGK collision of one moment in place (FP64 / generic T): rho = sum f, u = sum f c / rho
// (no vacuum guard, as the GPU path of the reference), f += (feq - f)/tau.
template <int Q, int D, class T>
__device__ __forceinline__ void collide_moment(T (&f)[Q], T tau, const LatK<Q, D>& L) {
  T rho = 0;
  T mom[D];
#pragma unroll
  for (int a = 0; a < D; ++a) mom[a] = 0;
#pragma unroll
  for (int k = 0; k < Q; ++k) {
    rho += f[k];
#pragma unroll
    for (int a = 0; a < D; ++a) mom[a] += f[k] * L.template c_as<T>(k, a);
  }
  T u[D];
#pragma unroll
  for (int a = 0; a < D; ++a) u[a] = mom[a] / rho;
  T feq[Q];
  equilibrium_all<Q, D, T>(rho, u, L, feq);
#pragma unroll
  for (int k = 0; k < Q; ++k) f[k] = f[k] + (feq[k] - f[k]) / tau;
}

// BGK collision in the deviation store: f_k = rho*W_k + dev_k, rho is invariant, u = sum dev c / rho;
// the equilibrium is projected onto the deviations' mass and momentum (conserve_moments_f32).
template <int Q, int D>
__device__ __forceinline__ void collide_moment_dev(float rho, float (&dev)[Q], float tau, const LatK<Q, D>& L) {
  float mom[D];
#pragma unroll
  for (int a = 0; a < D; ++a) mom[a] = 0.f;
#pragma unroll
  for (int k = 0; k < Q; ++k) {
#pragma unroll
    for (int a = 0; a < D; ++a) mom[a] += dev[k] * L.cf[k][a];
  }
  float u[D];
#pragma unroll
  for (int a = 0; a < D; ++a) u[a] = mom[a] / rho;
  float deq[Q];
  eq_deviation_f32<Q, D>(rho, u, L, deq);
  float m0 = 0.f;  // the deviations' own mass (zero up to rounding): rho itself is stored apart
#pragma unroll
  for (int k = 0; k < Q; ++k) m0 += dev[k];
  conserve_moments_f32<Q, D>(deq, m0, mom, L);
  const float inv_tau = 1.0f / tau;
#pragma unroll
  for (int k = 0; k < Q; ++k) dev[k] = dev[k] + (deq[k] - dev[k]) * inv_tau;
}

// Dispatch a lambda on the lattice id with a Lat<Q,D> tag.
template <class F>
int dispatch_lattice(int id, F&& fn) {
  switch (id) {
    case DBM_D2Q7: return fn(LD2Q7{});
    case DBM_D2Q9: return fn(LD2Q9{});
    case DBM_D3Q13: return fn(LD3Q13{});
    case DBM_D3Q19: return fn(LD3Q19{});
    default: set_last_error("unknown lattice id %d", id); return DBM_ERR_INVALID;
  }
}

}  // namespace dbm
