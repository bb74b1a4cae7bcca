// Hexagonal D2Q7 lattice Boltzmann: one fused push collide-stream kernel.
//
// Replaces direbm/warp/lbm.py:24-105, where a step is two Warp kernels over an (nj, ni, 7)
// array-of-structures (_lbm_collide in place, then _lbm_stream gathering each direction from its
// axial-shifted neighbour into a second array).  Here each thread reads the 7 populations of its
// node once (structure-of-arrays: every direction is a contiguous plane, so a warp's loads are
// coalesced), relaxes them, and writes population k straight to the neighbour (i+di_k, j+dj_k)
// in the destination plane k -- the collide-then-stream order of direbm/lbm.py:60-62 with one
// read and one write of f per node-step (56 B in FP32, 112 B in FP64).
//
// FP32DEV stores dev_k = f_k - W_k*rho0: the rest part carries no momentum, so rho = rho0 +
// sum(dev) and u = sum(dev*c)/rho are formed from small numbers and keep their precision.  The
// FP32 equilibrium is projected back onto the node's mass and momentum before the relaxation
// (conserve_moments_f32): without it the FP32-rounded weights give each collision a spurious
// momentum of ~3e-8 rho u, which slows the decay of a weak shear wave by several percent.
#include "lattice.cuh"

namespace dbm {

// Axial shift (di, dj) of each D2Q7 direction (direbm/lbm.py:23, warp/lbm.py:18-20), as
// compile-time constants so that every unrolled store resolves its neighbour row and column to a
// register chosen at compile time (no per-direction wrap arithmetic).
__host__ __device__ constexpr int lbm_di(int k) { return (k == 1 || k == 6) ? 1 : ((k == 3 || k == 4) ? -1 : 0); }
__host__ __device__ constexpr int lbm_dj(int k) { return (k == 2 || k == 3) ? 1 : ((k == 5 || k == 6) ? -1 : 0); }
// Rows (of one run) per block: 1/tau is formed once per block, so its barrier and the block's
// index set-up are shared by this many node rows.
constexpr int kLbmRows = 8;

// Wrapped neighbour columns {i-1, i, i+1} and row offsets {(j-1) ni, j ni, (j+1) ni}.
template <class IDX>
struct HexNbr {
  int col[3];
  IDX row[3];
  __device__ __forceinline__ HexNbr(int i, int j, int ni, int nj) {
    col[0] = i == 0 ? ni - 1 : i - 1;
    col[1] = i;
    col[2] = i + 1 == ni ? 0 : i + 1;
    row[0] = (IDX)(j == 0 ? nj - 1 : j - 1) * ni;
    row[1] = (IDX)j * ni;
    row[2] = (IDX)(j + 1 == nj ? 0 : j + 1) * ni;
  }
  template <int k>
  __device__ __forceinline__ IDX at() const { return row[lbm_dj(k) + 1] + col[lbm_di(k) + 1]; }
};

template <class IDX, int k>
struct HexStore {
  template <class T>
  __device__ __forceinline__ static void put(T* d, IDX plane, const HexNbr<IDX>& nb, const T (&v)[7]) {
    d[(IDX)k * plane + nb.template at<k>()] = v[k];
    HexStore<IDX, k + 1>::put(d, plane, nb, v);
  }
};
template <class IDX>
struct HexStore<IDX, 7> {
  template <class T>
  __device__ __forceinline__ static void put(T*, IDX, const HexNbr<IDX>&, const T (&)[7]) {}
};

// Block (x, y): columns x*blockDim.x.., rows kLbmRows * (y mod bpr).. of run y / bpr.
__device__ __forceinline__ void lbm_block_rows(int nj, int* r, int* j0, int* j1) {
  const int bpr = (nj + kLbmRows - 1) / kLbmRows;
  *r = blockIdx.y / bpr;
  *j0 = (blockIdx.y - *r * bpr) * kLbmRows;
  *j1 = min(*j0 + kLbmRows, nj);
}

// FP64: BGK with the reference's formula (direbm/lbm.py:44-62: rho = sum f, u = sum f c / rho,
// f += (feq - f) / tau), the divisions by rho and tau taken as products with one reciprocal each.
template <class IDX>
__global__ void __launch_bounds__(256) k_lbm_f64(const double* __restrict__ src, double* __restrict__ dst, int ni,
                                                 int nj, const double* __restrict__ taus, LatK<7, 2> L) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  int r, j0, j1;
  lbm_block_rows(nj, &r, &j0, &j1);
  if (i >= ni) return;
  const double inv_tau = 1.0 / taus[r];  // uniform in the block: one divide per thread row group
  const IDX plane = (IDX)ni * nj;
  const double* s = src + (IDX)r * 7 * plane;
  double* d = dst + (IDX)r * 7 * plane;
  for (int j = j0; j < j1; ++j) {
    const HexNbr<IDX> nb(i, j, ni, nj);
    double f[7];
#pragma unroll
    for (int k = 0; k < 7; ++k) f[k] = s[(IDX)k * plane + nb.row[1] + i];
    double rho = 0, mx = 0, my = 0;
#pragma unroll
    for (int k = 0; k < 7; ++k) {
      rho += f[k];
      mx += f[k] * L.c[k][0];
      my += f[k] * L.c[k][1];
    }
    const double ir = 1.0 / rho;
    const double u[2] = {mx * ir, my * ir};
    double feq[7];
    equilibrium_all<7, 2, double>(rho, u, L, feq);
    double out[7];
#pragma unroll
    for (int k = 0; k < 7; ++k) out[k] = f[k] + (feq[k] - f[k]) * inv_tau;
    HexStore<IDX, 0>::put(d, plane, nb, out);
  }
}

template <class IDX>
__global__ void __launch_bounds__(256, 8) k_lbm_dev(const float* __restrict__ src, float* __restrict__ dst, int ni,
                                                    int nj, const double* __restrict__ taus, float rho0,
                                                    LatK<7, 2> L) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  int r, j0, j1;
  lbm_block_rows(nj, &r, &j0, &j1);
  // the FP64 1/tau once per block (a divide per thread would keep the narrow FP64 pipe busy)
  __shared__ float s_inv_tau;
  if (threadIdx.x == 0) s_inv_tau = (float)(1.0 / taus[r]);
  __syncthreads();
  if (i >= ni) return;
  const float inv_tau = s_inv_tau;
  const IDX plane = (IDX)ni * nj;
  const float* s = src + (IDX)r * 7 * plane;
  float* d = dst + (IDX)r * 7 * plane;
  for (int j = j0; j < j1; ++j) {
    const HexNbr<IDX> nb(i, j, ni, nj);
    float dv[7];
#pragma unroll
    for (int k = 0; k < 7; ++k) dv[k] = s[(IDX)k * plane + nb.row[1] + i];
    // rho - rho0 and momentum from the deviations only
    float drho = 0.f, mx = 0.f, my = 0.f;
#pragma unroll
    for (int k = 0; k < 7; ++k) {
      drho += dv[k];
      mx += dv[k] * L.cf[k][0];
      my += dv[k] * L.cf[k][1];
    }
    const float rho = rho0 + drho;
    const float ir = __frcp_rn(rho);
    const float u[2] = {mx * ir, my * ir};
    float deq[7];
    eq_deviation_f32<7, 2>(rho, u, L, deq);  // rho*W*(...) without the rest part
    // feq - W*rho0 = W*(rho - rho0) + rho*W*(...), projected onto the node's mass and momentum
#pragma unroll
    for (int k = 0; k < 7; ++k) deq[k] += L.wf[k] * drho;
    const float j0[2] = {mx, my};
    conserve_moments_f32<7, 2>(deq, drho, j0, L);
    float out[7];
#pragma unroll
    for (int k = 0; k < 7; ++k) out[k] = dv[k] + (deq[k] - dv[k]) * inv_tau;
    HexStore<IDX, 0>::put(d, plane, nb, out);
  }
}

static int lbm_launch(int precision, const void* src, void* dst, int ni, int nj, int runs, const double* taus,
                      double rho0, const LatK<7, 2>& L, cudaStream_t s) {
  const int bx = ni >= 256 ? 256 : ((ni + 31) / 32) * 32;
  const int64_t bpr = (nj + kLbmRows - 1) / kLbmRows;
  dim3 grid(div_up(ni, bx), (unsigned)(bpr * runs));
  const bool small = (int64_t)7 * runs * (int64_t)ni * nj < 2147483647LL;  // 32-bit element indices
  if (precision == DBM_FP64) {
    if (small) k_lbm_f64<int><<<grid, bx, 0, s>>>((const double*)src, (double*)dst, ni, nj, taus, L);
    else k_lbm_f64<int64_t><<<grid, bx, 0, s>>>((const double*)src, (double*)dst, ni, nj, taus, L);
  } else {
    if (small) k_lbm_dev<int><<<grid, bx, 0, s>>>((const float*)src, (float*)dst, ni, nj, taus, (float)rho0, L);
    else k_lbm_dev<int64_t><<<grid, bx, 0, s>>>((const float*)src, (float*)dst, ni, nj, taus, (float)rho0, L);
  }
  DBM_LAUNCH_CHECK();
  return DBM_OK;
}

}  // namespace dbm

using namespace dbm;

extern "C" int dbm_lbm_step(int precision, const void* src, void* dst, int32_t ni, int32_t nj, int32_t runs,
                            const double* taus, double rho0, int32_t steps, void* tmp, void* stream) {
  if ((precision != DBM_FP64 && precision != DBM_FP32DEV) || ni < 1 || nj < 1 || runs < 1 || steps < 0 || !src ||
      !dst || !taus || (steps > 1 && !tmp) || (int64_t)nj * runs > 2147483647LL) {
    set_last_error("dbm_lbm_step: bad arguments");
    return DBM_ERR_INVALID;
  }
  if (src == dst) {
    set_last_error("dbm_lbm_step: src and dst must differ (push streaming)");
    return DBM_ERR_INVALID;
  }
  cudaStream_t s = (cudaStream_t)stream;
  auto L = make_latk<7, 2>(*lat_host(DBM_D2Q7), 1.0, 1.0);
  const void* cur = src;
  for (int st = 1; st <= steps; ++st) {
    void* target = ((steps - st) % 2 == 0) ? dst : tmp;
    DBM_TRY(lbm_launch(precision, cur, target, ni, nj, runs, taus, rho0, L, s));
    cur = target;
  }
  if (steps == 0) {
    const size_t bytes = (size_t)ni * nj * runs * 7 * (precision == DBM_FP64 ? 8 : 4);
    DBM_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToDevice, s));
  }
  return DBM_OK;
}
