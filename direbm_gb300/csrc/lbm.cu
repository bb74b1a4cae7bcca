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
// sum(dev) and u = sum(dev*c)/rho are formed from small numbers and keep their precision.
#include "lattice.cuh"

namespace dbm {

// Axial shift (di, dj) of each D2Q7 direction (direbm/lbm.py:23, warp/lbm.py:18-20).
__constant__ int c_lbm_di[7] = {0, 1, 0, -1, -1, 0, 1};
__constant__ int c_lbm_dj[7] = {0, 0, 1, 1, 0, -1, -1};

template <class T>
__global__ void __launch_bounds__(256) k_lbm_f64(const T* __restrict__ src, T* __restrict__ dst, int ni, int nj,
                                                 int runs, const double* __restrict__ taus, LatK<7, 2> L) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int jr = blockIdx.y;
  if (i >= ni) return;
  const int j = jr % nj, r = jr / nj;
  const int64_t plane = (int64_t)ni * nj;
  const T* s = src + (int64_t)r * 7 * plane + (int64_t)j * ni + i;
  T f[7];
#pragma unroll
  for (int k = 0; k < 7; ++k) f[k] = s[k * plane];
  collide_moment<7, 2, T>(f, (T)taus[r], L);
  T* d = dst + (int64_t)r * 7 * plane;
#pragma unroll
  for (int k = 0; k < 7; ++k) {
    int ii = i + c_lbm_di[k];
    int jj = j + c_lbm_dj[k];
    ii = ii < 0 ? ii + ni : (ii >= ni ? ii - ni : ii);
    jj = jj < 0 ? jj + nj : (jj >= nj ? jj - nj : jj);
    d[k * plane + (int64_t)jj * ni + ii] = f[k];
  }
}

__global__ void __launch_bounds__(256, 8) k_lbm_dev(const float* __restrict__ src, float* __restrict__ dst, int ni,
                                                    int nj, int runs, const double* __restrict__ taus, float rho0,
                                                    LatK<7, 2> L) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int jr = blockIdx.y;
  const int j = jr % nj, r = jr / nj;
  const int64_t plane = (int64_t)ni * nj;
  const bool live = i < ni;
  float dv[7];
  if (live) {
    const float* s = src + (int64_t)r * 7 * plane + (int64_t)j * ni + i;
#pragma unroll
    for (int k = 0; k < 7; ++k) dv[k] = s[k * plane];
  }
  // One block covers one row of one run, so 1/tau is formed once per block, while the loads
  // above are in flight: an FP64 divide in every thread made the narrow FP64 pipe the limiter.
  __shared__ float s_inv_tau;
  if (threadIdx.x == 0) s_inv_tau = (float)(1.0 / taus[r]);
  __syncthreads();
  if (!live) return;
  // rho - rho0 and momentum from the deviations only
  float drho = 0.f, mx = 0.f, my = 0.f;
#pragma unroll
  for (int k = 0; k < 7; ++k) {
    drho += dv[k];
    mx += dv[k] * L.cf[k][0];
    my += dv[k] * L.cf[k][1];
  }
  const float rho = rho0 + drho;
  const float u[2] = {mx / rho, my / rho};
  float deq[7];
  eq_deviation_f32<7, 2>(rho, u, L, deq);  // rho*W*(...) without the rest part
  const float inv_tau = s_inv_tau;
  float* d = dst + (int64_t)r * 7 * plane;
#pragma unroll
  for (int k = 0; k < 7; ++k) {
    // feq - W*rho0 = W*(rho - rho0) + rho*W*(...)
    const float target = L.wf[k] * drho + deq[k];
    const float out = dv[k] + (target - dv[k]) * inv_tau;
    int ii = i + c_lbm_di[k];
    int jj = j + c_lbm_dj[k];
    ii = ii < 0 ? ii + ni : (ii >= ni ? ii - ni : ii);
    jj = jj < 0 ? jj + nj : (jj >= nj ? jj - nj : jj);
    d[k * plane + (int64_t)jj * ni + ii] = out;
  }
}

static int lbm_launch(int precision, const void* src, void* dst, int ni, int nj, int runs, const double* taus,
                      double rho0, const LatK<7, 2>& L, cudaStream_t s) {
  const int bx = ni >= 256 ? 256 : ((ni + 31) / 32) * 32;
  dim3 grid(div_up(ni, bx), (unsigned)(nj * runs));
  if (precision == DBM_FP64) {
    k_lbm_f64<double><<<grid, bx, 0, s>>>((const double*)src, (double*)dst, ni, nj, runs, taus, L);
  } else {
    k_lbm_dev<<<grid, bx, 0, s>>>((const float*)src, (float*)dst, ni, nj, runs, taus, (float)rho0, L);
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
