// Shared definitions for the DiReBM GB300 library (sm_103a).
#pragma once

#include <cuda_runtime.h>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>

#include "../../include/direbm_gb300.h"

namespace dbm {

// ---- error plumbing (no exceptions cross the C ABI) ------------------------------------------
void set_last_error(const char* fmt, ...);
const char* last_error();

#define DBM_CUDA(expr)                                                                      \
  do {                                                                                      \
    cudaError_t _e = (expr);                                                                \
    if (_e != cudaSuccess) {                                                                \
      ::dbm::set_last_error("%s:%d %s -> %s", __FILE__, __LINE__, #expr,                   \
                            cudaGetErrorString(_e));                                        \
      return DBM_ERR_CUDA;                                                                  \
    }                                                                                       \
  } while (0)

#define DBM_TRY(expr)               \
  do {                              \
    int _s = (expr);                \
    if (_s != DBM_OK) return _s;    \
  } while (0)

// Every kernel launch in the library goes through this counter so callers can report how many
// of the library's kernels ran inside a timed region.
extern unsigned long long g_launches;
inline void count_launch(unsigned long long n = 1) { g_launches += n; }

#define DBM_LAUNCH_CHECK()                                                                 \
  do {                                                                                      \
    ::dbm::count_launch();                                                                  \
    cudaError_t _e = cudaGetLastError();                                                    \
    if (_e != cudaSuccess) {                                                                \
      ::dbm::set_last_error("%s:%d launch -> %s", __FILE__, __LINE__, cudaGetErrorString(_e)); \
      return DBM_ERR_CUDA;                                                                  \
    }                                                                                       \
  } while (0)

inline unsigned int div_up(long long a, long long b) { return (unsigned int)((a + b - 1) / b); }

// Number of SMs of the current device (152 on GB300); grids of grid-stride kernels are sized as
// a multiple of it.
int sm_count();

// ---- status word bits written by kernels ----------------------------------------------------
enum : uint32_t {
  ST_OUT_OF_BOX = 1u << 0,      // a component or control point left a non-periodic box
  ST_CAPACITY = 1u << 1,        // a buffer would overflow its capacity
  ST_NONFINITE = 1u << 2,       // a non-finite value was produced
  ST_BAD_INPUT = 1u << 3,       // set_state got a position outside its box
  ST_INTERNAL = 1u << 4,        // an internal consistency check failed (a bug: please report)
};

// ---- round-to-nearest arithmetic with no contraction -----------------------------------------
// Integer decisions (cell keys, the inclusive radius test) must be bit-identical to the CPU
// oracle, which evaluates each operation with IEEE round-to-nearest and never fuses a multiply
// with an add.  These wrappers pin that order for both precisions.
__device__ __forceinline__ double rn_add(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double rn_sub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double rn_mul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double rn_sqrt(double a) { return __dsqrt_rn(a); }
__device__ __forceinline__ float rn_add(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float rn_sub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float rn_mul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float rn_sqrt(float a) { return __fsqrt_rn(a); }
// Square root for bounds only (PTX sqrt.approx.f32, one instruction, relative error near 2^-23);
// callers inflate the result far beyond that error.
__device__ __forceinline__ float bound_sqrt(float a) {
  float r;
  asm("sqrt.approx.f32 %0, %1;" : "=f"(r) : "f"(a));
  return r;
}

template <class T>
__device__ __forceinline__ int ifloor(T x) { return (int)floor(x); }

// ---- compensated FP32 accumulation ----------------------------------------------------------
// Neumaier/TwoSum accumulation: the sum is carried as hi + lo.  With TwoProd terms it keeps
// products exact as well, so a sum of FP32 products is accurate to about 2^-44 relative.
struct CSum {
  float hi = 0.f, lo = 0.f;
  __device__ __forceinline__ void add(float x) {
    float t = __fadd_rn(hi, x);
    float bp = __fsub_rn(t, hi);
    float e = __fadd_rn(__fsub_rn(hi, __fsub_rn(t, bp)), __fsub_rn(x, bp));
    hi = t;
    lo = __fadd_rn(lo, e);
  }
  __device__ __forceinline__ void add_prod(float a, float b) {
    float p = __fmul_rn(a, b);
    float e = __fmaf_rn(a, b, -p);
    add(p);
    lo = __fadd_rn(lo, e);
  }
  __device__ __forceinline__ float value() const { return __fadd_rn(hi, lo); }
};

// Minimal double-float helpers (value = hi + lo, |lo| <= ulp(hi)/2 after renormalisation).
struct DF {
  float hi, lo;
};
__device__ __forceinline__ DF df_two_sum(float a, float b) {
  float s = __fadd_rn(a, b);
  float bp = __fsub_rn(s, a);
  float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bp)), __fsub_rn(b, bp));
  return {s, e};
}
__device__ __forceinline__ DF df_norm(float hi, float lo) { return df_two_sum(hi, lo); }
__device__ __forceinline__ DF df_add(DF a, DF b) {
  DF s = df_two_sum(a.hi, b.hi);
  float lo = __fadd_rn(s.lo, __fadd_rn(a.lo, b.lo));
  return df_norm(s.hi, lo);
}
__device__ __forceinline__ DF df_neg(DF a) { return {-a.hi, -a.lo}; }
// (w.hi + w.lo) * (x.hi + x.lo) to double-float accuracy.
__device__ __forceinline__ DF df_mul(DF w, DF x) {
  float p = __fmul_rn(w.hi, x.hi);
  float e = __fmaf_rn(w.hi, x.hi, -p);
  e = __fmaf_rn(w.hi, x.lo, e);
  e = __fmaf_rn(w.lo, x.hi, e);
  return df_norm(p, e);
}
__device__ __forceinline__ float df_float(DF a) { return __fadd_rn(a.hi, a.lo); }

}  // namespace dbm
