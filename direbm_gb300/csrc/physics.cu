// Library plumbing (errors, launch counter, lattice tables) and the BGK kernels on explicit arrays.
//
// dbm_collide_* / dbm_equilibrium_* replace direbm/warp/physics.py:78-97 (collide, equilibrium),
// whose Warp kernels _collide / _equilibrium (physics.py:45-75) run one thread per row of an
// (n, 7) array.  Here rows of any lattice are processed by one thread each; the row-major layout
// of the reference is kept because these entry points exchange arrays with numpy callers.
#include <cmath>
#include <cstdarg>
#include <mutex>

#include "lattice.cuh"

namespace dbm {

static thread_local char g_err[1024] = "";
unsigned long long g_launches = 0;

void set_last_error(const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof(g_err), fmt, ap);
  va_end(ap);
}
const char* last_error() { return g_err; }

int sm_count() {
  static int n = 0;
  if (n == 0) {
    int dev = 0;
    cudaGetDevice(&dev);
    if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0) n = 152;
  }
  return n;
}

static LatHost make_tables(int id) {
  LatHost h{};
  const double s = std::sqrt(3.0) / 2.0;
  if (id == DBM_D2Q7) {
    h.Q = 7; h.D = 2; h.cs2 = 0.25;
    const double c[7][2] = {{0, 0}, {1, 0}, {0.5, s}, {-0.5, s}, {-1, 0}, {-0.5, -s}, {0.5, -s}};
    for (int k = 0; k < 7; ++k) { h.c[k][0] = c[k][0]; h.c[k][1] = c[k][1]; h.w[k] = k ? 1.0 / 12.0 : 0.5; }
  } else if (id == DBM_D2Q9) {
    h.Q = 9; h.D = 2; h.cs2 = 1.0 / 3.0;
    const int c[9][2] = {{0, 0}, {1, 0}, {0, 1}, {-1, 0}, {0, -1}, {1, 1}, {-1, 1}, {-1, -1}, {1, -1}};
    for (int k = 0; k < 9; ++k) {
      h.c[k][0] = c[k][0]; h.c[k][1] = c[k][1];
      h.w[k] = k == 0 ? 4.0 / 9.0 : (k < 5 ? 1.0 / 9.0 : 1.0 / 36.0);
    }
  } else if (id == DBM_D3Q13) {
    h.Q = 13; h.D = 3; h.cs2 = 0.2;
    const double p = (1.0 + std::sqrt(5.0)) / 2.0;
    const double ico[12][3] = {{0, 1, p}, {0, 1, -p}, {0, -1, p}, {0, -1, -p}, {1, p, 0}, {1, -p, 0},
                               {-1, p, 0}, {-1, -p, 0}, {p, 0, 1}, {p, 0, -1}, {-p, 0, 1}, {-p, 0, -1}};
    const double nrm = std::sqrt(1.0 + p * p);
    h.c[0][0] = h.c[0][1] = h.c[0][2] = 0.0;
    h.w[0] = 2.0 / 5.0;
    for (int k = 0; k < 12; ++k) {
      for (int a = 0; a < 3; ++a) h.c[k + 1][a] = ico[k][a] / nrm;
      h.w[k + 1] = 1.0 / 20.0;
    }
  } else if (id == DBM_D3Q19) {
    h.Q = 19; h.D = 3; h.cs2 = 1.0 / 3.0;
    const int c[19][3] = {{0, 0, 0}, {1, 0, 0}, {-1, 0, 0}, {0, 1, 0}, {0, -1, 0}, {0, 0, 1}, {0, 0, -1},
                          {1, 1, 0}, {-1, -1, 0}, {1, -1, 0}, {-1, 1, 0}, {1, 0, 1}, {-1, 0, -1},
                          {1, 0, -1}, {-1, 0, 1}, {0, 1, 1}, {0, -1, -1}, {0, 1, -1}, {0, -1, 1}};
    for (int k = 0; k < 19; ++k) {
      for (int a = 0; a < 3; ++a) h.c[k][a] = c[k][a];
      h.w[k] = k == 0 ? 1.0 / 3.0 : (k < 7 ? 1.0 / 18.0 : 1.0 / 36.0);
    }
  } else {
    h.Q = 0;
  }
  return h;
}

const LatHost* lat_host(int id) {
  static LatHost tables[4];
  static std::once_flag once;
  std::call_once(once, [] {
    for (int i = 0; i < 4; ++i) tables[i] = make_tables(i);
  });
  if (id < 0 || id > 3) return nullptr;
  return &tables[id];
}

// ---- kernels -----------------------------------------------------------------------------------

template <int Q, int D, class T>
__global__ void k_collide_rows(T* __restrict__ f, int64_t n, T tau, LatK<Q, D> L) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    T r[Q];
#pragma unroll
    for (int k = 0; k < Q; ++k) r[k] = f[i * Q + k];
    collide_moment<Q, D, T>(r, tau, L);
#pragma unroll
    for (int k = 0; k < Q; ++k) f[i * Q + k] = r[k];
  }
}

template <int Q, int D, class T>
__global__ void k_equilibrium_rows(const T* __restrict__ rho, const T* __restrict__ u, int64_t n, LatK<Q, D> L,
                                   T* __restrict__ out) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    T uu[D];
#pragma unroll
    for (int a = 0; a < D; ++a) uu[a] = u[i * D + a];
    T feq[Q];
    equilibrium_all<Q, D, T>(rho[i], uu, L, feq);
#pragma unroll
    for (int k = 0; k < Q; ++k) out[i * Q + k] = feq[k];
  }
}

template <class T>
static int collide_rows(T* f, int64_t n, int lattice, T tau, void* stream) {
  if (n < 0 || (n > 0 && !f)) { set_last_error("collide: bad arguments"); return DBM_ERR_INVALID; }
  if (n == 0) return DBM_OK;
  return dispatch_lattice(lattice, [&](auto tag) -> int {
    using LT = decltype(tag);
    auto L = make_latk<LT::Q, LT::D>(*lat_host(lattice), 1.0, 1.0);
    unsigned grid = std::min<unsigned>(div_up(n, 256), (unsigned)sm_count() * 8);
    k_collide_rows<LT::Q, LT::D, T><<<grid, 256, 0, (cudaStream_t)stream>>>(f, n, tau, L);
    DBM_LAUNCH_CHECK();
    return DBM_OK;
  });
}

template <class T>
static int equilibrium_rows(const T* rho, const T* u, int64_t n, int lattice, T* out, void* stream) {
  if (n < 0 || (n > 0 && (!rho || !u || !out))) { set_last_error("equilibrium: bad arguments"); return DBM_ERR_INVALID; }
  if (n == 0) return DBM_OK;
  return dispatch_lattice(lattice, [&](auto tag) -> int {
    using LT = decltype(tag);
    auto L = make_latk<LT::Q, LT::D>(*lat_host(lattice), 1.0, 1.0);
    unsigned grid = std::min<unsigned>(div_up(n, 256), (unsigned)sm_count() * 8);
    k_equilibrium_rows<LT::Q, LT::D, T><<<grid, 256, 0, (cudaStream_t)stream>>>(rho, u, n, L, out);
    DBM_LAUNCH_CHECK();
    return DBM_OK;
  });
}

}  // namespace dbm

using namespace dbm;

extern "C" {

const char* dbm_last_error(void) { return last_error(); }
int dbm_version(void) { return 10000; }
unsigned long long dbm_launch_count(void) { return g_launches; }

int dbm_device_count(int* count) {
  if (!count) return DBM_ERR_INVALID;
  int n = 0;
  cudaError_t e = cudaGetDeviceCount(&n);
  if (e != cudaSuccess) n = 0;
  *count = n;
  return DBM_OK;
}

int dbm_collide_f32(float* f, int64_t n, int lattice, float tau, void* stream) {
  return collide_rows<float>(f, n, lattice, tau, stream);
}
int dbm_collide_f64(double* f, int64_t n, int lattice, double tau, void* stream) {
  return collide_rows<double>(f, n, lattice, tau, stream);
}
int dbm_equilibrium_f32(const float* rho, const float* u, int64_t n, int lattice, float* out, void* stream) {
  return equilibrium_rows<float>(rho, u, n, lattice, out, stream);
}
int dbm_equilibrium_f64(const double* rho, const double* u, int64_t n, int lattice, double* out, void* stream) {
  return equilibrium_rows<double>(rho, u, n, lattice, out, stream);
}

}  // extern "C"
