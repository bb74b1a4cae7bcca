// Macroscopic fields on the device: bin moments' mass and momentum onto a regular 2D grid.
//
// Replaces direbm/fields.py:17-41 (bin_fields, numpy histogram2d with mass and momentum weights)
// without leaving the device.  A moment's bin follows numpy's rule for the edge array
// (searchsorted(edges, x, "right") - 1, the last edge belonging to the last bin, values outside
// dropped).  Moments are stable-sorted by bin, so each bin's sum runs over its moments in input
// order -- the order histogram2d accumulates in -- with no float atomics.
#include <algorithm>

#include "lattice.cuh"
#include "sortscan.cuh"

namespace dbm {

__device__ __forceinline__ int bin_of(const double* __restrict__ edges, int ne, double x) {
  // searchsorted(edges, x, side="right") - 1 with the closed last bin of numpy's histogram
  if (!(x >= edges[0]) || !(x <= edges[ne - 1])) return -1;
  if (x == edges[ne - 1]) return ne - 2;
  int lo = 0, hi = ne;  // first index with edges[i] > x
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (edges[mid] > x) hi = mid; else lo = mid + 1;
  }
  return lo - 1;
}

__global__ void k_bin_keys(const double* __restrict__ x, int64_t n, const double* __restrict__ ex, int nex,
                           const double* __restrict__ ey, int ney, uint32_t* __restrict__ keys,
                           uint32_t* __restrict__ vals) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const int bx = bin_of(ex, nex, x[2 * i]);
    const int by = bin_of(ey, ney, x[2 * i + 1]);
    // bins are indexed [iy][ix] (image convention of the reference); dropped moments sort last
    keys[i] = (bx < 0 || by < 0) ? 0xffffffffu : (uint32_t)by * (uint32_t)(nex - 1) + (uint32_t)bx;
    vals[i] = (uint32_t)i;
  }
}

// One thread per bin: binary-search its range in the sorted keys, then sum in sorted order.
template <int Q>
__global__ void k_bin_sums(const uint32_t* __restrict__ keys, const uint32_t* __restrict__ order, int64_t n,
                           const double* __restrict__ f, LatK<Q, 2> L, int nbins, double* __restrict__ mass,
                           double* __restrict__ momx, double* __restrict__ momy) {
  for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < nbins; b += gridDim.x * blockDim.x) {
    int64_t lo = 0, hi = n;
    while (lo < hi) {
      const int64_t mid = (lo + hi) >> 1;
      if (keys[mid] < (uint32_t)b) lo = mid + 1; else hi = mid;
    }
    double sm = 0.0, sx = 0.0, sy = 0.0;
    for (int64_t j = lo; j < n && keys[j] == (uint32_t)b; ++j) {
      const double* fi = f + (int64_t)order[j] * Q;
      double m = 0.0, px = 0.0, py = 0.0;
#pragma unroll
      for (int k = 0; k < Q; ++k) {
        m = __dadd_rn(m, fi[k]);
        px = __dadd_rn(px, __dmul_rn(fi[k], L.c[k][0]));
        py = __dadd_rn(py, __dmul_rn(fi[k], L.c[k][1]));
      }
      sm = __dadd_rn(sm, m);
      sx = __dadd_rn(sx, px);
      sy = __dadd_rn(sy, py);
    }
    mass[b] = sm;
    momx[b] = sx;
    momy[b] = sy;
  }
}

}  // namespace dbm

using namespace dbm;

extern "C" int64_t dbm_bin_fields_tmp_bytes(int64_t n) {
  if (n < 0) return -1;
  const size_t a = ((size_t)std::max<int64_t>(n, 1) * 4 + 255) / 256 * 256;
  return (int64_t)(4 * a + radix_tmp_bytes(std::max<int64_t>(n, 1)));
}

extern "C" int dbm_bin_fields_f64(const double* x, const double* f, int64_t n, int lattice, const double* ex, int nex,
                                  const double* ey, int ney, double* mass, double* momx, double* momy, void* tmp,
                                  void* stream) {
  const LatHost* lh = lat_host(lattice);
  if (!lh || lh->D != 2 || n < 0 || nex < 2 || ney < 2 || !ex || !ey || !mass || !momx || !momy ||
      (n > 0 && (!x || !f || !tmp)) || n >= 0xffffffffLL) {
    set_last_error("bin_fields: bad arguments");
    return DBM_ERR_INVALID;
  }
  cudaStream_t s = (cudaStream_t)stream;
  const int nbins = (nex - 1) * (ney - 1);
  if (n == 0) {
    DBM_CUDA(cudaMemsetAsync(mass, 0, (size_t)nbins * 8, s));
    DBM_CUDA(cudaMemsetAsync(momx, 0, (size_t)nbins * 8, s));
    DBM_CUDA(cudaMemsetAsync(momy, 0, (size_t)nbins * 8, s));
    return DBM_OK;
  }
  const size_t a = ((size_t)n * 4 + 255) / 256 * 256;
  uint32_t* keys = (uint32_t*)tmp;
  uint32_t* vals = (uint32_t*)((char*)tmp + a);
  uint32_t* kalt = (uint32_t*)((char*)tmp + 2 * a);
  uint32_t* valt = (uint32_t*)((char*)tmp + 3 * a);
  void* rtmp = (char*)tmp + 4 * a;
  const unsigned grid = std::min<unsigned>(div_up(n, 256), (unsigned)sm_count() * 16);
  k_bin_keys<<<grid, 256, 0, s>>>(x, n, ex, nex, ey, ney, keys, vals);
  DBM_LAUNCH_CHECK();
  bool alt = false;
  DBM_TRY(radix_sort_pairs<uint32_t>(keys, vals, kalt, valt, n, nullptr, 32, rtmp, s, &alt));
  const uint32_t* ks = alt ? kalt : keys;
  const uint32_t* vs = alt ? valt : vals;
  return dispatch_lattice(lattice, [&](auto tag) -> int {
    using LT = decltype(tag);
    if constexpr (LT::D == 2) {
      auto L = make_latk<LT::Q, 2>(*lh, 1.0, 1.0);
      k_bin_sums<LT::Q><<<div_up(nbins, 128), 128, 0, s>>>(ks, vs, n, f, L, nbins, mass, momx, momy);
      DBM_LAUNCH_CHECK();
    }
    return DBM_OK;
  });
}
