// Macroscopic fields on the device: bin moments' mass and momentum onto a regular 2D or 3D grid.
//
// Replaces direbm/fields.py:17-41 (bin_fields, numpy histogram2d with mass and momentum weights)
// without leaving the device, and extends it to 3D (histogramdd's rule on three edge arrays; the
// reference bins in 2D only).  A moment's bin follows numpy's rule for the edge array
// (searchsorted(edges, x, "right") - 1, the last edge belonging to the last bin, values outside
// dropped).  Moments are stable-sorted by bin, so each bin's sum runs over its moments in input
// order -- the order the histogram accumulates in -- with no float atomics.
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

// Edge arrays of the D axes, and the D momentum outputs.
struct Edges {
  const double* e[3];
  int n[3];
};
struct MomOut {
  double* p[3];
};

__global__ void k_bin_keys(const double* __restrict__ x, int64_t n, int D, Edges E, uint32_t* __restrict__ keys,
                           uint32_t* __restrict__ vals) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    // bins are indexed [iz][iy][ix] (image convention of the reference); dropped moments sort last
    uint32_t key = 0;
    bool out = false;
    for (int a = D - 1; a >= 0; --a) {
      const int b = bin_of(E.e[a], E.n[a], x[(int64_t)D * i + a]);
      out |= b < 0;
      key = key * (uint32_t)(E.n[a] - 1) + (uint32_t)(b < 0 ? 0 : b);
    }
    keys[i] = out ? 0xffffffffu : key;
    vals[i] = (uint32_t)i;
  }
}

// One thread per bin: binary-search its range in the sorted keys, then sum in sorted order.
template <int Q, int D>
__global__ void k_bin_sums(const uint32_t* __restrict__ keys, const uint32_t* __restrict__ order, int64_t n,
                           const double* __restrict__ f, LatK<Q, D> L, int64_t nbins, double* __restrict__ mass,
                           MomOut mom) {
  for (int64_t b = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; b < nbins; b += (int64_t)gridDim.x * blockDim.x) {
    int64_t lo = 0, hi = n;
    while (lo < hi) {
      const int64_t mid = (lo + hi) >> 1;
      if (keys[mid] < (uint32_t)b) lo = mid + 1; else hi = mid;
    }
    double sm = 0.0, sp[D];
#pragma unroll
    for (int a = 0; a < D; ++a) sp[a] = 0.0;
    for (int64_t j = lo; j < n && keys[j] == (uint32_t)b; ++j) {
      const double* fi = f + (int64_t)order[j] * Q;
      double m = 0.0, p[D];
#pragma unroll
      for (int a = 0; a < D; ++a) p[a] = 0.0;
#pragma unroll
      for (int k = 0; k < Q; ++k) {
        m = __dadd_rn(m, fi[k]);
#pragma unroll
        for (int a = 0; a < D; ++a) p[a] = __dadd_rn(p[a], __dmul_rn(fi[k], L.c[k][a]));
      }
      sm = __dadd_rn(sm, m);
#pragma unroll
      for (int a = 0; a < D; ++a) sp[a] = __dadd_rn(sp[a], p[a]);
    }
    mass[b] = sm;
#pragma unroll
    for (int a = 0; a < D; ++a) mom.p[a][b] = sp[a];
  }
}

// The binning of n moments in D dimensions.
static int bin_fields_impl(int D, const double* x, const double* f, int64_t n, int lattice, const Edges& E,
                           double* mass, MomOut mom, void* tmp, cudaStream_t s) {
  int64_t nbins = 1;
  for (int a = 0; a < D; ++a) nbins *= (int64_t)(E.n[a] - 1);
  if (nbins >= 0xffffffffLL) {
    set_last_error("bin_fields: too many bins (the bin key is 32-bit)");
    return DBM_ERR_INVALID;
  }
  if (n == 0) {
    DBM_CUDA(cudaMemsetAsync(mass, 0, (size_t)nbins * 8, s));
    for (int a = 0; a < D; ++a) DBM_CUDA(cudaMemsetAsync(mom.p[a], 0, (size_t)nbins * 8, s));
    return DBM_OK;
  }
  const size_t al = ((size_t)n * 4 + 255) / 256 * 256;
  uint32_t* keys = (uint32_t*)tmp;
  uint32_t* vals = (uint32_t*)((char*)tmp + al);
  uint32_t* kalt = (uint32_t*)((char*)tmp + 2 * al);
  uint32_t* valt = (uint32_t*)((char*)tmp + 3 * al);
  void* rtmp = (char*)tmp + 4 * al;
  const unsigned grid = std::min<unsigned>(div_up(n, 256), (unsigned)sm_count() * 16);
  k_bin_keys<<<grid, 256, 0, s>>>(x, n, D, E, keys, vals);
  DBM_LAUNCH_CHECK();
  bool alt = false;
  DBM_TRY(radix_sort_pairs<uint32_t>(keys, vals, kalt, valt, n, nullptr, 32, rtmp, s, &alt));
  const uint32_t* ks = alt ? kalt : keys;
  const uint32_t* vs = alt ? valt : vals;
  const LatHost* lh = lat_host(lattice);
  const unsigned bgrid = (unsigned)std::min<int64_t>(div_up(nbins, 128), (int64_t)sm_count() * 64);
  return dispatch_lattice(lattice, [&](auto tag) -> int {
    using LT = decltype(tag);
    auto L = make_latk<LT::Q, LT::D>(*lh, 1.0, 1.0);
    k_bin_sums<LT::Q, LT::D><<<bgrid, 128, 0, s>>>(ks, vs, n, f, L, nbins, mass, mom);
    DBM_LAUNCH_CHECK();
    return DBM_OK;
  });
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
  const Edges E{{ex, ey, nullptr}, {nex, ney, 0}};
  return bin_fields_impl(2, x, f, n, lattice, E, mass, MomOut{{momx, momy, nullptr}}, tmp, (cudaStream_t)stream);
}

extern "C" int dbm_bin_fields3_f64(const double* x, const double* f, int64_t n, int lattice, const double* ex, int nex,
                                   const double* ey, int ney, const double* ez, int nez, double* mass, double* momx,
                                   double* momy, double* momz, void* tmp, void* stream) {
  const LatHost* lh = lat_host(lattice);
  if (!lh || lh->D != 3 || n < 0 || nex < 2 || ney < 2 || nez < 2 || !ex || !ey || !ez || !mass || !momx || !momy ||
      !momz || (n > 0 && (!x || !f || !tmp)) || n >= 0xffffffffLL) {
    set_last_error("bin_fields3: bad arguments");
    return DBM_ERR_INVALID;
  }
  const Edges E{{ex, ey, ez}, {nex, ney, nez}};
  return bin_fields_impl(3, x, f, n, lattice, E, mass, MomOut{{momx, momy, momz}}, tmp, (cudaStream_t)stream);
}
