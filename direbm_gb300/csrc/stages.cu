// Stage functions on explicit component arrays (FP32, 2D), the reference's propagation API.
//
// These keep the data layout of direbm/warp/propagation.py (positions (N,2), values (N,),
// directions (N,), moments (M,Q) row-major) so the drop-in Python module can hand them numpy
// arrays the way the reference tests do.  Components here are arbitrary points in an unbounded
// plane, so neighbour queries use a sorted-cell index: points sorted by a 64-bit (x-cell,
// y-cell) key, unique cells found by head flags + compaction, and a query binary-searches the
// unique keys of the 5x5 cells around it (a radius-dx disc spans at most 3x3 cells; the extra ring
// covers FP32 rounding of x/dx at cell borders -- the distance test decides).
//
// The radius test is |a - b| with round-to-nearest FP32 steps and no fused multiply-add, so the
// pairs found are the oracle's (oracle/stages.py) bit for bit.  Sums run in a fixed order per
// thread with compensated accumulators: there are no float atomics and results are reproducible.
#include <algorithm>

#include "lattice.cuh"
#include "sortscan.cuh"

namespace dbm {

__device__ __forceinline__ float dist32(float ax, float ay, float bx, float by) {
  const float dx = __fsub_rn(ax, bx), dy = __fsub_rn(ay, by);
  return __fsqrt_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)));
}

__device__ __forceinline__ uint64_t pack_cell(long long ix, long long iy) {
  return ((uint64_t)(uint32_t)(ix + 2147483648LL) << 32) | (uint64_t)(uint32_t)(iy + 2147483648LL);
}

__device__ __forceinline__ long long cell_of(float x, float cs) { return (long long)floorf(__fdiv_rn(x, cs)); }

template <int Q>
__global__ void k_disperse(const float* __restrict__ pos_m, const float* __restrict__ f_m, int64_t m,
                           LatK<Q, 2> L, float dx, float* __restrict__ pos_c, float* __restrict__ val_c,
                           int32_t* __restrict__ dir_c) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < m; i += (int64_t)gridDim.x * blockDim.x) {
    const float x = pos_m[2 * i], y = pos_m[2 * i + 1];
#pragma unroll
    for (int k = 0; k < Q; ++k) {
      const int64_t c = i * Q + k;
      pos_c[2 * c] = __fadd_rn(x, __fmul_rn(L.cf[k][0], dx));
      pos_c[2 * c + 1] = __fadd_rn(y, __fmul_rn(L.cf[k][1], dx));
      val_c[c] = f_m[c];
      dir_c[c] = k;
    }
  }
}

__global__ void k_keys(const float* __restrict__ pos, int64_t n, float cs, uint64_t* __restrict__ keys,
                       uint32_t* __restrict__ vals) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    keys[i] = pack_cell(cell_of(pos[2 * i], cs), cell_of(pos[2 * i + 1], cs));
    vals[i] = (uint32_t)i;
  }
}

__global__ void k_heads(const uint64_t* __restrict__ keys, int64_t n, uint32_t* __restrict__ flags) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    flags[i] = (i == 0 || keys[i] != keys[i - 1]) ? 1u : 0u;
}

// unique keys and run starts from the head positions; ustart[nu] = n
__global__ void k_runs(const uint64_t* __restrict__ keys, const uint32_t* __restrict__ head_idx, const uint32_t* d_nu,
                       int64_t n, uint64_t* __restrict__ ukeys, uint32_t* __restrict__ ustart) {
  const uint32_t nu = *d_nu;
  for (uint32_t r = blockIdx.x * blockDim.x + threadIdx.x; r <= nu; r += gridDim.x * blockDim.x) {
    if (r < nu) {
      ukeys[r] = keys[head_idx[r]];
      ustart[r] = head_idx[r];
    } else {
      ustart[r] = (uint32_t)n;
    }
  }
}

// Sequential FP32 centroid per run, in sorted order (propagation.py:54-68).
__global__ void k_centroid(const float* __restrict__ pos_c, const uint32_t* __restrict__ order,
                           const uint32_t* __restrict__ ustart, const uint32_t* d_nu, float* __restrict__ cp) {
  const uint32_t nu = *d_nu;
  for (uint32_t r = blockIdx.x * blockDim.x + threadIdx.x; r < nu; r += gridDim.x * blockDim.x) {
    const uint32_t s = ustart[r], e = ustart[r + 1];
    float sx = 0.f, sy = 0.f;
    for (uint32_t j = s; j < e; ++j) {
      const uint32_t c = order[j];
      sx = __fadd_rn(sx, pos_c[2 * c]);
      sy = __fadd_rn(sy, pos_c[2 * c + 1]);
    }
    const float n = (float)(e - s);
    cp[2 * r] = __fdiv_rn(sx, n);
    cp[2 * r + 1] = __fdiv_rn(sy, n);
  }
}

// A sorted-cell index over n points (cell size cs).
struct PointIndex {
  uint64_t* keys = nullptr;   // sorted cell keys [n]
  uint32_t* order = nullptr;  // point index in sorted order [n]
  uint64_t* ukeys = nullptr;  // unique keys [n]
  uint32_t* ustart = nullptr; // [n + 1]
  uint32_t* nu = nullptr;     // device count of unique keys
};

struct Arena {  // stream-ordered temporaries, freed together
  static constexpr int kMax = 64;
  cudaStream_t s;
  void* ptrs[kMax];
  int n = 0;
  explicit Arena(cudaStream_t st) : s(st) {}
  template <class T>
  int get(T** p, int64_t count) {
    if (n >= kMax) {
      set_last_error("internal: more than %d temporaries in one stage call", kMax);
      return DBM_ERR_STATE;
    }
    void* q = nullptr;
    cudaError_t e = cudaMallocAsync(&q, (size_t)std::max<int64_t>(count, 1) * sizeof(T), s);
    if (e != cudaSuccess) { set_last_error("cudaMallocAsync: %s", cudaGetErrorString(e)); return DBM_ERR_CUDA; }
    ptrs[n++] = q;
    *p = (T*)q;
    return DBM_OK;
  }
  ~Arena() {
    for (int i = 0; i < n; ++i) cudaFreeAsync(ptrs[i], s);
  }
};

static unsigned grid_for(int64_t n) { return std::min<unsigned>(div_up(std::max<int64_t>(n, 1), 256), (unsigned)sm_count() * 16); }

static int build_index(const float* pos, int64_t n, float cs, Arena& ar, PointIndex* ix) {
  cudaStream_t s = ar.s;
  uint64_t *k_alt;
  uint32_t *v_alt, *flags, *heads, *dummy;
  void* rtmp;
  void* ctmp;
  DBM_TRY(ar.get(&ix->keys, n));
  DBM_TRY(ar.get(&ix->order, n));
  DBM_TRY(ar.get(&k_alt, n));
  DBM_TRY(ar.get(&v_alt, n));
  DBM_TRY(ar.get(&flags, n));
  DBM_TRY(ar.get(&heads, n));
  DBM_TRY(ar.get(&dummy, n));
  DBM_TRY(ar.get(&ix->ukeys, n));
  DBM_TRY(ar.get(&ix->ustart, n + 1));
  DBM_TRY(ar.get(&ix->nu, 1));
  DBM_TRY(ar.get((char**)&rtmp, (int64_t)radix_tmp_bytes(n)));
  DBM_TRY(ar.get((char**)&ctmp, (int64_t)compact_tmp_bytes(n)));
  k_keys<<<grid_for(n), 256, 0, s>>>(pos, n, cs, ix->keys, ix->order);
  DBM_LAUNCH_CHECK();
  bool alt = false;
  DBM_TRY(radix_sort_pairs<uint64_t>(ix->keys, ix->order, k_alt, v_alt, n, nullptr, 64, rtmp, s, &alt));
  if (alt) {
    ix->keys = k_alt;
    ix->order = v_alt;
  }
  k_heads<<<grid_for(n), 256, 0, s>>>(ix->keys, n, flags);
  DBM_LAUNCH_CHECK();
  DBM_TRY(compact_flags_u32(flags, flags, dummy, heads, n, ix->nu, ctmp, s));
  k_runs<<<grid_for(n + 1), 256, 0, s>>>(ix->keys, heads, ix->nu, n, ix->ukeys, ix->ustart);
  DBM_LAUNCH_CHECK();
  return DBM_OK;
}

__device__ __forceinline__ bool find_cell(const PointIndex& ix, uint64_t key, uint32_t* b, uint32_t* e) {
  uint32_t lo = 0, hi = *ix.nu;
  while (lo < hi) {
    uint32_t mid = (lo + hi) >> 1;
    if (ix.ukeys[mid] < key) lo = mid + 1; else hi = mid;
  }
  if (lo < *ix.nu && ix.ukeys[lo] == key) {
    *b = ix.ustart[lo];
    *e = ix.ustart[lo + 1];
    return true;
  }
  return false;
}

__global__ void k_refine(const float* __restrict__ cp, int64_t p, const float* __restrict__ pos_c,
                         const float* __restrict__ val_c, const int32_t* __restrict__ dir_c, PointIndex ix, float dx,
                         int kappa_hard, float* __restrict__ out) {
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < p; r += (int64_t)gridDim.x * blockDim.x) {
    const float px = cp[2 * r], py = cp[2 * r + 1];
    const long long cx = cell_of(px, dx), cy = cell_of(py, dx);
    uint32_t mask = 0;
    CSum sw, sx, sy;
    for (int ox = -2; ox <= 2; ++ox)
      for (int oy = -2; oy <= 2; ++oy) {
        uint32_t b, e;
        if (!find_cell(ix, pack_cell(cx + ox, cy + oy), &b, &e)) continue;
        for (uint32_t j = b; j < e; ++j) {
          const uint32_t c = ix.order[j];
          const float qx = pos_c[2 * c], qy = pos_c[2 * c + 1];
          if (dist32(qx, qy, px, py) <= dx) {
            mask |= 1u << dir_c[c];
            const float w = expf(val_c[c]);
            sw.add(w);
            sx.add_prod(w, qx);
            sy.add_prod(w, qy);
          }
        }
      }
    const int kappa = __popc(mask);
    if (kappa <= kappa_hard) {
      out[2 * r] = px;
      out[2 * r + 1] = py;
    } else {
      const float s = sw.value();
      out[2 * r] = sx.value() / s;
      out[2 * r + 1] = sy.value() / s;
    }
  }
}

// Pass 1 of the resampling gather: sw per component over the control points within dx.
__global__ void k_comp_sw(const float* __restrict__ pos_c, int64_t nc, const float* __restrict__ cp, PointIndex cpi,
                          float dx, float* __restrict__ sw_out) {
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < nc; c += (int64_t)gridDim.x * blockDim.x) {
    const float qx = pos_c[2 * c], qy = pos_c[2 * c + 1];
    const long long cx = cell_of(qx, dx), cy = cell_of(qy, dx);
    CSum sw;
    for (int ox = -2; ox <= 2; ++ox)
      for (int oy = -2; oy <= 2; ++oy) {
        uint32_t b, e;
        if (!find_cell(cpi, pack_cell(cx + ox, cy + oy), &b, &e)) continue;
        for (uint32_t j = b; j < e; ++j) {
          const uint32_t r = cpi.order[j];
          const float d = dist32(cp[2 * r], cp[2 * r + 1], qx, qy);
          if (d <= dx) sw.add(__fsub_rn(dx, d));
        }
      }
    sw_out[c] = sw.value();
  }
}

// Pass 2 as the reference's scatter (propagation.py:156-186), without its float atomics: every
// component (m, k) with sw > 0 writes one record per control point r within dx, key r * Q + k and
// value (dx - d)/sw * f, at offsets from a scan of its count (records in component order, control
// points in index-walk order); the records are stable-sorted by key and each key's run is summed
// by the warp-level segmented reduction (segreduce.cu).
__global__ void k_scatter_count(const float* __restrict__ pos_c, int64_t nc, const float* __restrict__ cp,
                                PointIndex cpi, const float* __restrict__ sw, float dx, uint32_t* __restrict__ cnt) {
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < nc; c += (int64_t)gridDim.x * blockDim.x) {
    uint32_t n = 0;
    if (sw[c] > 0.f) {
      const float qx = pos_c[2 * c], qy = pos_c[2 * c + 1];
      const long long cx = cell_of(qx, dx), cy = cell_of(qy, dx);
      for (int ox = -2; ox <= 2; ++ox)
        for (int oy = -2; oy <= 2; ++oy) {
          uint32_t b, e;
          if (!find_cell(cpi, pack_cell(cx + ox, cy + oy), &b, &e)) continue;
          for (uint32_t j = b; j < e; ++j) {
            const uint32_t r = cpi.order[j];
            if (dist32(cp[2 * r], cp[2 * r + 1], qx, qy) <= dx) ++n;
          }
        }
    }
    cnt[c] = n;
  }
}

template <int Q>
__global__ void k_scatter_write(const float* __restrict__ pos_c, int64_t nc, const float* __restrict__ val_c,
                                const int32_t* __restrict__ dir_c, const float* __restrict__ cp, PointIndex cpi,
                                const float* __restrict__ sw, float dx, const uint32_t* __restrict__ pos_of,
                                uint32_t* __restrict__ keys, float* __restrict__ vals) {
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < nc; c += (int64_t)gridDim.x * blockDim.x) {
    const float s = sw[c];
    if (!(s > 0.f)) continue;
    const float qx = pos_c[2 * c], qy = pos_c[2 * c + 1];
    const long long cx = cell_of(qx, dx), cy = cell_of(qy, dx);
    const uint32_t k = (uint32_t)dir_c[c];
    const float v = val_c[c];
    uint32_t w = pos_of[c];
    for (int ox = -2; ox <= 2; ++ox)
      for (int oy = -2; oy <= 2; ++oy) {
        uint32_t b, e;
        if (!find_cell(cpi, pack_cell(cx + ox, cy + oy), &b, &e)) continue;
        for (uint32_t j = b; j < e; ++j) {
          const uint32_t r = cpi.order[j];
          const float d = dist32(cp[2 * r], cp[2 * r + 1], qx, qy);
          if (d <= dx) {
            keys[w] = r * (uint32_t)Q + k;
            vals[w] = __fmul_rn(__fdiv_rn(__fsub_rn(dx, d), s), v);
            ++w;
          }
        }
      }
  }
}

// The emptiness mask of each control point from its resampled f (before the gap fill).
template <int Q>
__global__ void k_cp_emask(const float* __restrict__ cpf, int64_t p, float eps, uint32_t* __restrict__ emask) {
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < p; r += (int64_t)gridDim.x * blockDim.x) {
    uint32_t em = 0;
#pragma unroll
    for (int q = 0; q < Q; ++q)
      if (cpf[r * Q + q] < eps) em |= 1u << q;
    emask[r] = em;
  }
}

template <int Q>
__global__ void k_cp_fill(const float* __restrict__ cp, int64_t p, PointIndex cpi, const uint32_t* __restrict__ emask,
                          const float* __restrict__ f_rest, float dx, float* __restrict__ cpf,
                          float* __restrict__ out_pos, float* __restrict__ out_f) {
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < p; r += (int64_t)gridDim.x * blockDim.x) {
    const float px = cp[2 * r], py = cp[2 * r + 1];
    const uint32_t em = emask[r];
    CSum sw[Q];
    if (em) {
      const long long cx = cell_of(px, dx), cy = cell_of(py, dx);
      for (int ox = -2; ox <= 2; ++ox)
        for (int oy = -2; oy <= 2; ++oy) {
          uint32_t b, e;
          if (!find_cell(cpi, pack_cell(cx + ox, cy + oy), &b, &e)) continue;
          for (uint32_t j = b; j < e; ++j) {
            const uint32_t o = cpi.order[j];
            const uint32_t both = emask[o] & em;
            if (!both) continue;
            const float d = dist32(cp[2 * o], cp[2 * o + 1], px, py);
            if (d <= dx) {
              const float w = __fsub_rn(dx, d);
#pragma unroll
              for (int q = 0; q < Q; ++q)
                if ((both >> q) & 1u) sw[q].add(w);
            }
          }
        }
    }
#pragma unroll
    for (int q = 0; q < Q; ++q) {
      float v = cpf[r * Q + q];
      const float s = sw[q].value();
      if (((em >> q) & 1u) && s > 0.f) v = (dx / s) * f_rest[q];
      out_f[r * Q + q] = v;
    }
    out_pos[2 * r] = px;
    out_pos[2 * r + 1] = py;
  }
}

}  // namespace dbm

using namespace dbm;

static int check_2d(int lattice) {
  const LatHost* h = lat_host(lattice);
  if (!h || h->D != 2) {
    set_last_error("stage functions take a 2D lattice (got id %d)", lattice);
    return DBM_ERR_INVALID;
  }
  return DBM_OK;
}

extern "C" {

int dbm_disperse_f32(const float* pos_m, const float* f_m, int64_t m, int lattice, float dx, float* pos_c,
                     float* val_c, int32_t* dir_c, void* stream) {
  DBM_TRY(check_2d(lattice));
  if (m < 0 || (m > 0 && (!pos_m || !f_m || !pos_c || !val_c || !dir_c))) {
    set_last_error("disperse: bad arguments");
    return DBM_ERR_INVALID;
  }
  if (m == 0) return DBM_OK;
  return dispatch_lattice(lattice, [&](auto tag) -> int {
    using LT = decltype(tag);
    if constexpr (LT::D == 2) {
      auto L = make_latk<LT::Q, 2>(*lat_host(lattice), 1.0, 1.0);
      k_disperse<LT::Q><<<grid_for(m), 256, 0, (cudaStream_t)stream>>>(pos_m, f_m, m, L, dx, pos_c, val_c, dir_c);
      DBM_LAUNCH_CHECK();
    }
    return DBM_OK;
  });
}

int dbm_create_control_points_f32(const float* pos_c, int64_t nc, float cs, float* cp_pos, int64_t* p_out,
                                  void* stream) {
  if (nc < 0 || !p_out || (nc > 0 && (!pos_c || !cp_pos)) || !(cs > 0.f) || nc >= 0x7fffffffLL) {
    set_last_error("create_control_points: bad arguments");
    return DBM_ERR_INVALID;
  }
  *p_out = 0;
  if (nc == 0) return DBM_OK;
  cudaStream_t s = (cudaStream_t)stream;
  uint32_t nu = 0;
  {
    Arena ar(s);
    PointIndex ix;
    DBM_TRY(build_index(pos_c, nc, cs, ar, &ix));
    k_centroid<<<grid_for(nc), 256, 0, s>>>(pos_c, ix.order, ix.ustart, ix.nu, cp_pos);
    DBM_LAUNCH_CHECK();
    DBM_CUDA(cudaMemcpyAsync(&nu, ix.nu, 4, cudaMemcpyDeviceToHost, s));
  }
  DBM_CUDA(cudaStreamSynchronize(s));
  *p_out = nu;
  return DBM_OK;
}

int dbm_refine_control_points_f32(const float* cp, int64_t p, const float* pos_c, const float* val_c,
                                  const int32_t* dir_c, int64_t nc, float dx, int kappa_hard, float* new_pos,
                                  void* stream) {
  if (p < 0 || nc < 0 || !(dx > 0.f) || (p > 0 && (!cp || !new_pos)) || (nc > 0 && (!pos_c || !val_c || !dir_c))) {
    set_last_error("refine_control_points: bad arguments");
    return DBM_ERR_INVALID;
  }
  if (p == 0) return DBM_OK;
  cudaStream_t s = (cudaStream_t)stream;
  Arena ar(s);
  PointIndex ix;
  if (nc > 0) {
    DBM_TRY(build_index(pos_c, nc, dx, ar, &ix));
  } else {
    DBM_TRY(ar.get(&ix.nu, 1));
    DBM_CUDA(cudaMemsetAsync(ix.nu, 0, 4, s));
  }
  k_refine<<<grid_for(p), 256, 0, s>>>(cp, p, pos_c, val_c, dir_c, ix, dx, kappa_hard, new_pos);
  DBM_LAUNCH_CHECK();
  return DBM_OK;
}

int dbm_resample_f32(const float* pos_c, const float* val_c, const int32_t* dir_c, int64_t nc, const float* cp,
                     int64_t p, float dx, const float* f_rest, int lattice, float eps, float* out_pos, float* out_f,
                     void* stream) {
  DBM_TRY(check_2d(lattice));
  if (p < 0 || nc < 0 || !(dx > 0.f) || (p > 0 && (!cp || !out_pos || !out_f || !f_rest)) ||
      (nc > 0 && (!pos_c || !val_c || !dir_c))) {
    set_last_error("resample: bad arguments");
    return DBM_ERR_INVALID;
  }
  if (p == 0) return DBM_OK;
  cudaStream_t s = (cudaStream_t)stream;
  return dispatch_lattice(lattice, [&](auto tag) -> int {
    using LT = decltype(tag);
    if constexpr (LT::D == 2) {
      constexpr int Q = LT::Q;
      Arena ar(s);
      PointIndex cpi, ci;
      DBM_TRY(build_index(cp, p, dx, ar, &cpi));
      float *sw, *cpf;
      uint32_t* em;
      DBM_TRY(ar.get(&sw, nc));
      DBM_TRY(ar.get(&cpf, p * Q));
      DBM_TRY(ar.get(&em, p));
      if (nc > 0) {
        DBM_TRY(build_index(pos_c, nc, dx, ar, &ci));
        k_comp_sw<<<grid_for(nc), 256, 0, s>>>(pos_c, nc, cp, cpi, dx, sw);
        DBM_LAUNCH_CHECK();
      } else {
        DBM_TRY(ar.get(&ci.nu, 1));
        DBM_CUDA(cudaMemsetAsync(ci.nu, 0, 4, s));
      }
      DBM_CUDA(cudaMemsetAsync(cpf, 0, (size_t)p * Q * sizeof(float), s));
      if (nc > 0) {
        // the scatter: pair records, stable sort by (control point, direction), segmented sums
        uint32_t *cnt, *pos_of, *d_total;
        DBM_TRY(ar.get(&cnt, nc));
        DBM_TRY(ar.get(&pos_of, nc));
        DBM_TRY(ar.get(&d_total, 1));
        char* stmp;
        DBM_TRY(ar.get(&stmp, (int64_t)scan_tmp_bytes(nc)));
        k_scatter_count<<<grid_for(nc), 256, 0, s>>>(pos_c, nc, cp, cpi, sw, dx, cnt);
        DBM_LAUNCH_CHECK();
        DBM_TRY(scan_exclusive_u32(cnt, pos_of, nc, nullptr, d_total, stmp, s));
        uint32_t total = 0;  // the record count sizes the sort
        DBM_CUDA(cudaMemcpyAsync(&total, d_total, 4, cudaMemcpyDeviceToHost, s));
        DBM_CUDA(cudaStreamSynchronize(s));
        if (total > 0) {
          uint32_t *rk, *rv, *rk2, *rv2;
          DBM_TRY(ar.get(&rk, total));
          DBM_TRY(ar.get(&rv, total));
          DBM_TRY(ar.get(&rk2, total));
          DBM_TRY(ar.get(&rv2, total));
          char* rtmp;
          DBM_TRY(ar.get(&rtmp, (int64_t)radix_tmp_bytes(total)));
          k_scatter_write<Q><<<grid_for(nc), 256, 0, s>>>(pos_c, nc, val_c, dir_c, cp, cpi, sw, dx, pos_of, rk,
                                                         reinterpret_cast<float*>(rv));
          DBM_LAUNCH_CHECK();
          int bits = 1;
          while (bits < 32 && ((uint64_t)1 << bits) < (uint64_t)p * Q) ++bits;
          bool alt = false;  // the values travel as their bit patterns
          DBM_TRY(radix_sort_pairs<uint32_t>(rk, rv, rk2, rv2, total, nullptr, bits, rtmp, s, &alt));
          DBM_TRY(segmented_sum_f32(alt ? rk2 : rk, reinterpret_cast<const float*>(alt ? rv2 : rv), total, cpf, s));
        }
      }
      k_cp_emask<Q><<<grid_for(p), 256, 0, s>>>(cpf, p, eps, em);
      DBM_LAUNCH_CHECK();
      k_cp_fill<Q><<<grid_for(p), 256, 0, s>>>(cp, p, cpi, em, f_rest, dx, cpf, out_pos, out_f);
      DBM_LAUNCH_CHECK();
    }
    return DBM_OK;
  });
}

}  // extern "C"
