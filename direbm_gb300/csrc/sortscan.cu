// Device-wide exclusive scan, flag compaction and stable LSD radix sort.
//
// Replaces the Warp primitives called at direbm/warp/propagation.py:138-149 (radix_sort_pairs,
// runlength_encode, array_scan).  Stable sort order matters: the cell-thinning centroid is a sum
// in sorted order, so equal keys must keep their input order for the result to be reproducible.
#include "sortscan.cuh"

namespace dbm {

__device__ __forceinline__ int64_t dev_count(const uint32_t* d_n, int64_t cap) {
  if (!d_n) return cap;
  int64_t n = (int64_t)*d_n;
  return n < cap ? n : cap;
}

__device__ __forceinline__ int pad32(int i) { return i + (i >> 5); }

// ---- scan ---------------------------------------------------------------------------------------

__global__ void __launch_bounds__(SCAN_THREADS) k_scan_reduce(const uint32_t* __restrict__ in, int64_t cap,
                                                              const uint32_t* d_n, uint32_t* __restrict__ partial) {
  __shared__ uint32_t sm[8];
  const int64_t n = dev_count(d_n, cap);
  const int64_t base = (int64_t)blockIdx.x * SCAN_TILE;
  uint32_t sum = 0;
#pragma unroll
  for (int i = 0; i < SCAN_IPT; ++i) {
    int64_t idx = base + i * SCAN_THREADS + threadIdx.x;
    if (idx < n) sum += in[idx];
  }
  uint32_t tot;
  block_exclusive_scan_256(sum, sm, &tot);
  if (threadIdx.x == 0) partial[blockIdx.x] = tot;
}

// One block scans the tile partials in place (exclusive) in chunks of SCAN_TILE.
__global__ void __launch_bounds__(SCAN_THREADS) k_scan_partials(uint32_t* __restrict__ partial, int nb,
                                                                uint32_t* d_total) {
  __shared__ uint32_t sm[8];
  uint32_t carry = 0;
  for (int c0 = 0; c0 < nb; c0 += SCAN_TILE) {
    uint32_t v[SCAN_IPT];
    uint32_t tsum = 0;
#pragma unroll
    for (int i = 0; i < SCAN_IPT; ++i) {
      int idx = c0 + threadIdx.x * SCAN_IPT + i;
      v[i] = idx < nb ? partial[idx] : 0u;
      tsum += v[i];
    }
    uint32_t tot;
    uint32_t pre = block_exclusive_scan_256(tsum, sm, &tot) + carry;
#pragma unroll
    for (int i = 0; i < SCAN_IPT; ++i) {
      int idx = c0 + threadIdx.x * SCAN_IPT + i;
      if (idx < nb) partial[idx] = pre;
      pre += v[i];
    }
    carry += tot;
  }
  if (threadIdx.x == 0 && d_total) *d_total = carry;
}

struct EmitPrefix {
  uint32_t* out;
  __device__ __forceinline__ void operator()(int64_t idx, uint32_t prefix) const { out[idx] = prefix; }
};

struct EmitCompact {
  const uint32_t* flags;
  const uint32_t* key_in;
  uint32_t* keys_out;
  uint32_t* vals_out;
  __device__ __forceinline__ void operator()(int64_t idx, uint32_t prefix) const {
    if (flags[idx]) {
      keys_out[prefix] = key_in[idx];
      vals_out[prefix] = (uint32_t)idx;
    }
  }
};

template <class Emit>
__global__ void __launch_bounds__(SCAN_THREADS) k_scan_down(const uint32_t* __restrict__ in, int64_t cap,
                                                            const uint32_t* d_n, const uint32_t* __restrict__ partial,
                                                            Emit emit) {
  __shared__ uint32_t s[SCAN_TILE + SCAN_TILE / 32];
  __shared__ uint32_t sm[8];
  const int64_t n = dev_count(d_n, cap);
  const int64_t base = (int64_t)blockIdx.x * SCAN_TILE;
  if (base >= n) return;
  const int t = threadIdx.x;
#pragma unroll
  for (int i = 0; i < SCAN_IPT; ++i) {
    int li = i * SCAN_THREADS + t;
    int64_t idx = base + li;
    s[pad32(li)] = idx < n ? in[idx] : 0u;
  }
  __syncthreads();
  uint32_t v[SCAN_IPT];
  uint32_t tsum = 0;
#pragma unroll
  for (int i = 0; i < SCAN_IPT; ++i) {
    v[i] = s[pad32(t * SCAN_IPT + i)];
    tsum += v[i];
  }
  uint32_t tot;
  uint32_t pre = block_exclusive_scan_256(tsum, sm, &tot) + partial[blockIdx.x];
#pragma unroll
  for (int i = 0; i < SCAN_IPT; ++i) {
    s[pad32(t * SCAN_IPT + i)] = pre;
    pre += v[i];
  }
  __syncthreads();
#pragma unroll
  for (int i = 0; i < SCAN_IPT; ++i) {
    int li = i * SCAN_THREADS + t;
    int64_t idx = base + li;
    if (idx < n) emit(idx, s[pad32(li)]);
  }
}

size_t scan_tmp_bytes(int64_t cap) { return ((size_t)div_up(cap > 0 ? cap : 1, SCAN_TILE) + 8) * sizeof(uint32_t); }
size_t compact_tmp_bytes(int64_t cap) { return scan_tmp_bytes(cap); }

template <class Emit>
static int scan_impl(const uint32_t* in, int64_t cap, const uint32_t* d_n, uint32_t* d_total, void* tmp,
                     cudaStream_t s, Emit emit) {
  if (cap <= 0) {
    if (d_total) DBM_CUDA(cudaMemsetAsync(d_total, 0, sizeof(uint32_t), s));
    return DBM_OK;
  }
  const int nb = (int)div_up(cap, SCAN_TILE);
  uint32_t* partial = (uint32_t*)tmp;
  k_scan_reduce<<<nb, SCAN_THREADS, 0, s>>>(in, cap, d_n, partial);
  DBM_LAUNCH_CHECK();
  k_scan_partials<<<1, SCAN_THREADS, 0, s>>>(partial, nb, d_total);
  DBM_LAUNCH_CHECK();
  k_scan_down<<<nb, SCAN_THREADS, 0, s>>>(in, cap, d_n, partial, emit);
  DBM_LAUNCH_CHECK();
  return DBM_OK;
}

int scan_exclusive_u32(const uint32_t* in, uint32_t* out, int64_t cap, const uint32_t* d_n, uint32_t* d_total,
                       void* tmp, cudaStream_t s) {
  return scan_impl(in, cap, d_n, d_total, tmp, s, EmitPrefix{out});
}

int compact_flags_u32(const uint32_t* flags, const uint32_t* key_in, uint32_t* keys_out, uint32_t* vals_out,
                      int64_t cap, uint32_t* d_count, void* tmp, cudaStream_t s) {
  return scan_impl(flags, cap, nullptr, d_count, tmp, s, EmitCompact{flags, key_in, keys_out, vals_out});
}

// ---- radix sort ---------------------------------------------------------------------------------

template <class K>
__global__ void __launch_bounds__(RS_THREADS) k_rs_hist(const K* __restrict__ keys, int64_t cap, const uint32_t* d_n,
                                                        int shift, uint32_t* __restrict__ hist, int nb) {
  __shared__ uint32_t h[RS_BUCKETS];
  h[threadIdx.x] = 0;
  __syncthreads();
  const int64_t n = dev_count(d_n, cap);
  const int64_t base = (int64_t)blockIdx.x * RS_TILE;
#pragma unroll
  for (int i = 0; i < RS_IPT; ++i) {
    int64_t idx = base + i * RS_THREADS + threadIdx.x;
    if (idx < n) atomicAdd(&h[(uint32_t)(keys[idx] >> shift) & (RS_BUCKETS - 1)], 1u);
  }
  __syncthreads();
  hist[(int64_t)threadIdx.x * nb + blockIdx.x] = h[threadIdx.x];
}

// Stable scatter of one tile.  Warp w owns items [w*256, w*256+256) of the tile and walks them in
// 8 rounds of 32 consecutive items; __match_any_sync groups equal digits within a round and the
// group leader advances the warp's private digit counter, so ranks follow the input order.
template <class K>
__global__ void __launch_bounds__(RS_THREADS) k_rs_scatter(const K* __restrict__ keys_in,
                                                           const uint32_t* __restrict__ vals_in,
                                                           K* __restrict__ keys_out, uint32_t* __restrict__ vals_out,
                                                           int64_t cap, const uint32_t* d_n, int shift,
                                                           const uint32_t* __restrict__ offs, int nb) {
  __shared__ uint32_t whist[RS_THREADS / 32][RS_BUCKETS];
  __shared__ uint32_t dstart[RS_BUCKETS];
  __shared__ K s_keys[RS_TILE];
  __shared__ uint32_t s_vals[RS_TILE];
  __shared__ uint32_t sm[8];
  const int64_t n = dev_count(d_n, cap);
  const int64_t base = (int64_t)blockIdx.x * RS_TILE;
  if (base >= n) return;
  const int tile_n = (int)((n - base) < RS_TILE ? (n - base) : RS_TILE);
  const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
  for (int i = t; i < (RS_THREADS / 32) * RS_BUCKETS; i += RS_THREADS) (&whist[0][0])[i] = 0u;
  __syncthreads();

  K k[RS_IPT];
  uint32_t v[RS_IPT], r[RS_IPT], dg[RS_IPT];
#pragma unroll
  for (int i = 0; i < RS_IPT; ++i) {
    const int li = warp * (RS_IPT * 32) + i * 32 + lane;
    const bool valid = li < tile_n;
    k[i] = valid ? keys_in[base + li] : (K)0;
    v[i] = valid ? vals_in[base + li] : 0u;
    const uint32_t d = valid ? ((uint32_t)(k[i] >> shift) & (RS_BUCKETS - 1)) : (uint32_t)RS_BUCKETS;
    dg[i] = d;
    const uint32_t peers = __match_any_sync(0xffffffffu, d);
    const int leader = __ffs(peers) - 1;
    uint32_t old = 0;
    if (valid && lane == leader) {
      old = whist[warp][d];
      whist[warp][d] = old + __popc(peers);
    }
    old = __shfl_sync(0xffffffffu, old, leader);
    r[i] = old + __popc(peers & ((1u << lane) - 1u));
    __syncwarp();
  }
  __syncthreads();
  {
    uint32_t run = 0;
#pragma unroll
    for (int w = 0; w < RS_THREADS / 32; ++w) {
      uint32_t c = whist[w][t];
      whist[w][t] = run;
      run += c;
    }
    uint32_t tot;
    dstart[t] = block_exclusive_scan_256(run, sm, &tot);
  }
  __syncthreads();
#pragma unroll
  for (int i = 0; i < RS_IPT; ++i) {
    if (dg[i] < (uint32_t)RS_BUCKETS) {
      const uint32_t pos = dstart[dg[i]] + whist[warp][dg[i]] + r[i];
      s_keys[pos] = k[i];
      s_vals[pos] = v[i];
    }
  }
  __syncthreads();
  for (int p = t; p < tile_n; p += RS_THREADS) {
    const K key = s_keys[p];
    const uint32_t d = (uint32_t)(key >> shift) & (RS_BUCKETS - 1);
    const uint32_t g = offs[(int64_t)d * nb + blockIdx.x] + (uint32_t)p - dstart[d];
    keys_out[g] = key;
    vals_out[g] = s_vals[p];
  }
}

size_t radix_tmp_bytes(int64_t cap) {
  const int64_t nb = div_up(cap > 0 ? cap : 1, RS_TILE);
  return (size_t)(RS_BUCKETS * nb) * sizeof(uint32_t) + scan_tmp_bytes(RS_BUCKETS * nb) + 256;
}

template <class K>
int radix_sort_pairs(K* keys, uint32_t* vals, K* keys_alt, uint32_t* vals_alt, int64_t cap, const uint32_t* d_n,
                     int key_bits, void* tmp, cudaStream_t s, bool* result_in_alt) {
  *result_in_alt = false;
  if (cap <= 0 || key_bits <= 0) return DBM_OK;
  if (key_bits > (int)(8 * sizeof(K))) key_bits = 8 * sizeof(K);
  const int nb = (int)div_up(cap, RS_TILE);
  uint32_t* hist = (uint32_t*)tmp;
  void* scan_tmp = (char*)tmp + (size_t)RS_BUCKETS * nb * sizeof(uint32_t);
  K* ks = keys;
  uint32_t* vs = vals;
  K* kd = keys_alt;
  uint32_t* vd = vals_alt;
  const int passes = (key_bits + RS_BITS - 1) / RS_BITS;
  for (int p = 0; p < passes; ++p) {
    const int shift = p * RS_BITS;
    k_rs_hist<K><<<nb, RS_THREADS, 0, s>>>(ks, cap, d_n, shift, hist, nb);
    DBM_LAUNCH_CHECK();
    DBM_TRY(scan_exclusive_u32(hist, hist, (int64_t)RS_BUCKETS * nb, nullptr, nullptr, scan_tmp, s));
    k_rs_scatter<K><<<nb, RS_THREADS, 0, s>>>(ks, vs, kd, vd, cap, d_n, shift, hist, nb);
    DBM_LAUNCH_CHECK();
    K* tk = ks; ks = kd; kd = tk;
    uint32_t* tv = vs; vs = vd; vd = tv;
  }
  *result_in_alt = (passes & 1) != 0;
  return DBM_OK;
}

template int radix_sort_pairs<uint32_t>(uint32_t*, uint32_t*, uint32_t*, uint32_t*, int64_t, const uint32_t*, int,
                                        void*, cudaStream_t, bool*);
template int radix_sort_pairs<uint64_t>(uint64_t*, uint32_t*, uint64_t*, uint32_t*, int64_t, const uint32_t*, int,
                                        void*, cudaStream_t, bool*);

}  // namespace dbm

using namespace dbm;

template <class K>
static int sort_public(K* keys, uint32_t* vals, int64_t n, int key_bits, void* tmp, void* stream) {
  if (n < 0 || (n > 0 && (!keys || !vals || !tmp)) || key_bits < 0 || key_bits > (int)(8 * sizeof(K))) {
    set_last_error("radix_sort_pairs: bad arguments");
    return DBM_ERR_INVALID;
  }
  if (n == 0) return DBM_OK;
  cudaStream_t s = (cudaStream_t)stream;
  const size_t a = ((size_t)n * sizeof(K) + 255) / 256 * 256;
  const size_t b = ((size_t)n * 4 + 255) / 256 * 256;
  K* kalt = (K*)tmp;
  uint32_t* valt = (uint32_t*)((char*)tmp + a);
  void* rtmp = (char*)tmp + a + b;
  bool in_alt = false;
  DBM_TRY(radix_sort_pairs<K>(keys, vals, kalt, valt, n, nullptr, key_bits, rtmp, s, &in_alt));
  if (in_alt) {
    DBM_CUDA(cudaMemcpyAsync(keys, kalt, (size_t)n * sizeof(K), cudaMemcpyDeviceToDevice, s));
    DBM_CUDA(cudaMemcpyAsync(vals, valt, (size_t)n * 4, cudaMemcpyDeviceToDevice, s));
  }
  return DBM_OK;
}

extern "C" {

int64_t dbm_radix_sort_tmp_bytes(int64_t n, int key_bytes) {
  if (n < 0 || (key_bytes != 4 && key_bytes != 8)) return -1;
  const size_t a = ((size_t)n * key_bytes + 255) / 256 * 256;
  const size_t b = ((size_t)n * 4 + 255) / 256 * 256;
  return (int64_t)(a + b + radix_tmp_bytes(n));
}

int dbm_radix_sort_pairs_u32(uint32_t* keys, uint32_t* vals, int64_t n, int key_bits, void* tmp, void* stream) {
  return sort_public<uint32_t>(keys, vals, n, key_bits, tmp, stream);
}
int dbm_radix_sort_pairs_u64(uint64_t* keys, uint32_t* vals, int64_t n, int key_bits, void* tmp, void* stream) {
  return sort_public<uint64_t>(keys, vals, n, key_bits, tmp, stream);
}

}  // extern "C"
