// Device-wide exclusive scan and stable LSD radix sort (library-internal interface).
//
// These replace the Warp library primitives the reference calls (wp.utils.array_scan,
// runlength_encode and radix_sort_pairs at direbm/warp/propagation.py:138-149).  Both use a
// reduce-then-scan structure -- per-tile partials, one small scan of the partials, then a
// per-tile pass -- so no block ever waits on another block.  Item counts may live on the device
// (d_n): launches are sized by a host-side capacity and tiles past the device count do nothing,
// which keeps every launch capturable in a CUDA graph.
#pragma once

#include "common.cuh"

namespace dbm {

constexpr int SCAN_THREADS = 256;
constexpr int SCAN_IPT = 8;
constexpr int SCAN_TILE = SCAN_THREADS * SCAN_IPT;

constexpr int RS_THREADS = 256;             // 8 warps
constexpr int RS_IPT = 8;                   // items per lane
constexpr int RS_TILE = RS_THREADS * RS_IPT;  // 2048 items per block
constexpr int RS_BITS = 8;
constexpr int RS_BUCKETS = 1 << RS_BITS;

// Scratch bytes for scan_exclusive_u32 over up to `cap` items.
size_t scan_tmp_bytes(int64_t cap);
// out[i] = sum_{j<i} in[i] for i < n (n = *d_n if d_n else n_host); *d_total = sum (if non-null).
// `in` and `out` may alias.
int scan_exclusive_u32(const uint32_t* in, uint32_t* out, int64_t cap, const uint32_t* d_n, uint32_t* d_total,
                       void* tmp, cudaStream_t s);

// Stream compaction driven by 0/1 flags: for every i < cap with flag[i] != 0 (in index order),
// writes keys_out[rank] = key_in[i] and vals_out[rank] = i; *d_count = number of flags set.
int compact_flags_u32(const uint32_t* flags, const uint32_t* key_in, uint32_t* keys_out, uint32_t* vals_out,
                      int64_t cap, uint32_t* d_count, void* tmp, cudaStream_t s);
size_t compact_tmp_bytes(int64_t cap);

// Stable ascending sort of (key, value) pairs on the low key_bits bits.  Input in keys/vals,
// ping-pong buffers keys_alt/vals_alt; on return *result_in_alt tells where the sorted data is.
size_t radix_tmp_bytes(int64_t cap);
template <class K>
int radix_sort_pairs(K* keys, uint32_t* vals, K* keys_alt, uint32_t* vals_alt, int64_t cap, const uint32_t* d_n,
                     int key_bits, void* tmp, cudaStream_t s, bool* result_in_alt);

// Reduce-by-key: out[keys[i]] = sum of the values of the run of equal keys keys[i] in a key-sorted
// array (keys < 0xffffffff), with warp-level segmented scans in a fixed order (segreduce.cu).  Keys
// without records leave out untouched.
int segmented_sum_f32(const uint32_t* keys, const float* vals, int64_t n, float* out, cudaStream_t s);

// ---- block-level helpers shared with other kernels -------------------------------------------

// Exclusive scan across a 256-thread block of one value per thread; returns the prefix and the
// block total.  `smem` needs 8 words.  Contains __syncthreads(); all threads must call.
__device__ __forceinline__ uint32_t block_exclusive_scan_256(uint32_t v, uint32_t* smem, uint32_t* total) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) smem[warp] = x;
  __syncthreads();
  if (warp == 0) {
    uint32_t w = lane < 8 ? smem[lane] : 0u;
#pragma unroll
    for (int o = 1; o < 8; o <<= 1) {
      uint32_t y = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w += y;
    }
    if (lane < 8) smem[lane] = w;  // inclusive warp totals
  }
  __syncthreads();
  uint32_t warp_prefix = warp ? smem[warp - 1] : 0u;
  *total = smem[7];
  __syncthreads();
  return warp_prefix + x - v;
}

}  // namespace dbm
