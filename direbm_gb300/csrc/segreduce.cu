// Reduce-by-key with warp-level segmented scans: the deterministic replacement for a scatter with
// float atomics.
//
// The reference scatters each resampled component into its control point's f with wp.atomic_add
// (direbm/warp/propagation.py:186), so the order of the additions -- and the result's last bits --
// changes from run to run.  Here the scatter writes one record (key = control point * Q +
// direction, value) per pair, the records are stable-sorted by key, and segmented_sum_f32 adds the
// values of each run of equal keys:
//   - each warp takes a range of whole runs (its nominal share of the records, both ends moved
//     forward to the next run head, so consecutive warps partition the records by runs);
//   - it walks the range 32 records at a time; a segmented inclusive scan over the lanes
//     (Kogge-Stone, five shuffle steps, the head flags stopping each sum at its run's head) adds
//     the values as (hi, lo) pairs with TwoSum, and the run still open at the chunk's end carries
//     into the next chunk;
//   - the last lane of each run writes out[key].
// Every key is written by one lane and every sum has one fixed order: results are bitwise
// reproducible, whatever the launch configuration.
#include <algorithm>

#include "sortscan.cuh"

namespace dbm {

__device__ __forceinline__ void two_sum_pair(float ah, float al, float bh, float bl, float* sh, float* sl) {
  const float s = __fadd_rn(ah, bh);
  const float bp = __fsub_rn(s, ah);
  const float e = __fadd_rn(__fsub_rn(ah, __fsub_rn(s, bp)), __fsub_rn(bh, bp));
  *sh = s;
  *sl = __fadd_rn(__fadd_rn(al, bl), e);
}

// First run head at or after i (i itself if i == 0 or i >= n); the warp searches 32 at a time.
__device__ __forceinline__ int64_t next_head(const uint32_t* __restrict__ keys, int64_t n, int64_t i) {
  if (i <= 0) return 0;
  const int lane = threadIdx.x & 31;
  for (int64_t b = i; b < n; b += 32) {
    const int64_t j = b + lane;
    const bool head = j < n && keys[j] != keys[j - 1];
    const uint32_t bal = __ballot_sync(0xffffffffu, head || j >= n);
    if (bal) return b + __ffs(bal) - 1 < n ? b + __ffs(bal) - 1 : n;
  }
  return n;
}

__global__ void __launch_bounds__(256) k_seg_sum(const uint32_t* __restrict__ keys, const float* __restrict__ vals,
                                                 int64_t n, int64_t per_warp, float* __restrict__ out) {
  const int lane = threadIdx.x & 31;
  const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int64_t b0 = next_head(keys, n, std::min<int64_t>(warp * per_warp, n));
  const int64_t b1 = next_head(keys, n, std::min<int64_t>((warp + 1) * per_warp, n));
  float ch = 0.f, cl = 0.f;  // the run still open at the previous chunk's end
  for (int64_t c = b0; c < b1; c += 32) {
    const int64_t j = c + lane;
    const bool act = j < b1;
    const uint32_t key = act ? keys[j] : 0xffffffffu;
    float h = act ? vals[j] : 0.f, l = 0.f;
    // head of a run within this chunk (lane 0: a new run unless it continues the carried one)
    const uint32_t prev_key = __shfl_up_sync(0xffffffffu, key, 1);
    bool head = lane == 0 ? (c == b0 || keys[j - 1] != key) : (prev_key != key);
    if (lane == 0 && !head) two_sum_pair(ch, cl, h, l, &h, &l);  // continue the carried run
    // segmented inclusive scan: add the partial of lane - d unless a head lies in between
    bool seg = head;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const float yh = __shfl_up_sync(0xffffffffu, h, d);
      const float yl = __shfl_up_sync(0xffffffffu, l, d);
      const bool ys = __shfl_up_sync(0xffffffffu, seg, d);
      if (lane >= d && !seg) two_sum_pair(yh, yl, h, l, &h, &l);
      if (lane >= d) seg = seg || ys;
    }
    // the last lane of each run inside the chunk writes; a run reaching the chunk's end carries
    const uint32_t next_key = __shfl_down_sync(0xffffffffu, key, 1);
    const bool last_in_chunk = lane == 31 || !(j + 1 < b1);
    if (act && !last_in_chunk && next_key != key) out[key] = __fadd_rn(h, l);
    const int last = (int)std::min<int64_t>(31, b1 - 1 - c);
    const float lh = __shfl_sync(0xffffffffu, h, last), ll = __shfl_sync(0xffffffffu, l, last);
    const uint32_t lk = __shfl_sync(0xffffffffu, key, last);
    const bool run_ends = c + last + 1 >= b1 || keys[c + last + 1] != lk;
    if (run_ends) {
      if (lane == last) out[lk] = __fadd_rn(lh, ll);
      ch = cl = 0.f;
    } else {
      ch = lh;
      cl = ll;
    }
  }
}

int segmented_sum_f32(const uint32_t* keys, const float* vals, int64_t n, float* out, cudaStream_t s) {
  if (n <= 0) return DBM_OK;
  const int64_t warps_max = (int64_t)sm_count() * 64;
  int64_t per_warp = std::max<int64_t>(256, (n + warps_max - 1) / warps_max);
  per_warp = (per_warp + 31) / 32 * 32;
  const int64_t warps = (n + per_warp - 1) / per_warp;
  const unsigned blocks = (unsigned)((warps * 32 + 255) / 256);
  k_seg_sum<<<blocks, 256, 0, s>>>(keys, vals, n, per_warp, out);
  DBM_LAUNCH_CHECK();
  return DBM_OK;
}

}  // namespace dbm

using namespace dbm;

extern "C" int dbm_segmented_sum_f32(const uint32_t* keys, const float* vals, int64_t n, float* out, void* stream) {
  if (n < 0 || (n > 0 && (!keys || !vals || !out))) {
    set_last_error("segmented_sum: bad arguments");
    return DBM_ERR_INVALID;
  }
  return segmented_sum_f32(keys, vals, n, out, (cudaStream_t)stream);
}
