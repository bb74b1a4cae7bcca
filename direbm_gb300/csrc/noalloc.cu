// Radix sort with library-owned scratch, for callers that must not allocate device memory.
//
// dbm_radix_sort_pairs_u32 needs the caller to supply a scratch buffer, which means someone has
// to call cudaMalloc (or an allocator built on it).  Some callers cannot: a host application that
// hands this library device memory from its own pool and forbids any other allocation, or a
// real-time loop where the implicit device-wide synchronisation of cudaMalloc/cudaFree would
// stall other streams.  dbm_radix_sort_pairs_u32_noalloc serves them: its scratch is a
// file-scope __device__ array that exists on every GPU that loads this library, for as long as
// the process lives, so the call itself never allocates or frees anything.
//
// Limits and rules:
//  * at most DBM_NOALLOC_SORT_MAX_PAIRS pairs per call; larger requests are rejected with
//    DBM_ERR_CAPACITY before any work is queued;
//  * the first call on a device looks up the array's device address (cudaGetSymbolAddress, with
//    that device current) and caches it; make that first call before any stream capture.  The
//    cached address is valid only while the device's primary context lives: after a
//    cudaDeviceReset in the same process it would point at freed memory, so such a process must
//    not call this entry point again;
//  * all calls share the one array: two calls whose work overlaps on the GPU (different streams,
//    no ordering between them) race and corrupt each other's results; order them on one stream
//    or with events;
//  * the array keeps whatever the last call left in it.  Nothing in it has to start at zero:
//    each pass writes every histogram entry and scan partial it later reads, and the alternate
//    key/value buffers are written before they are read.
#include <mutex>

#include "sortscan.cuh"

namespace dbm {

namespace {

constexpr int64_t kMaxPairs = DBM_NOALLOC_SORT_MAX_PAIRS;
constexpr size_t kAltKeyBytes = (size_t)kMaxPairs * sizeof(uint32_t);
constexpr size_t kAltValBytes = (size_t)kMaxPairs * sizeof(uint32_t);
// radix_tmp_bytes(kMaxPairs) = 256 digits x ceil(kMaxPairs / 2048) blocks x 4 B of histograms plus
// a few KB of scan partials; reserve the histograms and 64 KB more.
constexpr size_t kRadixBytes = (size_t)256 * ((kMaxPairs + 2047) / 2048) * 4 + 65536;
constexpr size_t kScratchBytes = kAltKeyBytes + kAltValBytes + kRadixBytes;

// The scratch itself: one copy per device, about 2.2 MB.  Host code must never pass the name
// g_sort_scratch to a kernel -- on the host it is only a stand-in symbol, not a device address.
static __device__ __align__(256) unsigned char g_sort_scratch[kScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_scratch_mu;
void* g_scratch_ptr[kMaxDevices] = {};

// Device address of g_sort_scratch on the current device, looked up once per device.
int scratch_for_current_device(void** out) {
  int dev = 0;
  DBM_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices) {
    set_last_error("noalloc sort: device index %d out of range", dev);
    return DBM_ERR_INVALID;
  }
  std::lock_guard<std::mutex> lock(g_scratch_mu);
  if (!g_scratch_ptr[dev]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_sort_scratch);
    if (e != cudaSuccess || !p) {
      set_last_error("noalloc sort: cudaGetSymbolAddress failed on device %d: %s", dev, cudaGetErrorString(e));
      return DBM_ERR_CUDA;
    }
    g_scratch_ptr[dev] = p;
  }
  *out = g_scratch_ptr[dev];
  return DBM_OK;
}

}  // namespace
}  // namespace dbm

using namespace dbm;

extern "C" int dbm_radix_sort_pairs_u32_noalloc(uint32_t* keys, uint32_t* vals, int64_t n, int key_bits,
                                                void* stream) {
  if (n < 0 || (n > 0 && (!keys || !vals)) || key_bits < 0 || key_bits > 32) {
    set_last_error("radix_sort_pairs_u32_noalloc: bad arguments");
    return DBM_ERR_INVALID;
  }
  if (n > kMaxPairs) {
    set_last_error("radix_sort_pairs_u32_noalloc: %lld pairs exceed the static scratch limit of %lld pairs "
                   "(use dbm_radix_sort_pairs_u32 with caller scratch)", (long long)n, (long long)kMaxPairs);
    return DBM_ERR_CAPACITY;
  }
  if (n == 0) return DBM_OK;
  if (radix_tmp_bytes(n) > kRadixBytes) {  // guards the layout above against future changes
    set_last_error("radix_sort_pairs_u32_noalloc: internal scratch layout too small");
    return DBM_ERR_CAPACITY;
  }
  void* base = nullptr;
  DBM_TRY(scratch_for_current_device(&base));
  cudaStream_t s = (cudaStream_t)stream;
  uint32_t* kalt = (uint32_t*)base;
  uint32_t* valt = (uint32_t*)((char*)base + kAltKeyBytes);
  void* rtmp = (char*)base + kAltKeyBytes + kAltValBytes;
  bool in_alt = false;
  DBM_TRY(radix_sort_pairs<uint32_t>(keys, vals, kalt, valt, n, nullptr, key_bits, rtmp, s, &in_alt));
  if (in_alt) {
    DBM_CUDA(cudaMemcpyAsync(keys, kalt, (size_t)n * 4, cudaMemcpyDeviceToDevice, s));
    DBM_CUDA(cudaMemcpyAsync(vals, valt, (size_t)n * 4, cudaMemcpyDeviceToDevice, s));
  }
  return DBM_OK;
}
