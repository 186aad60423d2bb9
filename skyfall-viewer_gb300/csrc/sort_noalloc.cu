// sky_sort_pairs_noalloc: the stable radix sort of sky_sort_pairs for
// callers that cannot let the library allocate device memory.
//
// Who needs it: a host that owns every byte of the GPU it runs on -- an
// engine or service that reserves its device memory once at start-up and
// hands out buffers from its own pool, a framework whose caching allocator
// already holds the device, or latency-bound code that must not call
// cudaMalloc (which can synchronise the device and take unbounded time) in
// the middle of its work.  sky_sort_pairs allocates (and caches) its
// scratch with cudaMalloc on first use; this entry point never allocates:
// its scratch is one file-scope device array of fixed size, reserved when
// the module is loaded on a device and kept until the process exits
// (about 9 MiB per GPU that loads the library).
//
// Limits and rules:
//  * at most SKY_SORT_NOALLOC_MAX_KEYS (2^20) keys per call; larger n is
//    rejected with SKY_ERR_ARG (use sky_sort_pairs for those);
//  * the first call on a device looks up the array's device address with
//    cudaGetSymbolAddress (with that device current); make that first call
//    before any stream capture is begun on the device.  The address is kept
//    until the process exits: a cudaDeviceReset after the first call would
//    leave it stale, so resetting the device is not supported once this
//    entry point has been used on it;
//  * every call shares the one array, so calls whose GPU work overlaps in
//    time (different streams, different host threads) race and corrupt
//    each other's results: serialise them;
//  * like sky_sort_pairs, the call returns once the sort has finished: it
//    reads the error word back and waits for `stream`.
#include <cuda_runtime.h>

#include <mutex>

#include "skyfall.h"
#include "sort.cuh"

namespace sky {
int record_error(int code, const char* msg);
}

namespace {

using namespace sky;

constexpr uint32_t kMaxKeys = SKY_SORT_NOALLOC_MAX_KEYS;

// Bytes sort_scratch_carve() takes for kMaxKeys keys (histograms, tile
// tickets, look-back words, ping-pong keys and values, with 256-byte
// alignment slack), then the error word.
constexpr size_t kScratchBytes =
    (size_t)kMaxPasses * kRadix * 4 + 256 +
    (size_t)kMaxPasses * ((kMaxKeys + kSortTile - 1) / kSortTile + 1) * kRadix * 4 +
    (size_t)(kMaxKeys + 64) * 4 * 2 + 4096;
constexpr size_t kErrOffset = (kScratchBytes + 255) & ~(size_t)255;
constexpr size_t kArrayBytes = kErrOffset + 256;

// The scratch of every call on a device.  Host code must not take its
// address directly (that yields a host-side stand-in, not a device
// address); device_scratch() looks the device address up.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kArrayBytes];

std::mutex g_setup_mu;
void* g_scratch_addr[64] = {};  // per device, filled by the first call on it

// Device address of g_noalloc_scratch on `dev` (the current device).
int device_scratch(int dev, void** out) {
  std::lock_guard<std::mutex> lock(g_setup_mu);
  if (!g_scratch_addr[dev]) {
    if (sort_scratch_bytes(kMaxKeys) > kErrOffset)
      return record_error(SKY_ERR_STATE, "sky_sort_pairs_noalloc: scratch array too small");
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || p == nullptr)
      return record_error(SKY_ERR_CUDA, "sky_sort_pairs_noalloc: cudaGetSymbolAddress failed");
    g_scratch_addr[dev] = p;
  }
  *out = g_scratch_addr[dev];
  return SKY_OK;
}

}  // namespace

extern "C" int sky_sort_pairs_noalloc(const uint32_t* keys_in, const uint32_t* vals_in,
                                      uint32_t* keys_out, uint32_t* vals_out, uint32_t n,
                                      uint32_t key_bits, void* stream) {
  if (!keys_in || !keys_out || !vals_out)
    return record_error(SKY_ERR_ARG, "sky_sort_pairs_noalloc: null device pointer");
  if (key_bits == 0 || key_bits > 32)
    return record_error(SKY_ERR_ARG, "sky_sort_pairs_noalloc: key_bits outside 1..32");
  if (n > kMaxKeys)
    return record_error(SKY_ERR_ARG,
                        "sky_sort_pairs_noalloc: n exceeds SKY_SORT_NOALLOC_MAX_KEYS (1048576); "
                        "use sky_sort_pairs");
  if (keys_in == keys_out || (vals_in && vals_in == vals_out))
    return record_error(SKY_ERR_ARG, "sky_sort_pairs_noalloc: input and output arrays must differ");
  if (n == 0) return SKY_OK;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess)
    return record_error(SKY_ERR_CUDA, "sky_sort_pairs_noalloc: no current CUDA device");
  if (dev < 0 || dev >= 64) return record_error(SKY_ERR_ARG, "sky_sort_pairs_noalloc: device index unsupported");
  void* base = nullptr;
  int rc = device_scratch(dev, &base);
  if (rc != SKY_OK) return rc;
  cudaStream_t s = (cudaStream_t)stream;
  // The array keeps the previous call's contents: the error word is cleared
  // here, sort_pairs_launch clears the digit histograms and tile tickets, and
  // its histogram kernel clears the look-back words of the tiles it uses.
  uint32_t* err = (uint32_t*)((char*)base + kErrOffset);
  if (cudaMemsetAsync(err, 0, 4, s) != cudaSuccess)
    return record_error(SKY_ERR_CUDA, "sky_sort_pairs_noalloc: clearing the error word failed");
  SortScratch sc = sort_scratch_carve(base, kMaxKeys);
  SortSegment seg{nullptr, n};
  if (sort_pairs_launch(keys_in, vals_in, keys_out, vals_out, seg, n, key_bits, sc, err, s) !=
      cudaSuccess)
    return record_error(SKY_ERR_CUDA, "sky_sort_pairs_noalloc: kernel launch failed");
  uint32_t h_err = 0;
  if (cudaMemcpyAsync(&h_err, err, 4, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
      cudaStreamSynchronize(s) != cudaSuccess)
    return record_error(SKY_ERR_CUDA, "sky_sort_pairs_noalloc: synchronisation failed");
  if (h_err & SKY_DEVERR_SORT_TIMEOUT)
    return record_error(SKY_ERR_TIMEOUT, "sky_sort_pairs_noalloc: look-back wait gave up");
  return SKY_OK;
}
