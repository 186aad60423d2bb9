// Onesweep LSD radix sort of (u32 key, u32 value) pairs.
//
// Replaces the reference's Fuchsia-derived radix sort (src/sort/radix_sort.wgsl:
// 55-519, host src/sort/sort.ts:260-370): same result -- a stable ascending
// sort by key with 8-bit digits -- but each digit pass is a single kernel
// (Adinets & Merrill, "Onesweep", 2022): one upfront histogram kernel counts
// the digits of every pass in one read of the keys, then each pass ranks a
// tile of keys in shared memory, obtains its global digit offsets through a
// decoupled look-back over the preceding tiles, and scatters.  Look-back waits
// are bounded: after kSpinLimit polls the tile records SKY_DEVERR_SORT_TIMEOUT
// in the status word and stops (the host reports SKY_ERR_TIMEOUT) -- the
// reference's look-back (radix_sort.wgsl:372-393) has no bound.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace sky {

constexpr int kSortThreads = 256;
constexpr int kSortItems = 16;
constexpr int kSortTile = kSortThreads * kSortItems;  // 4096 keys per tile
constexpr int kRadix = 256;
constexpr int kMaxPasses = 4;

// Device error bits (status word 0).
constexpr uint32_t SKY_DEVERR_CAPACITY = 1u;
constexpr uint32_t SKY_DEVERR_SORT_TIMEOUT = 2u;
// The intersection lists disagree with themselves: key emission wrote a
// different number of tiles than the preprocess counted for an item, or the
// tile ranges met sorted keys out of order.  Later kernels of the step skip.
constexpr uint32_t SKY_DEVERR_LISTS = 4u;

struct SortScratch {
  uint32_t* hist;          // kMaxPasses * 256 digit counts, then exclusive offsets
  uint32_t* tile_counter;  // kMaxPasses tile tickets
  uint32_t* lookback;      // kMaxPasses * max_tiles * 256 status words
  uint32_t* keys_tmp;      // ping-pong
  uint32_t* vals_tmp;
  uint32_t max_tiles;
};

// Segment of one sort: [begin, end) read from device memory (so a captured
// graph sorts however many intersections a step produced).
struct SortSegment {
  const uint32_t* bounds;  // bounds[0] = begin, bounds[1] = end; NULL -> [0, n)
  uint32_t n;              // used when bounds == NULL
};

// Launch the full sort on `stream`.  keys_in/vals_in: input (vals_in may be
// NULL, meaning value = the key's position in keys_in); results in
// keys_out/vals_out at the same positions.  key_bits: 1..32.  err: device
// word receiving error bits.  max_n: bound on the segment size (grid size).
// digit_lo: 8-bit digits below it are not sorted on -- for keys whose input
// order is already ascending in those bits among equal higher bits, the
// result is the full sort.
// fault_point: the sort counts for SKY_FAULT=lookback:N (host fault
// injection, used by tests); only callers whose later kernels check the
// error word before indexing with the sort's output pass true.
cudaError_t sort_pairs_launch(const uint32_t* keys_in, const uint32_t* vals_in,
                              uint32_t* keys_out, uint32_t* vals_out, SortSegment seg,
                              uint32_t max_n, uint32_t key_bits, const SortScratch& sc,
                              uint32_t* err, cudaStream_t stream, int digit_lo = 0,
                              bool fault_point = false);

// Host fault injection (SKY_FAULT=lookback:N, api.cu): true for the N-th
// fault-point sort launched outside graph capture in the process.  Without
// that setting it returns false and makes no CUDA call.
bool fault_lookback_next(cudaStream_t stream);

// Multiprocessors of the current device (cached per device).
int sm_count();

// Bytes of scratch needed for segments up to max_n keys (excluding nothing).
size_t sort_scratch_bytes(uint32_t max_n);
// Carves a SortScratch out of one device allocation of sort_scratch_bytes(max_n).
SortScratch sort_scratch_carve(void* base, uint32_t max_n);

}  // namespace sky
