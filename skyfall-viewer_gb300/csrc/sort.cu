// Onesweep LSD radix sort (see sort.cuh).
#include "sort.cuh"

#include <algorithm>
#include <atomic>

namespace sky {
namespace {

constexpr uint32_t kFlagAgg = 1u << 30;
constexpr uint32_t kFlagPrefix = 2u << 30;
constexpr uint32_t kValueMask = (1u << 30) - 1u;
constexpr uint32_t kSpinLimit = 1u << 20;
constexpr int kWarps = kSortThreads / 32;

__device__ __forceinline__ uint32_t ld_relaxed(const uint32_t* p) {
  uint32_t v;
  asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_relaxed(uint32_t* p, uint32_t v) {
  asm volatile("st.relaxed.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ uint32_t lanemask_lt() {
  uint32_t m;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}

// Mask of digit `pass`: 8 bits, fewer in the last pass when key_bits is not
// a multiple of 8 (bits above key_bits do not take part in the order).
__device__ __forceinline__ uint32_t digit_mask(uint32_t key_bits, int pass) {
  const int left = (int)key_bits - 8 * pass;
  return left >= 8 ? 0xFFu : ((1u << left) - 1u);
}

__device__ __forceinline__ void seg_bounds(const SortSegment& s, uint32_t& b, uint32_t& n) {
  if (s.bounds) {
    b = s.bounds[0];
    uint32_t e = s.bounds[1];
    n = e > b ? e - b : 0u;
  } else {
    b = 0;
    n = s.n;
  }
}

// Digit counts of every pass in one read of the keys; also clears the
// look-back words of the tiles this segment will use.
__global__ void __launch_bounds__(kSortThreads)
k_sort_hist(const uint32_t* __restrict__ keys, SortSegment seg, int passes, int digit_lo,
            uint32_t key_bits, uint32_t* __restrict__ hist, uint32_t* __restrict__ lookback,
            uint32_t max_tiles) {
  __shared__ uint32_t s_hist[kMaxPasses][kRadix];
  for (int i = threadIdx.x; i < kMaxPasses * kRadix; i += kSortThreads) (&s_hist[0][0])[i] = 0;
  uint32_t begin, n;
  seg_bounds(seg, begin, n);
  // clear look-back words of this segment's tiles
  uint32_t tiles = (n + kSortTile - 1) / kSortTile;
  uint64_t words = (uint64_t)tiles * kRadix;
  for (int p = 0; p < passes; ++p)
    for (uint64_t w = (uint64_t)blockIdx.x * kSortThreads + threadIdx.x; w < words;
         w += (uint64_t)gridDim.x * kSortThreads)
      lookback[(uint64_t)p * max_tiles * kRadix + w] = 0u;
  __syncthreads();
  const uint32_t lane = threadIdx.x & 31;
  const uint32_t warp_global = (blockIdx.x * kSortThreads + threadIdx.x) >> 5;
  const uint32_t nwarps = (gridDim.x * kSortThreads) >> 5;
  const uint32_t above = lane == 31 ? 0u : (0xFFFFFFFFu << (lane + 1));  // lanes after this one
  // Warp-strided chunks of 128 consecutive keys, 4 per lane (positions
  // 4 lane .. 4 lane + 3).  Keys arrive in emission order, where neighbours
  // mostly share their digits (consecutive tiles of one Gaussian), so each
  // pass counts runs of equal digits: four ballots give every run start of
  // the chunk, and the key that starts a run adds the run's length (distance
  // to the next start, or to the chunk's end).
  for (uint32_t base = warp_global * 128; base < n; base += nwarps * 128) {
    const uint32_t idx = base + 4 * lane;
    const uint32_t N = min(128u, n - base);  // valid keys of the chunk (a prefix)
    const uint32_t nvalid = idx >= n ? 0u : min(4u, n - idx);
    uint32_t k[4];
    if (nvalid == 4u && ((begin + idx) & 3u) == 0u) {
      const uint4 q = *reinterpret_cast<const uint4*>(keys + begin + idx);
      k[0] = q.x; k[1] = q.y; k[2] = q.z; k[3] = q.w;
    } else {
#pragma unroll
      for (int j = 0; j < 4; ++j) k[j] = (uint32_t)j < nvalid ? keys[begin + idx + j] : 0u;
    }
    for (int p = digit_lo; p < passes; ++p) {
      const uint32_t dm = digit_mask(key_bits, p);
      uint32_t d[4];
#pragma unroll
      for (int j = 0; j < 4; ++j) d[j] = (k[j] >> (8 * p)) & dm;
      // a lane with valid keys follows a full lane, so d[3] of lane - 1 is valid
      const uint32_t prev = __shfl_up_sync(0xFFFFFFFFu, d[3], 1);
      bool s[4];
      s[0] = nvalid > 0u && (lane == 0u || d[0] != prev);
      s[1] = nvalid > 1u && d[1] != d[0];
      s[2] = nvalid > 2u && d[2] != d[1];
      s[3] = nvalid > 3u && d[3] != d[2];
      const uint32_t B0 = __ballot_sync(0xFFFFFFFFu, s[0]), B1 = __ballot_sync(0xFFFFFFFFu, s[1]);
      const uint32_t B2 = __ballot_sync(0xFFFFFFFFu, s[2]), B3 = __ballot_sync(0xFFFFFFFFu, s[3]);
      const uint32_t later = (B0 | B1 | B2 | B3) & above;
      // first run start after this lane's keys
      uint32_t next_lane_start = N;
      if (later) {
        const uint32_t l2 = (uint32_t)__ffs(later) - 1u;
        const uint32_t j2 = ((B0 >> l2) & 1u) ? 0u : ((B1 >> l2) & 1u) ? 1u : ((B2 >> l2) & 1u) ? 2u : 3u;
        next_lane_start = 4u * l2 + j2;
      }
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        if (!s[j]) continue;
        uint32_t next = next_lane_start;
#pragma unroll
        for (int jj = 3; jj > j; --jj)
          if (s[jj]) next = 4u * lane + (uint32_t)jj;
        atomicAdd(&s_hist[p][d[j]], next - (4u * lane + (uint32_t)j));
      }
    }
  }
  __syncthreads();
  for (int i = threadIdx.x; i < passes * kRadix; i += kSortThreads) {
    uint32_t v = (&s_hist[0][0])[i];
    if (v) atomicAdd(&hist[i], v);
  }
}

// Exclusive scan of each pass's 256 digit counts (one block per pass), and
// trivial[pass] = 1 when one digit holds every key (the pass would be the
// identity permutation, e.g. the high byte of the integer depth).
__global__ void __launch_bounds__(kRadix)
k_sort_scan(uint32_t* __restrict__ hist, SortSegment seg, uint32_t* __restrict__ trivial,
            int digit_lo) {
  __shared__ uint32_t s_warp[kRadix / 32];
  uint32_t begin, n;
  seg_bounds(seg, begin, n);
  uint32_t* h = hist + blockIdx.x * kRadix;
  uint32_t v = h[threadIdx.x];
  const int one_digit = __syncthreads_or(v == n);
  if (threadIdx.x == 0) trivial[blockIdx.x] = (one_digit || (int)blockIdx.x < digit_lo) ? 1u : 0u;
  uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    uint32_t y = __shfl_up_sync(0xFFFFFFFFu, x, o);
    if (lane >= (uint32_t)o) x += y;
  }
  if (lane == 31) s_warp[warp] = x;
  __syncthreads();
  uint32_t add = 0;
  for (uint32_t w = 0; w < warp; ++w) add += s_warp[w];
  h[threadIdx.x] = x - v + add;
}

__global__ void __launch_bounds__(kSortThreads)
k_onesweep(const uint32_t* keys_src, const uint32_t* vals_src, uint32_t* keys_dst_out,
           uint32_t* vals_dst_out, uint32_t* keys_tmp, uint32_t* vals_tmp, SortSegment seg,
           int pass, int passes, int digit_lo, const uint32_t* __restrict__ trivial, uint32_t key_bits,
           const uint32_t* __restrict__ hist, uint32_t* __restrict__ tile_counter,
           uint32_t* __restrict__ lookback, uint32_t max_tiles, uint32_t* __restrict__ err,
           uint32_t spin_limit, uint32_t withhold_tile0) {
  __shared__ uint32_t s_keys[kSortTile];
  __shared__ uint32_t s_vals[kSortTile];
  __shared__ uint32_t s_warp_hist[kWarps][kRadix];
  __shared__ uint32_t s_block_excl[kRadix];
  __shared__ uint32_t s_global[kRadix];
  __shared__ uint32_t s_scan[kWarps];
  __shared__ uint32_t s_tile;

  // Trivial passes (and those below digit_lo, which are not launched) are
  // skipped; the m remaining passes alternate between the temporary and the
  // output buffers so that the last one writes the output (with m == 0, pass
  // digit_lo runs anyway and copies: its digit is the same for every key).
  int m = 0, j = 0;
  bool skip = false;
  for (int p = 0; p < passes; ++p) {
    const bool t = trivial[p] != 0u;
    if (!t) {
      if (p < pass) ++j;
      ++m;
    }
    if (p == pass) skip = t;
  }
  if (m == 0) {
    if (pass != digit_lo) return;
    skip = false;
    m = 1;
  }
  if (skip) return;
  auto buf_of = [&](int jj, bool key) -> uint32_t* {
    const bool to_out = ((m - 1 - jj) % 2) == 0;
    return key ? (to_out ? keys_dst_out : keys_tmp) : (to_out ? vals_dst_out : vals_tmp);
  };
  const uint32_t* __restrict__ keys_in = j == 0 ? keys_src : buf_of(j - 1, true);
  const uint32_t* __restrict__ vals_in = j == 0 ? vals_src : buf_of(j - 1, false);
  uint32_t* __restrict__ keys_out = buf_of(j, true);
  uint32_t* __restrict__ vals_out = buf_of(j, false);

  uint32_t begin, n;
  seg_bounds(seg, begin, n);
  const uint32_t tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  // Persistent: each block takes tile tickets in order until the segment is
  // done.  A block only waits (look-back) on lower tickets, which were handed
  // to blocks already running, so any grid size makes progress.
  for (;;) {
  __syncthreads();  // the previous tile's shared-memory reads are complete
  if (tid == 0) s_tile = atomicAdd(&tile_counter[pass], 1u);
  for (int i = tid; i < kWarps * kRadix; i += kSortThreads) (&s_warp_hist[0][0])[i] = 0u;
  __syncthreads();
  const uint32_t tile = s_tile;
  const uint32_t base = tile * (uint32_t)kSortTile;
  if (base >= n) return;
  const int shift = 8 * pass;
  const uint32_t dmask = digit_mask(key_bits, pass);

  uint32_t key[kSortItems], val[kSortItems], rank[kSortItems];
  const uint32_t lt = lanemask_lt();
#pragma unroll
  for (int k = 0; k < kSortItems; ++k) {
    uint32_t idx = base + warp * (32 * kSortItems) + k * 32 + lane;
    bool valid = idx < n;
    key[k] = valid ? keys_in[begin + idx] : 0xFFFFFFFFu;
    val[k] = valid ? (vals_in ? vals_in[begin + idx] : begin + idx) : 0u;
  }
#pragma unroll
  for (int k = 0; k < kSortItems; ++k) {
    uint32_t idx = base + warp * (32 * kSortItems) + k * 32 + lane;
    bool valid = idx < n;
    uint32_t d = (key[k] >> shift) & dmask;
    uint32_t active = __ballot_sync(0xFFFFFFFFu, valid);
    uint32_t peers = 0, cnt = 0;
    if (valid) {
      peers = __match_any_sync(active, d);
      cnt = s_warp_hist[warp][d];
    }
    __syncwarp();
    if (valid && (peers & lt) == 0) s_warp_hist[warp][d] = cnt + __popc(peers);
    __syncwarp();
    rank[k] = valid ? cnt + __popc(peers & lt) : 0xFFFFFFFFu;
  }
  __syncthreads();

  // Per digit (thread = digit): per-warp exclusive prefix and tile count.
  const uint32_t d = tid;
  uint32_t run = 0;
#pragma unroll
  for (int w = 0; w < kWarps; ++w) {
    uint32_t c = s_warp_hist[w][d];
    s_warp_hist[w][d] = run;
    run += c;
  }
  uint32_t* lb = lookback + ((uint64_t)pass * max_tiles) * kRadix;
  // (host fault injection only: tile 0 keeps its word back, so tile 1's
  // bounded wait runs out)
  if (tile != 0 || !withhold_tile0)
    st_relaxed(&lb[(uint64_t)tile * kRadix + d], (tile == 0 ? kFlagPrefix : kFlagAgg) | run);

  // Exclusive scan of tile counts over digits.
  uint32_t x = run;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    uint32_t y = __shfl_up_sync(0xFFFFFFFFu, x, o);
    if (lane >= (uint32_t)o) x += y;
  }
  if (lane == 31) s_scan[warp] = x;

  // Decoupled look-back for this digit.
  uint32_t excl = 0;
  if (tile > 0) {
    int64_t j = (int64_t)tile - 1;
    uint32_t spins = 0;
    while (j >= 0) {
      uint32_t v = ld_relaxed(&lb[(uint64_t)j * kRadix + d]);
      uint32_t flag = v & ~kValueMask;
      if (flag == 0u) {
        if (++spins > spin_limit) {
          atomicOr(err, SKY_DEVERR_SORT_TIMEOUT);
          break;
        }
        if (spins > 16) __nanosleep(64);
        continue;
      }
      excl += v & kValueMask;
      if (flag == kFlagPrefix) break;
      --j;
    }
    st_relaxed(&lb[(uint64_t)tile * kRadix + d], kFlagPrefix | (excl + run));
  }
  __syncthreads();
  uint32_t add = 0;
  for (uint32_t w = 0; w < warp; ++w) add += s_scan[w];
  const uint32_t bex = x - run + add;
  s_block_excl[d] = bex;
  s_global[d] = hist[pass * kRadix + d] + excl;
  __syncthreads();

  // Local scatter (stable) into shared memory.
#pragma unroll
  for (int k = 0; k < kSortItems; ++k) {
    if (rank[k] != 0xFFFFFFFFu) {
      uint32_t dk = (key[k] >> shift) & dmask;
      uint32_t lp = s_block_excl[dk] + s_warp_hist[warp][dk] + rank[k];
      s_keys[lp] = key[k];
      s_vals[lp] = val[k];
    }
  }
  __syncthreads();
  const uint32_t cnt = min((uint32_t)kSortTile, n - base);
  for (uint32_t i = tid; i < cnt; i += kSortThreads) {
    uint32_t kk = s_keys[i];
    uint32_t dk = (kk >> shift) & dmask;
    uint32_t gp = s_global[dk] + (i - s_block_excl[dk]);
    if (gp >= n) {  // only after a timed-out look-back; never write out of range
      atomicOr(err, SKY_DEVERR_SORT_TIMEOUT);
      continue;
    }
    keys_out[begin + gp] = kk;
    vals_out[begin + gp] = s_vals[i];
  }
  }  // next tile
}

}  // namespace

int sm_count() {
  static std::atomic<int> cache[64];  // per device; threads racing to fill it store the same value
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) dev = 0;
  int v = cache[dev].load(std::memory_order_relaxed);
  if (!v) {
    cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev);
    if (v <= 0) v = 132;
    cache[dev].store(v, std::memory_order_relaxed);
  }
  return v;
}

size_t sort_scratch_bytes(uint32_t max_n) {
  uint32_t tiles = (max_n + kSortTile - 1) / kSortTile + 1;
  size_t b = 0;
  b += kMaxPasses * kRadix * 4;                    // hist
  b += 256;                                        // tile counters (padded)
  b += (size_t)kMaxPasses * tiles * kRadix * 4;    // look-back
  b += (size_t)(max_n + 64) * 4 * 2;               // ping-pong
  return b + 4096;                                 // 256-byte alignment of 5 pieces
}

SortScratch sort_scratch_carve(void* base, uint32_t max_n) {
  uint32_t tiles = (max_n + kSortTile - 1) / kSortTile + 1;
  char* p = (char*)base;
  auto take = [&](size_t bytes) {
    char* r = p;
    p += (bytes + 255) & ~(size_t)255;
    return r;
  };
  SortScratch s;
  s.hist = (uint32_t*)take(kMaxPasses * kRadix * 4);
  s.tile_counter = (uint32_t*)take(256);
  s.lookback = (uint32_t*)take((size_t)kMaxPasses * tiles * kRadix * 4);
  s.keys_tmp = (uint32_t*)take((size_t)(max_n + 64) * 4);
  s.vals_tmp = (uint32_t*)take((size_t)(max_n + 64) * 4);
  s.max_tiles = tiles;
  return s;
}

cudaError_t sort_pairs_launch(const uint32_t* keys_in, const uint32_t* vals_in,
                              uint32_t* keys_out, uint32_t* vals_out, SortSegment seg,
                              uint32_t max_n, uint32_t key_bits, const SortScratch& sc,
                              uint32_t* err, cudaStream_t stream, int digit_lo,
                              bool fault_point) {
  if (key_bits == 0) key_bits = 1;
  if (key_bits > 32) key_bits = 32;
  const int passes = (int)((key_bits + 7) / 8);
  digit_lo = std::max(0, std::min(digit_lo, passes - 1));
  cudaError_t e = cudaMemsetAsync(sc.hist, 0, kMaxPasses * kRadix * 4, stream);
  if (e != cudaSuccess) return e;
  e = cudaMemsetAsync(sc.tile_counter, 0, 256, stream);
  if (e != cudaSuccess) return e;
  uint32_t tiles = (max_n + kSortTile - 1) / kSortTile;
  if (tiles == 0) tiles = 1;
  uint32_t hist_blocks = tiles < 1024u ? tiles : 1024u;
  k_sort_hist<<<hist_blocks, kSortThreads, 0, stream>>>(keys_in, seg, passes, digit_lo, key_bits,
                                                         sc.hist, sc.lookback, sc.max_tiles);
  uint32_t* trivial = sc.tile_counter + 8;  // cleared with the tile tickets above
  k_sort_scan<<<passes, kRadix, 0, stream>>>(sc.hist, seg, trivial, digit_lo);
  // Host fault injection (SKY_FAULT=lookback:N): in the N-th fault-point sort
  // of the process, tile 0 of every digit pass withholds its look-back word
  // and the waits give up after 64 polls -- the timeout path, without a
  // hang.  Never taken while a graph is being captured (the fault would be
  // replayed).
  const bool inject = fault_point && fault_lookback_next(stream);
  const uint32_t spin_limit = inject ? 64u : kSpinLimit;
  for (int p = digit_lo; p < passes; ++p)
    k_onesweep<<<std::min<uint32_t>(tiles, (uint32_t)sm_count() * 4), kSortThreads, 0,
                 stream>>>(keys_in, vals_in, keys_out, vals_out,
                                                    sc.keys_tmp, sc.vals_tmp, seg, p, passes,
                                                    digit_lo, trivial, key_bits, sc.hist,
                                                    sc.tile_counter, sc.lookback, sc.max_tiles, err,
                                                    spin_limit, inject ? 1u : 0u);
  return cudaGetLastError();
}

}  // namespace sky
