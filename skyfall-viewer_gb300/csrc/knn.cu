// k-nearest-neighbour scale initialisation: knn_init (knn-init.wgsl:40-90,
// dispatched by initializeKnn, gaussian-renderer.ts:2131-2171) without its
// O(N^2) scan.  Points (positions read through f16, as the reference's
// packed buffer holds them) are binned into a uniform grid and sorted by
// cell; each point then visits the cells in shells of growing Chebyshev
// radius r around its own and stops once its third-smallest distance is
// below the distance to any unvisited cell, (r - 0.001) h: cell assignment
// in f32 places a point at most 2.4e-4 cells from its true cell, so no
// unvisited point can be closer.  The three smallest distances are the ones
// the brute-force scan finds (the insertion keeps values; ties do not
// reorder them), so the result is bit-identical to it.
#include <cstring>

#include "knn.cuh"
#include "sky_math.cuh"

namespace sky {
namespace {

SKY_DEV uint32_t enc(float f) {  // order-preserving float -> u32
  const uint32_t b = __float_as_uint(f);
  return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}

SKY_DEV float pos16(const float* P, uint32_t stride, int k, uint32_t i) {
  return round_f16(P[(size_t)k * stride + i]);
}

__global__ void __launch_bounds__(256)
k_knn_bounds(const float* __restrict__ P, uint32_t stride, uint32_t n, uint32_t* __restrict__ out) {
  uint32_t mn[3] = {0xFFFFFFFFu, 0xFFFFFFFFu, 0xFFFFFFFFu}, mx[3] = {0u, 0u, 0u};
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    for (int k = 0; k < 3; ++k) {
      const float v = pos16(P, stride, k, i);
      if (v != v) continue;
      const uint32_t e = enc(v);
      mn[k] = min(mn[k], e);
      mx[k] = max(mx[k], e);
    }
  for (int k = 0; k < 3; ++k) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      mn[k] = min(mn[k], __shfl_xor_sync(0xFFFFFFFFu, mn[k], o));
      mx[k] = max(mx[k], __shfl_xor_sync(0xFFFFFFFFu, mx[k], o));
    }
    if ((threadIdx.x & 31) == 0) {
      atomicMin(&out[k], mn[k]);
      atomicMax(&out[3 + k], mx[k]);
    }
  }
}

SKY_DEV uint32_t cell_of(float v, float lo, float h, uint32_t dim) {
  const float q = (v - lo) / h;
  if (!(q > 0.0f)) return 0u;
  const float c = floorf(q);
  return c >= (float)(dim - 1) ? dim - 1 : (uint32_t)c;
}

__global__ void __launch_bounds__(256)
k_knn_keys(const float* __restrict__ P, uint32_t stride, uint32_t n, KnnGrid g,
           uint32_t* __restrict__ keys) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint32_t cx = cell_of(pos16(P, stride, 0, i), g.lo[0], g.h, g.dims[0]);
  const uint32_t cy = cell_of(pos16(P, stride, 1, i), g.lo[1], g.h, g.dims[1]);
  const uint32_t cz = cell_of(pos16(P, stride, 2, i), g.lo[2], g.h, g.dims[2]);
  keys[i] = (cz * g.dims[1] + cy) * g.dims[0] + cx;
}

__global__ void k_knn_cell_ranges(const uint32_t* __restrict__ keys, uint32_t n, uint32_t cells,
                                  uint32_t* __restrict__ start) {
  const uint32_t c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c > cells) return;
  uint32_t lo = 0, hi = n;
  while (lo < hi) {
    const uint32_t mid = lo + ((hi - lo) >> 1);
    if (keys[mid] < c) lo = mid + 1;
    else hi = mid;
  }
  start[c] = lo;
}

SKY_DEV void insert3(float d[3], float v) {  // insert_sorted (knn-init.wgsl:27-38)
  if (v < d[0]) {
    d[2] = d[1];
    d[1] = d[0];
    d[0] = v;
  } else if (v < d[1]) {
    d[2] = d[1];
    d[1] = v;
  } else if (v < d[2]) {
    d[2] = v;
  }
}

__global__ void __launch_bounds__(256)
k_knn_query(const float* __restrict__ P, uint32_t stride, uint32_t n, KnnGrid g,
            const uint32_t* __restrict__ order, const uint32_t* __restrict__ start, float extent,
            float* __restrict__ density, float* __restrict__ log_sigma) {
  const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  const uint32_t self = order[k];
  const float px = pos16(P, stride, 0, self), py = pos16(P, stride, 1, self),
              pz = pos16(P, stride, 2, self);
  const int cx = (int)cell_of(px, g.lo[0], g.h, g.dims[0]);
  const int cy = (int)cell_of(py, g.lo[1], g.h, g.dims[1]);
  const int cz = (int)cell_of(pz, g.lo[2], g.h, g.dims[2]);
  const int DX = (int)g.dims[0], DY = (int)g.dims[1], DZ = (int)g.dims[2];
  float d[3] = {1e10f, 1e10f, 1e10f};
  auto visit = [&](int x, int y, int z) {
    const uint32_t c = ((uint32_t)z * g.dims[1] + (uint32_t)y) * g.dims[0] + (uint32_t)x;
    const uint32_t e = start[c + 1];
    for (uint32_t j = start[c]; j < e; ++j) {
      const uint32_t o = order[j];
      if (o == self) continue;
      const float dx = px - pos16(P, stride, 0, o);
      const float dy = py - pos16(P, stride, 1, o);
      const float dz = pz - pos16(P, stride, 2, o);
      float s = dx * dx + dy * dy;
      s = s + dz * dz;
      insert3(d, sqrtf(s));
    }
  };
  const int rmax = max(DX, max(DY, DZ));
  for (int r = 0; r <= rmax; ++r) {
    for (int z = max(cz - r, 0); z <= min(cz + r, DZ - 1); ++z)
      for (int y = max(cy - r, 0); y <= min(cy + r, DY - 1); ++y) {
        if (abs(z - cz) == r || abs(y - cy) == r) {
          for (int x = max(cx - r, 0); x <= min(cx + r, DX - 1); ++x) visit(x, y, z);
        } else {
          if (cx - r >= 0) visit(cx - r, y, z);
          if (r > 0 && cx + r < DX) visit(cx + r, y, z);
        }
      }
    if (r >= 1 && (double)d[2] <= ((double)r - 0.001) * (double)g.h) break;
    if (cx - r <= 0 && cy - r <= 0 && cz - r <= 0 && cx + r >= DX - 1 && cy + r >= DY - 1 &&
        cz + r >= DZ - 1)
      break;  // every cell visited
  }
  const float mean = ((d[0] + d[1]) + d[2]) / 3.0f;
  const float lo_s = extent * 0.0007f, hi_s = extent * 0.007f, bias = extent * 0.0015f;
  float sig = fmax_(mean / 3.0f, bias);
  sig = clampf_(sig, lo_s, hi_s);
  sig = fmin_(sig, 0.1f);
  if (density) density[self] = mean;
  log_sigma[self] = round_f16(sky_logf(fmax_(sig, 1e-6f)));
}

__global__ void __launch_bounds__(256)
k_knn_write(float* __restrict__ P, uint32_t stride, uint32_t n, const float* __restrict__ ls) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  for (int k = 0; k < 59; ++k) {
    float* v = P + (size_t)k * stride + i;
    *v = (k >= 3 && k < 6) ? ls[i] : round_f16(*v);
  }
}

uint32_t blocks(uint32_t n) { return (n + 255) / 256; }

}  // namespace

uint32_t knn_bounds_init(int k) { return k < 3 ? 0xFFFFFFFFu : 0u; }

float knn_bounds_decode(uint32_t u) {
  const uint32_t b = (u & 0x80000000u) ? (u & 0x7FFFFFFFu) : ~u;
  float f;
  memcpy(&f, &b, 4);
  return f;
}

void launch_knn_bounds(const float* params, uint32_t stride, uint32_t n, uint32_t* out,
                       cudaStream_t s) {
  if (n) k_knn_bounds<<<min(blocks(n), 1024u), 256, 0, s>>>(params, stride, n, out);
}

void launch_knn_keys(const float* params, uint32_t stride, uint32_t n, const KnnGrid& g,
                     uint32_t* keys, cudaStream_t s) {
  if (n) k_knn_keys<<<blocks(n), 256, 0, s>>>(params, stride, n, g, keys);
}

void launch_knn_cell_ranges(const uint32_t* keys_sorted, uint32_t n, uint32_t cells,
                            uint32_t* cell_start, cudaStream_t s) {
  k_knn_cell_ranges<<<blocks(cells + 1), 256, 0, s>>>(keys_sorted, n, cells, cell_start);
}

void launch_knn_query(float* params, uint32_t stride, uint32_t n, const KnnGrid& g,
                      const uint32_t* order, const uint32_t* cell_start, float extent,
                      float* density, float* log_sigma, cudaStream_t s) {
  if (n)
    k_knn_query<<<blocks(n), 256, 0, s>>>(params, stride, n, g, order, cell_start, extent, density,
                                          log_sigma);
}

void launch_knn_write(float* params, uint32_t stride, uint32_t n, const float* log_sigma,
                      cudaStream_t s) {
  if (n) k_knn_write<<<blocks(n), 256, 0, s>>>(params, stride, n, log_sigma);
}

}  // namespace sky
