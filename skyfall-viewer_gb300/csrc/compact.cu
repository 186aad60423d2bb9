// Prune flags, order-preserving stream compaction of the parameter planes,
// and the opacity reset -- the device versions of the reference's CPU
// round trips applyPruneMask (gaussian-renderer.ts:2917-3000) and
// resetOpacity (:3867-3906).
#include "kernels.cuh"
#include "sky_math.cuh"

namespace sky {
namespace {

// keep flag (1 = survivor) per Gaussian: prunable when sigmoid(logit) <
// min_opacity or max(exp(log sigma)) > max_scale (applyMultiViewPrune
// :2840-2858), or when the caller's mask says so.
__global__ void k_prune_flags(const float* __restrict__ P, uint32_t stride, uint32_t n,
                              float min_opacity, float max_scale, const uint8_t* __restrict__ mask,
                              uint32_t* __restrict__ flags) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  bool prune;
  if (mask) {
    prune = mask[i] != 0;
  } else {
    const float logit = P[(size_t)10 * stride + i];
    const double op = 1.0 / (1.0 + exp(-(double)logit));
    const double s0 = exp((double)P[(size_t)3 * stride + i]);
    const double s1 = exp((double)P[(size_t)4 * stride + i]);
    const double s2 = exp((double)P[(size_t)5 * stride + i]);
    const double ms = fmax(fmax(s0, s1), s2);
    prune = op < (double)min_opacity || ms > (double)max_scale;
  }
  flags[i] = prune ? 0u : 1u;
}

// dst plane k, position scan[i] - 1 <- src plane k, position i, for survivors.
// One thread per Gaussian walks all planes (the survivor test is read once;
// eight plane loads in flight per thread), neighbouring threads touching
// neighbouring addresses of each plane.
__global__ void __launch_bounds__(256) k_compact(const float* __restrict__ src, float* __restrict__ dst,
                                                 uint32_t src_stride, uint32_t dst_stride,
                                                 uint32_t planes, uint32_t n,
                                                 const uint32_t* __restrict__ keep_scan) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint32_t incl = keep_scan[i];
  const uint32_t prev = i ? keep_scan[i - 1] : 0u;
  if (incl == prev) return;
  const size_t d = incl - 1;
#pragma unroll 8
  for (uint32_t k = 0; k < planes; ++k)
    dst[(size_t)k * dst_stride + d] = src[(size_t)k * src_stride + i];
}

__global__ void k_reset_opacity(float* __restrict__ P, uint32_t stride, uint32_t n, float max_logit) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float* v = P + (size_t)10 * stride + i;
  if (*v > max_logit) *v = max_logit;
}

}  // namespace

void launch_prune_flags(const float* params, uint32_t stride, uint32_t n, float min_opacity,
                        float max_scale, const uint8_t* mask, uint32_t* flags, cudaStream_t s) {
  if (n == 0) return;
  k_prune_flags<<<(n + 255) / 256, 256, 0, s>>>(params, stride, n, min_opacity, max_scale, mask,
                                                flags);
}

void launch_compact(const float* src, float* dst, uint32_t src_stride, uint32_t dst_stride,
                    uint32_t planes, uint32_t n, const uint32_t* keep_scan, cudaStream_t s) {
  if (n == 0) return;
  k_compact<<<(n + 255) / 256, 256, 0, s>>>(src, dst, src_stride, dst_stride, planes, n, keep_scan);
}

void launch_reset_opacity(float* params, uint32_t stride, uint32_t n, float max_logit,
                          cudaStream_t s) {
  if (n == 0) return;
  k_reset_opacity<<<(n + 255) / 256, 256, 0, s>>>(params, stride, n, max_logit);
}

}  // namespace sky
