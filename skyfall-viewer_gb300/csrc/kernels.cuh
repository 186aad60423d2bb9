// Launch interface of the hot-path kernels (kernels.cu).
#pragma once

#include "sky_types.cuh"
#include "sort.cuh"

namespace sky {

void launch_preprocess(const DevBuffers& b, uint32_t n, uint32_t views, cudaStream_t s);
void launch_scan(const DevBuffers& b, uint32_t n_items, cudaStream_t s);
uint32_t scan_block_count(uint32_t n_items);
void launch_group_bounds(const DevBuffers& b, cudaStream_t s);
void launch_emit(const DevBuffers& b, uint32_t n, uint32_t views, cudaStream_t s);
void launch_ranges(const DevBuffers& b, uint32_t icap, cudaStream_t s);
// Zeroes the partials the last exact backward left unwritten, for a read-back.
void launch_partials_fill(const DevBuffers& b, uint32_t total, cudaStream_t s);
// Completes flatten (the item of every sorted intersection) for a read-back.
void launch_flatten_fill(const DevBuffers& b, uint32_t total, cudaStream_t s);
// Splat-batch depths of the rasterizers: the forward stages fb splats per
// batch (64, 128 or 256), the 16x16-tile exact backward bb (32, 64 or 128);
// other values select the defaults.  Results do not depend on them.
constexpr uint32_t kBwdBatch16 = 64;  // default backward depth for 16x16 tiles
// count: the pair-counting variants (16x16 tiles at the default depths
// only; other shapes launch the plain kernels and count nothing).
void launch_forward(const DevBuffers& b, uint32_t max_tiles, uint32_t ts, uint32_t fb, bool ssim,
                    uint32_t views, uint32_t max_view_pixels, bool count, cudaStream_t s);
void launch_loss_final(const DevBuffers& b, cudaStream_t s);
void launch_backward(const DevBuffers& b, uint32_t max_tiles, uint32_t ts, uint32_t bb, bool ref,
                     bool count, cudaStream_t s);
void launch_geom_adam(const DevBuffers& b, uint32_t n, cudaStream_t s);
// Exact mode, before launch_geom_adam: per-item sums of the partials.
void launch_item_sums(const DevBuffers& b, uint64_t items, cudaStream_t s);

// Prune / densify / opacity reset (compact.cu).
void launch_prune_flags(const float* params, uint32_t stride, uint32_t n, float min_opacity,
                        float max_scale, const uint8_t* mask, uint32_t* flags, cudaStream_t s);
void launch_compact(const float* src, float* dst, uint32_t src_stride, uint32_t dst_stride,
                    uint32_t planes, uint32_t n, const uint32_t* keep_scan, cudaStream_t s);
void launch_reset_opacity(float* params, uint32_t stride, uint32_t n, float max_logit,
                          cudaStream_t s);

}  // namespace sky
