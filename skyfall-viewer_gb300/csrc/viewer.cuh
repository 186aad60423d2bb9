// Launch interface of the headless viewer render (viewer.cu).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace sky {

constexpr int kViewTile = 16;

// Everything the viewer kernels read that is not a buffer.
struct ViewerParams {
  float view[16], proj[16];
  float focal[2];
  float viewport[2];        // RenderSettings.viewport_x / viewport_y
  float gaussian_scaling;   // RenderSettings.gaussian_scaling
  uint32_t sh_deg;          // RenderSettings.sh_deg
  uint32_t round_f16;       // parameters read through f16 storage
  uint32_t n, plane_stride;
  uint32_t width, height, tiles_x, tiles_y;
};

// Per Gaussian: 3 float4 {cx, cy, a, b | c, opacity, r, g | b, radius, 0, 0},
// the depth sort key (0xFFFFFFFF when culled), the tile count and rectangle;
// *total (zeroed by the caller) receives the sum of the tile counts.
void launch_viewer_project(const ViewerParams& vp, const float* params, float4* splats,
                           uint32_t* keys, uint32_t* counts, uint2* rects,
                           unsigned long long* total, cudaStream_t s);
// Intersections in depth order: for sorted position k (Gaussian order[k])
// its tiles at cum[k] - counts[order[k]] ..., value = Gaussian index.
void launch_viewer_gather_counts(const uint32_t* order, const uint32_t* counts, uint32_t n,
                                 uint32_t* counts_sorted, cudaStream_t s);
void launch_viewer_emit(const ViewerParams& vp, const uint32_t* order, const uint32_t* cum,
                        const uint32_t* counts_sorted, const uint2* rects, uint32_t n,
                        uint32_t* tile_keys, uint32_t* gidx, cudaStream_t s);
// offsets[t] = first intersection of tile t (lower bound), offsets[T] = total.
void launch_viewer_ranges(const uint32_t* tile_keys, uint32_t total, uint32_t tiles,
                          uint32_t* offsets, cudaStream_t s);
// Back-to-front "over" blending of every splat whose quad covers the pixel.
void launch_viewer_raster(const ViewerParams& vp, const float4* splats, const uint32_t* offsets,
                          const uint32_t* gidx, float4* rgba, cudaStream_t s);

}  // namespace sky
