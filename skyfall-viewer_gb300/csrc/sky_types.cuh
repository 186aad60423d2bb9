// Types shared by the host runtime and the kernels of the skyfall library.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace sky {

constexpr int kMaxViews = 64;   // views per step
constexpr int kMaxGroups = 16;  // sort groups per step
constexpr int kPlanes = 59;     // parameter planes per Gaussian
constexpr int kPartialF4 = 3;   // float4 per intersection partial (9 values used)

// One view of a step.  Global tile t of the step belongs to the view with
// tile_base <= t < tile_base + tiles_x * tiles_y; its sort key holds
// key_tile = t - (first tile of the view's sort group).
struct ViewInfo {
  float view[16];   // column-major world -> camera
  float proj[16];   // column-major projection
  float focal[2];
  uint32_t width, height;
  uint32_t tiles_x, tiles_y;
  uint32_t tile_base;
  uint32_t group;
  uint32_t key_tile_base;
  uint32_t pixel_base;   // first pixel of the view in the step's image buffers
  uint32_t target_base;  // first pixel of the camera's target image
  uint32_t has_target;
  uint32_t camera;
  uint32_t pad[3];
};

struct GroupInfo {
  uint32_t tile_begin, tile_end;  // global tiles of the group
  uint32_t item_begin, item_end;  // (view, Gaussian) items of the group
  uint32_t key_bits;
  uint32_t pad[3];
};

// Everything a step's kernels read that is not a buffer.  Lives in device
// memory and is refreshed by one host-to-device copy per step (also inside a
// captured graph, where the copy reads the pinned host mirror at replay).
struct StepParams {
  uint32_t num_views, n, num_tiles, num_groups;
  uint32_t sh_deg, sh_update, bwd_mode, round_f16;
  uint32_t tile_size, has_loss, apply_adam, write_grads;
  uint32_t icap, num_pixels, plane_stride;
  uint32_t tile_cull;  // 1: items list only the tiles their alpha >= 1/255 ellipse reaches
  float near_plane, far_plane, radius_clip, eps2d;
  float bg[4];
  float w_l2, w_l1, w_ssim, pad1;
  float lr_pos, lr_scale, lr_rot, lr_opacity;
  float lr_sh, beta1, beta2, adam_eps;
  float bc1_rcp, bc2_sqrt_rcp, importance_decay, pad3;
  GroupInfo groups[kMaxGroups];
  ViewInfo views[kMaxViews];
};

// Device status of a step, copied back to the host after it.
struct DevStatus {
  uint32_t error;        // SKY_DEVERR_* bits
  uint32_t total_isect;  // intersections of the step (unclamped)
  uint32_t pad[2];
  uint32_t group_bounds[kMaxGroups][2];  // [begin, end) clamped to capacity
  double loss;
  double pad2;
  // Work counters of the rasterizers, filled only by their counting variants
  // (profiling level 2): forward (pixel, splat) pairs evaluated, pairs
  // composited, warp list entries; backward pixel pairs evaluated, pairs
  // contributing, warp list entries (each entry covers 64 pixels), entries
  // at which no pixel of the warp contributed; one spare word.
  unsigned long long pairs[8];
};

// Device buffers of a context (all owned by the host runtime).
struct DevBuffers {
  float* params;
  float* m1;
  float* m2;
  float* grads;
  float4* records;    // 3 float4 per (view, Gaussian) item: raster record
  float2* aux;        // depth, radius per item
  uint32_t* counts;   // tiles per item
  uint2* rects;       // packed tile rectangle per item
  uint4* rowspans;    // culled lists: per item of at most kSpanRows rows, each row's
                      // tile span (first tile - x0, length) as two bytes
  uint32_t* ikeys;    // per item (min(count, 0xFFFF) << 16) | depth16; sorted on depth16
                      // per group
  uint32_t* ikeys_sorted;  // the item keys in emission (perm) order
  uint32_t* perm;     // item at each emission position: by (group, depth16, item)
                      // (NULL: item order)
  uint32_t* cumsum;   // inclusive scan of counts, in perm order
  uint32_t* item_end; // per item, the end of its emitted range (cumsum at its position)
  uint32_t* block_sums;
  uint32_t* keys;         // emission order
  uint32_t* keys_sorted;
  uint32_t* vals_sorted;  // emission index per sorted intersection
  uint32_t* rec_of;       // item per emitted intersection
  uint32_t* flatten;      // item per sorted intersection
  uint8_t* fmask;         // 16x16 tiles: per sorted intersection the forward staged, its
                          // 8x4-block ellipse mask (bit 2 band + column)
  float4* partials;       // 3 float4 per intersection (emission order)
  uint8_t* reached;       // per emission index: 1 when the exact backward wrote its partial
  float4* item_sums;      // exact mode: 3 float4 per item, its partials summed
  int32_t* tile_grads;    // reference mode: 54 per sorted intersection
  long long* gsum54;      // reference mode: 54 per item
  uint32_t* offsets;      // tile ranges, num_tiles + 1
  double* loss_partials;  // per tile
  float4* color;
  float* alpha;
  float* tfinal;      // final transmittance, product of (1 - alpha)
  uint32_t* last;
  float4* residual;
  const float4* targets;  // all cameras' target images
  float* densify_accum;   // 4 per Gaussian: |dmean2d| sum, 0, |dconic| sum, count
  float* importance;      // 4 per Gaussian: sum, count, max radius, 0
  const StepParams* sp;
  DevStatus* status;
};

}  // namespace sky
