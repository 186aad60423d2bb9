// Launch interface of multi-view scoring, densification and scored pruning
// (densify.cu).
#pragma once

#include "sky_types.cuh"

namespace sky {

// Statistics of one view's per-pixel L1 map (computePixelLossStats,
// gaussian-renderer.ts:2706-2743).
struct MetricStats {
  float min_value, max_value, inv_range, pad;
  double mean;
};

// Candidate rule of performDensification (gaussian-renderer.ts:3248-3290),
// all in f64 as the reference's JavaScript evaluates it.
struct DensifyRule {
  double grad_px;          // grad_threshold * width / 2
  double grad_abs_px;      // grad_abs_threshold * width / 2
  double size_threshold;   // scene extent * dense size ratio
  double min_visibility;   // max(1, min_visibility)
  double importance_threshold;
  double sample_count;     // views scored
};

// Prunable rule and selection weights of applyMultiViewPrune
// (gaussian-renderer.ts:2836-2886).
struct PruneRule {
  double min_opacity, max_scale, max_screen_radius;
  double opacity_bonus, scale_bonus, screen_bonus;
  uint32_t use_screen, pad[3];
};

// Uniform double in (0, 1) from a counter-based generator: draw `draw` of
// Gaussian `index` at training iteration `iteration` under `seed`.
__host__ __device__ inline double counter_uniform(uint64_t seed, uint64_t iteration, uint64_t index,
                                                  uint32_t draw) {
  uint64_t z = seed * 0x9E3779B97F4A7C15ull + iteration * 0xD1B54A32D192ED03ull +
               index * 0x94D049BB133111EBull + (uint64_t)draw * 0xBF58476D1CE4E5B9ull +
               0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  z = z ^ (z >> 31);
  return ((double)(z >> 11) + 0.5) * (1.0 / 9007199254740992.0);
}

void launch_metric_map(const float4* color, const float4* target, uint32_t pixel_base,
                       uint32_t target_base, uint32_t npx, float* l1, cudaStream_t s);
// nblocks partial slots in pmin/pmax/psum; result in *out.
void launch_metric_stats(const float* l1, uint32_t npx, float* pmin, float* pmax, double* psum,
                         uint32_t nblocks, MetricStats* out, cudaStream_t s);
void launch_metric_accum(const DevBuffers& b, uint32_t view, uint32_t npx, const float* l1,
                         const MetricStats* st, float threshold, uint32_t* counts, cudaStream_t s);
// importance += counts, pruning += counts * mean (f32, as the reference's
// Float32Array), counts reset to 0.
void launch_metric_combine(uint32_t* counts, uint32_t n, const MetricStats* st,
                           uint32_t* importance, float* pruning, cudaStream_t s);

// action (0 none, 1 clone, 2 split) and a 64-bit sort key (two u32 halves)
// ordering candidates by descending score, then index; ncand counts them.
void launch_densify_decide(const float* P, uint32_t stride, uint32_t n, const float4* accum,
                           const uint32_t* importance, const DensifyRule& rule, uint32_t* action,
                           uint32_t* key_lo, uint32_t* key_hi, uint32_t* ncand, cudaStream_t s);
void launch_gather_u32(const uint32_t* src, const uint32_t* idx, uint32_t n, uint32_t* dst,
                       cudaStream_t s);
// keep (1 unless split) and new-count (1 clone, 2 split) flags of the first
// `allowed` candidates in `order`.
void launch_densify_select(const uint32_t* order, uint32_t n, uint32_t allowed,
                           const uint32_t* action, uint32_t* keep, uint32_t* newc, cudaStream_t s);
void launch_densify_build(const float* P, const float* M1, const float* M2, uint32_t stride,
                          uint32_t n, const uint32_t* keep_scan, const uint32_t* new_scan,
                          uint32_t survivors, float* NP, float* NM1, float* NM2, uint32_t nstride,
                          uint64_t seed, uint64_t iteration, cudaStream_t s);

// Normalised pruning scores (scores - min) / max(1e-6, max - min) for
// positions < base (0 beyond), as f32.
void launch_prune_normalise(const float* scores, uint32_t base, uint32_t n, float* norm,
                            float* pmin, float* pmax, uint32_t nblocks, cudaStream_t s);
void launch_prune_weights(const float* P, uint32_t stride, uint32_t n, const float* norm,
                          const float4* importance, const PruneRule& rule, uint32_t* key_lo,
                          uint32_t* key_hi, uint32_t* nprunable, uint64_t seed, uint64_t iteration,
                          cudaStream_t s);
// keep = 0 for the first `budget` Gaussians in `order`, 1 for the rest.
void launch_prune_select(const uint32_t* order, uint32_t n, uint32_t budget, uint32_t* keep,
                         cudaStream_t s);

}  // namespace sky
