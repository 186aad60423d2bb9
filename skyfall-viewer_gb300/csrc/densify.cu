// Multi-view scoring, densification and scored pruning on the device: the
// reference's metric maps (metric-map.wgsl:32-147 with the host statistics of
// gaussian-renderer.ts:2706-2788), the clone/split decision and construction
// of performDensification (:3211-3433) and the weighted prune of
// applyMultiViewPrune (:2800-2915).  The reference reads every training
// buffer back to the CPU for these; here only a few counters cross the bus.
//
// Random draws (clone jitter, split samples, prune selection) come from
// counter_uniform: draw r of Gaussian i at iteration t, so the results are
// reproducible and independent of launch order.  The reference draws from
// Math.random() in index order; the distributions are the same.
#include "densify.cuh"
#include "sky_math.cuh"

namespace sky {
namespace {

constexpr uint32_t kFull = 0xFFFFFFFFu;

// Per-pixel L1 map of one view (compute_metric_map, metric-map.wgsl:32-50).
// The target is sampled at texel centres of an image of the view's size, so
// the bilinear sample is the texel itself.
__global__ void k_metric_map(const float4* __restrict__ color, const float4* __restrict__ target,
                             uint32_t pixel_base, uint32_t target_base, uint32_t npx,
                             float* __restrict__ l1) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= npx) return;
  const float4 p = color[(size_t)pixel_base + i];
  const float4 t = target[(size_t)target_base + i];
  const float dr = fabsf(p.x - t.x), dg = fabsf(p.y - t.y), db = fabsf(p.z - t.z);
  l1[i] = ((dr + dg) + db) / 3.0f;
}

// Block partials of min, max (order-independent) and the f64 sum of the map.
__global__ void __launch_bounds__(256)
k_metric_partials(const float* __restrict__ l1, uint32_t npx, float* __restrict__ pmin,
                  float* __restrict__ pmax, double* __restrict__ psum) {
  __shared__ float smin[8], smax[8];
  __shared__ double ssum[8];
  float mn = INFINITY, mx = -INFINITY;
  double sm = 0.0;
  for (uint32_t i = blockIdx.x * 256 + threadIdx.x; i < npx; i += gridDim.x * 256) {
    const float v = l1[i];
    if (!isfinite(v)) continue;  // computePixelLossStats skips non-finite values
    mn = fminf(mn, v);
    mx = fmaxf(mx, v);
    sm += (double)v;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    mn = fminf(mn, __shfl_xor_sync(kFull, mn, o));
    mx = fmaxf(mx, __shfl_xor_sync(kFull, mx, o));
    sm += __shfl_xor_sync(kFull, sm, o);
  }
  const int w = threadIdx.x >> 5;
  if ((threadIdx.x & 31) == 0) {
    smin[w] = mn;
    smax[w] = mx;
    ssum[w] = sm;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    float a = smin[0], b = smax[0];
    double t = ssum[0];
    for (int k = 1; k < 8; ++k) {
      a = fminf(a, smin[k]);
      b = fmaxf(b, smax[k]);
      t += ssum[k];
    }
    pmin[blockIdx.x] = a;
    pmax[blockIdx.x] = b;
    psum[blockIdx.x] = t;
  }
}

__global__ void k_metric_final(const float* __restrict__ pmin, const float* __restrict__ pmax,
                               const double* __restrict__ psum, uint32_t nblocks, uint32_t npx,
                               MetricStats* __restrict__ out) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  float mn = INFINITY, mx = -INFINITY;
  double sm = 0.0;
  for (uint32_t k = 0; k < nblocks; ++k) {
    mn = fminf(mn, pmin[k]);
    mx = fmaxf(mx, pmax[k]);
    sm += psum[k];
  }
  out->min_value = mn;
  out->max_value = mx;
  out->pad = 0.0f;
  out->mean = npx ? sm / (double)npx : 0.0;
  // invRange in f64, written to the f32 threshold uniform
  out->inv_range = mx > mn ? (float)(1.0 / ((double)mx - (double)mn)) : 0.0f;
}

// threshold_metric_map (:56-66) and accumulate_metric_counts (:86-147): for
// every flagged pixel, each intersection of its tile up to the pixel's last
// visited one whose Gaussian has 0 <= s <= 6 there adds one to that Gaussian.
__global__ void __launch_bounds__(256)
k_metric_accum(DevBuffers b, uint32_t view, const float* __restrict__ l1,
               const MetricStats* __restrict__ st, float threshold, uint32_t* __restrict__ counts) {
  const StepParams& sp = *b.sp;
  const ViewInfo& vi = sp.views[view];
  const uint32_t npx = vi.width * vi.height;
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= npx) return;
  const float value = (l1[i] - st->min_value) * st->inv_range;
  if (!(value > threshold)) return;
  const uint32_t x = i % vi.width, y = i / vi.width;
  const uint32_t ts = sp.tile_size;
  const uint32_t tile = vi.tile_base + (y / ts) * vi.tiles_x + (x / ts);
  const uint32_t start = b.offsets[tile], end = b.offsets[tile + 1];
  if (start >= end) return;
  const uint32_t last = b.last[(size_t)vi.pixel_base + i];
  if (last < start) return;
  const uint32_t fin = min(last, end - 1);
  const float px = (float)x + 0.5f, py = (float)y + 0.5f;
  for (uint32_t k = start; k <= fin; ++k) {
    const uint32_t r = b.flatten[k];
    const float4 q0 = b.records[(size_t)r * 3 + 0];
    const float cc = b.records[(size_t)r * 3 + 1].x;
    const float dx = px - q0.x, dy = py - q0.y;
    const float s = 0.5f * ((q0.z * dx) * dx + (cc * dy) * dy) + (q0.w * dx) * dy;
    if (s < 0.0f || s > 6.0f) continue;
    atomicAdd(&counts[r % sp.n], 1u);
  }
}

__global__ void k_metric_combine(uint32_t* __restrict__ counts, uint32_t n,
                                 const MetricStats* __restrict__ st,
                                 uint32_t* __restrict__ importance, float* __restrict__ pruning) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint32_t c = counts[i];
  importance[i] += c;
  pruning[i] = (float)((double)pruning[i] + (double)c * st->mean);
  counts[i] = 0u;
}

__device__ double max_sigma(const float* __restrict__ P, uint32_t stride, uint32_t i) {
  const double s0 = exp((double)P[(size_t)3 * stride + i]);
  const double s1 = exp((double)P[(size_t)4 * stride + i]);
  const double s2 = exp((double)P[(size_t)5 * stride + i]);
  return fmax(fmax(s0, s1), s2);
}

__global__ void k_densify_decide(const float* __restrict__ P, uint32_t stride, uint32_t n,
                                 const float4* __restrict__ accum,
                                 const uint32_t* __restrict__ importance, DensifyRule rule,
                                 uint32_t* __restrict__ action, uint32_t* __restrict__ key_lo,
                                 uint32_t* __restrict__ key_hi, uint32_t* __restrict__ ncand) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  uint32_t act = 0;
  double score = 0.0;
  const float4 a = accum[i];
  const double denom = (double)a.w;
  if (!(denom < rule.min_visibility)) {
    const double avg = (double)a.x / denom, avg_abs = (double)a.z / denom;
    const double ms = max_sigma(P, stride, i);
    const double imp = (double)importance[i] / fmax(1.0, rule.sample_count);
    if (imp > rule.importance_threshold) {
      if (ms <= rule.size_threshold && avg >= rule.grad_px) {
        act = 1;
        score = rule.grad_px > 1e-8 ? avg / rule.grad_px : avg;
      } else if (ms > rule.size_threshold && avg_abs >= rule.grad_abs_px) {
        act = 2;
        score = rule.grad_abs_px > 1e-8 ? avg_abs / rule.grad_abs_px : avg_abs;
      }
    }
  }
  action[i] = act;
  // Ascending key = descending score; the stable sort keeps index order
  // among equal scores.  Scores are >= 0, so their bit patterns order like
  // the values; candidates clear the top bit, which every other key keeps.
  uint64_t key = ~0ull;
  if (act) {
    key = ~(uint64_t)__double_as_longlong(score) & 0x7FFFFFFFFFFFFFFFull;
    atomicAdd(ncand, 1u);
  }
  key_lo[i] = (uint32_t)key;
  key_hi[i] = (uint32_t)(key >> 32);
}

__global__ void k_gather_u32(const uint32_t* __restrict__ src, const uint32_t* __restrict__ idx,
                             uint32_t n, uint32_t* __restrict__ dst) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) dst[i] = src[idx[i]];
}

__global__ void k_densify_select(const uint32_t* __restrict__ order, uint32_t n, uint32_t allowed,
                                 const uint32_t* __restrict__ action, uint32_t* __restrict__ keep,
                                 uint32_t* __restrict__ newc) {
  const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  const uint32_t i = order[k];  // a permutation: one writer per Gaussian
  const uint32_t a = k < allowed ? action[i] : 0u;
  keep[i] = a == 2u ? 0u : 1u;
  newc[i] = a;  // clone adds 1 Gaussian, split adds 2
}

// New planes: survivors (everything but split originals) in index order,
// then per selected candidate in index order its clone or its two split
// samples, with zero Adam moments (performDensification :3325-3420).
__global__ void k_densify_build(const float* __restrict__ P, const float* __restrict__ M1,
                                const float* __restrict__ M2, uint32_t stride, uint32_t n,
                                const uint32_t* __restrict__ keep_scan,
                                const uint32_t* __restrict__ new_scan, uint32_t survivors,
                                float* __restrict__ NP, float* __restrict__ NM1,
                                float* __restrict__ NM2, uint32_t nstride, uint64_t seed,
                                uint64_t iteration) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint32_t kin = keep_scan[i], kprev = i ? keep_scan[i - 1] : 0u;
  const uint32_t nin = new_scan[i], nprev = i ? new_scan[i - 1] : 0u;
  if (kin != kprev) {
    const uint32_t o = kin - 1;
    for (int p = 0; p < kPlanes; ++p) {
      NP[(size_t)p * nstride + o] = P[(size_t)p * stride + i];
      NM1[(size_t)p * nstride + o] = M1[(size_t)p * stride + i];
      NM2[(size_t)p * nstride + o] = M2[(size_t)p * stride + i];
    }
  }
  const uint32_t made = nin - nprev;
  if (made == 0) return;
  const uint32_t o = survivors + nprev;
  for (uint32_t m = 0; m < made; ++m)
    for (int p = 0; p < kPlanes; ++p) {
      NP[(size_t)p * nstride + o + m] = P[(size_t)p * stride + i];
      NM1[(size_t)p * nstride + o + m] = 0.0f;
      NM2[(size_t)p * nstride + o + m] = 0.0f;
    }
  const double s0 = P[(size_t)3 * stride + i], s1 = P[(size_t)4 * stride + i],
               s2 = P[(size_t)5 * stride + i];
  const double sig[3] = {exp(s0), exp(s1), exp(s2)};
  const double pos[3] = {P[i], P[(size_t)stride + i], P[(size_t)2 * stride + i]};
  if (made == 1) {
    // clone: offset by max sigma * 0.25 * U(0.5, 1) along a random direction
    const double mag = fmax(fmax(sig[0], sig[1]), sig[2]) * 0.25 *
                       (0.5 + counter_uniform(seed, iteration, i, 0) * 0.5);
    double d[3];
    for (int k = 0; k < 3; ++k) d[k] = counter_uniform(seed, iteration, i, 1 + k) * 2.0 - 1.0;
    double nrm = sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
    if (nrm == 0.0) nrm = 1.0;
    for (int k = 0; k < 3; ++k) NP[(size_t)k * nstride + o] = (float)(pos[k] + d[k] / nrm * mag);
    return;
  }
  // split: two samples of N(0, diag(sigma^2)) by Box-Muller, rotated by the
  // matrix of the (unnormalised) quaternion; log sigma - ln(1.6)
  const double x = P[(size_t)6 * stride + i], y = P[(size_t)7 * stride + i],
               z = P[(size_t)8 * stride + i], w = P[(size_t)9 * stride + i];
  const double x2 = x + x, y2 = y + y, z2 = z + z;
  const double xx = x * x2, xy = x * y2, xz = x * z2, yy = y * y2, yz = y * z2, zz = z * z2;
  const double wx = w * x2, wy = w * y2, wz = w * z2;
  const double R[3][3] = {{1 - (yy + zz), xy - wz, xz + wy},
                          {xy + wz, 1 - (xx + zz), yz - wx},
                          {xz - wy, yz + wx, 1 - (xx + yy)}};
  const double red = log(0.8 * 2.0);
  const double two_pi = 6.283185307179586;
  for (int smp = 0; smp < 2; ++smp) {
    const double u1 = counter_uniform(seed, iteration, i, 4 + 4 * smp);
    const double u2 = counter_uniform(seed, iteration, i, 5 + 4 * smp);
    const double u3 = counter_uniform(seed, iteration, i, 6 + 4 * smp);
    const double u4 = counter_uniform(seed, iteration, i, 7 + 4 * smp);
    const double r1 = sqrt(-2.0 * log(u1)), r3 = sqrt(-2.0 * log(u3));
    const double l[3] = {r1 * cos(two_pi * u2) * sig[0], r1 * sin(two_pi * u2) * sig[1],
                         r3 * cos(two_pi * u4) * sig[2]};
    const uint32_t at = o + smp;
    for (int k = 0; k < 3; ++k)
      NP[(size_t)k * nstride + at] =
          (float)(pos[k] + (R[k][0] * l[0] + R[k][1] * l[1] + R[k][2] * l[2]));
    NP[(size_t)3 * nstride + at] = (float)(s0 - red);
    NP[(size_t)4 * nstride + at] = (float)(s1 - red);
    NP[(size_t)5 * nstride + at] = (float)(s2 - red);
  }
}

// Min and max of the finite scores of positions < base (block partials).
__global__ void __launch_bounds__(256)
k_score_partials(const float* __restrict__ scores, uint32_t base, float* __restrict__ pmin,
                 float* __restrict__ pmax) {
  __shared__ float smin[8], smax[8];
  float mn = INFINITY, mx = -INFINITY;
  for (uint32_t i = blockIdx.x * 256 + threadIdx.x; i < base; i += gridDim.x * 256) {
    const float v = scores[i];
    if (!isfinite(v)) continue;
    mn = fminf(mn, v);
    mx = fmaxf(mx, v);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    mn = fminf(mn, __shfl_xor_sync(kFull, mn, o));
    mx = fmaxf(mx, __shfl_xor_sync(kFull, mx, o));
  }
  const int w = threadIdx.x >> 5;
  if ((threadIdx.x & 31) == 0) {
    smin[w] = mn;
    smax[w] = mx;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    float a = smin[0], b = smax[0];
    for (int k = 1; k < 8; ++k) {
      a = fminf(a, smin[k]);
      b = fmaxf(b, smax[k]);
    }
    pmin[blockIdx.x] = a;
    pmax[blockIdx.x] = b;
  }
}

__global__ void k_score_normalise(const float* __restrict__ scores, uint32_t base, uint32_t n,
                                  const float* __restrict__ pmin, const float* __restrict__ pmax,
                                  uint32_t nblocks, float* __restrict__ norm) {
  __shared__ double s_min, s_range;
  if (threadIdx.x == 0) {
    float mn = INFINITY, mx = -INFINITY;
    for (uint32_t k = 0; k < nblocks; ++k) {
      mn = fminf(mn, pmin[k]);
      mx = fmaxf(mx, pmax[k]);
    }
    double dmn = mn, dmx = mx;
    if (!isfinite(dmn) || !isfinite(dmx)) {
      dmn = 0.0;
      dmx = 1.0;
    }
    s_min = dmn;
    s_range = fmax(1e-6, dmx - dmn);
  }
  __syncthreads();
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  norm[i] = i < base ? (float)(((double)scores[i] - s_min) / s_range) : 0.0f;
}

// Prunable test and weighted-sampling key of applyMultiViewPrune.  The
// reference draws removeBudget Gaussians one after another with probability
// proportional to w among those left; sorting by -log(u) / w ascending and
// taking the first removeBudget draws from the same distribution
// (Efraimidis & Spirakis, "Weighted random sampling with a reservoir", 2006).
__global__ void k_prune_weights(const float* __restrict__ P, uint32_t stride, uint32_t n,
                                const float* __restrict__ norm, const float4* __restrict__ imp,
                                PruneRule rule, uint32_t* __restrict__ key_lo,
                                uint32_t* __restrict__ key_hi, uint32_t* __restrict__ nprunable,
                                uint64_t seed, uint64_t iteration) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double op = 1.0 / (1.0 + exp(-(double)P[(size_t)10 * stride + i]));
  const bool low = op < rule.min_opacity;
  const bool large = max_sigma(P, stride, i) > rule.max_scale;
  bool screen = false;
  if (rule.use_screen && imp) {
    const float r = imp[i].z;
    screen = isfinite(r) && (double)r > rule.max_screen_radius;
  }
  uint64_t key = ~0ull;
  if (low || large || screen) {
    double ws = (double)norm[i];
    if (!isfinite(ws)) ws = 0.0;
    if (low) ws += rule.opacity_bonus;
    if (large) ws += rule.scale_bonus;
    if (screen) ws += rule.screen_bonus;
    ws = fmin(0.999, fmax(0.0, ws));
    const double w = 1.0 / (1e-6 + (1.0 - ws));
    const double e = -log(counter_uniform(seed, iteration, i, 64)) / w;  // > 0
    key = (uint64_t)__double_as_longlong(e) & 0x7FFFFFFFFFFFFFFFull;
    atomicAdd(nprunable, 1u);
  }
  key_lo[i] = (uint32_t)key;
  key_hi[i] = (uint32_t)(key >> 32);
}

__global__ void k_prune_select(const uint32_t* __restrict__ order, uint32_t n, uint32_t budget,
                               uint32_t* __restrict__ keep) {
  const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  keep[order[k]] = k < budget ? 0u : 1u;
}

uint32_t blocks_for(uint32_t n, uint32_t threads) { return (n + threads - 1) / threads; }

}  // namespace

void launch_metric_map(const float4* color, const float4* target, uint32_t pixel_base,
                       uint32_t target_base, uint32_t npx, float* l1, cudaStream_t s) {
  if (npx)
    k_metric_map<<<blocks_for(npx, 256), 256, 0, s>>>(color, target, pixel_base, target_base, npx, l1);
}

void launch_metric_stats(const float* l1, uint32_t npx, float* pmin, float* pmax, double* psum,
                         uint32_t nblocks, MetricStats* out, cudaStream_t s) {
  k_metric_partials<<<nblocks, 256, 0, s>>>(l1, npx, pmin, pmax, psum);
  k_metric_final<<<1, 32, 0, s>>>(pmin, pmax, psum, nblocks, npx, out);
}

void launch_metric_accum(const DevBuffers& b, uint32_t view, uint32_t npx, const float* l1,
                         const MetricStats* st, float threshold, uint32_t* counts, cudaStream_t s) {
  if (npx) k_metric_accum<<<blocks_for(npx, 256), 256, 0, s>>>(b, view, l1, st, threshold, counts);
}

void launch_metric_combine(uint32_t* counts, uint32_t n, const MetricStats* st,
                           uint32_t* importance, float* pruning, cudaStream_t s) {
  if (n) k_metric_combine<<<blocks_for(n, 256), 256, 0, s>>>(counts, n, st, importance, pruning);
}

void launch_densify_decide(const float* P, uint32_t stride, uint32_t n, const float4* accum,
                           const uint32_t* importance, const DensifyRule& rule, uint32_t* action,
                           uint32_t* key_lo, uint32_t* key_hi, uint32_t* ncand, cudaStream_t s) {
  if (n)
    k_densify_decide<<<blocks_for(n, 256), 256, 0, s>>>(P, stride, n, accum, importance, rule,
                                                        action, key_lo, key_hi, ncand);
}

void launch_gather_u32(const uint32_t* src, const uint32_t* idx, uint32_t n, uint32_t* dst,
                       cudaStream_t s) {
  if (n) k_gather_u32<<<blocks_for(n, 256), 256, 0, s>>>(src, idx, n, dst);
}

void launch_densify_select(const uint32_t* order, uint32_t n, uint32_t allowed,
                           const uint32_t* action, uint32_t* keep, uint32_t* newc, cudaStream_t s) {
  if (n) k_densify_select<<<blocks_for(n, 256), 256, 0, s>>>(order, n, allowed, action, keep, newc);
}

void launch_densify_build(const float* P, const float* M1, const float* M2, uint32_t stride,
                          uint32_t n, const uint32_t* keep_scan, const uint32_t* new_scan,
                          uint32_t survivors, float* NP, float* NM1, float* NM2, uint32_t nstride,
                          uint64_t seed, uint64_t iteration, cudaStream_t s) {
  if (n)
    k_densify_build<<<blocks_for(n, 128), 128, 0, s>>>(P, M1, M2, stride, n, keep_scan, new_scan,
                                                       survivors, NP, NM1, NM2, nstride, seed,
                                                       iteration);
}

void launch_prune_normalise(const float* scores, uint32_t base, uint32_t n, float* norm,
                            float* pmin, float* pmax, uint32_t nblocks, cudaStream_t s) {
  if (!n) return;
  k_score_partials<<<nblocks, 256, 0, s>>>(scores, base, pmin, pmax);
  k_score_normalise<<<blocks_for(n, 256), 256, 0, s>>>(scores, base, n, pmin, pmax, nblocks, norm);
}

void launch_prune_weights(const float* P, uint32_t stride, uint32_t n, const float* norm,
                          const float4* importance, const PruneRule& rule, uint32_t* key_lo,
                          uint32_t* key_hi, uint32_t* nprunable, uint64_t seed, uint64_t iteration,
                          cudaStream_t s) {
  if (n)
    k_prune_weights<<<blocks_for(n, 256), 256, 0, s>>>(P, stride, n, norm, importance, rule, key_lo,
                                                       key_hi, nprunable, seed, iteration);
}

void launch_prune_select(const uint32_t* order, uint32_t n, uint32_t budget, uint32_t* keep,
                         cudaStream_t s) {
  if (n) k_prune_select<<<blocks_for(n, 256), 256, 0, s>>>(order, n, budget, keep);
}

}  // namespace sky
