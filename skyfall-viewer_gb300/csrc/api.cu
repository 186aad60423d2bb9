// Host runtime and C-ABI of the skyfall library (include/skyfall.h).
//
// A context owns every device buffer of one scene: the 59 f32 parameter
// planes with their Adam moments, the cameras' target images, and the step
// buffers (projection records, intersection keys, tile ranges, images,
// per-intersection partial gradients).  sky_step runs, on one CUDA stream:
//   preprocess -> scan -> emit keys -> onesweep sort (per group of views) ->
//   tile ranges -> forward (+loss) -> backward -> geometry adjoint + Adam
// and, when the context was created with use_graph, replays that sequence as
// one captured CUDA graph.
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "densify.cuh"
#include "kernels.cuh"
#include "knn.cuh"
#include "plyio.cuh"
#include "skyfall.h"
#include "viewer.cuh"

using namespace sky;

namespace {

thread_local std::string g_err;

int fail(int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_err = buf;
  return code;
}

#define CK(x)                                                                        \
  do {                                                                               \
    cudaError_t e_ = (x);                                                            \
    if (e_ != cudaSuccess)                                                           \
      return fail(e_ == cudaErrorMemoryAllocation ? SKY_ERR_OOM : SKY_ERR_CUDA,       \
                  "%s failed: %s", #x, cudaGetErrorString(e_));                      \
  } while (0)

#define TRY(x)                 \
  do {                         \
    int r_ = (x);              \
    if (r_ != SKY_OK) return r_; \
  } while (0)

// Host-side fault injection for tests of the error paths: SKY_FAULT=alloc:N
// makes the N-th device allocation (1-based, process wide) fail with
// SKY_ERR_INJECTED; SKY_FAULT=launch:N makes the N-th pass (step, forward,
// backward or render) fail before it launches anything; SKY_FAULT=lookback:N
// makes the N-th radix sort of a pass (item or intersection sort) or of
// sky_sort_pairs run its bounded look-back waits out (tile 0 withholds its
// word, 64 polls; see sort.cu), so that the call reports SKY_ERR_TIMEOUT.
// Read once, when the first counted event happens.
struct FaultPlan {
  long alloc_at = -1, launch_at = -1, lookback_at = -1;
  long allocs = 0, launches = 0, sorts = 0;
  FaultPlan() {
    const char* f = getenv("SKY_FAULT");
    if (!f) return;
    if (!strncmp(f, "alloc:", 6)) alloc_at = atol(f + 6);
    if (!strncmp(f, "launch:", 7)) launch_at = atol(f + 7);
    if (!strncmp(f, "lookback:", 9)) lookback_at = atol(f + 9);
  }
};
std::mutex g_fault_mu;
FaultPlan& faults() {
  static FaultPlan p;
  return p;
}
bool inject_alloc() {
  std::lock_guard<std::mutex> l(g_fault_mu);
  FaultPlan& p = faults();
  return p.alloc_at > 0 && ++p.allocs == p.alloc_at;
}
bool inject_launch() {
  std::lock_guard<std::mutex> l(g_fault_mu);
  FaultPlan& p = faults();
  return p.launch_at > 0 && ++p.launches == p.launch_at;
}

}  // namespace

bool sky::fault_lookback_next(cudaStream_t stream) {
  std::lock_guard<std::mutex> l(g_fault_mu);
  FaultPlan& p = faults();
  if (p.lookback_at <= 0) return false;
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(stream, &cap) != cudaSuccess || cap != cudaStreamCaptureStatusNone)
    return false;
  return ++p.sorts == p.lookback_at;
}

namespace {

uint64_t splitmix64(uint64_t& s) {
  uint64_t z = (s += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

// Decimal literal the reference's JavaScript uses for an f32 hyperparameter
// (0.9f -> 0.9): round the f32 value to 7 significant digits in double.
double js_literal(float f) {
  if (f == 0.0f) return 0.0;
  char buf[64];
  snprintf(buf, sizeof(buf), "%.7g", (double)f);
  return strtod(buf, nullptr);
}

enum Mode { kRender = 0, kForward = 1, kBackward = 2, kTrain = 3 };

struct Buf {
  void* p = nullptr;
  size_t bytes = 0;
};

// Launch geometry of one pass.  Direct passes size the grids for the step;
// a captured graph sizes them for the largest step it may replay (kernels
// read the actual counts from the step parameters and exit early).
struct Shape {
  uint32_t nv = 0, n = 0, stride = 0, mode = 0, icap = 0;
  uint32_t max_tiles = 0, max_view_px = 0, ngroups = 0;
  uint32_t key_bits[kMaxGroups] = {};
  uint32_t fwd_batch = 0, bwd_batch = 0;  // splat-batch depths (kernel variants)
  bool with_loss = false, ssim = false, ref = false, prof = false;
  bool count = false;  // pair-counting raster variants (profiling level 2)
  bool same(const Shape& o) const { return memcmp(this, &o, sizeof(Shape)) == 0; }
};

struct Context {
  SkyConfig cfg{};
  int device = 0;
  cudaStream_t stream = nullptr;
  uint32_t n = 0, stride = 0;
  Buf params, m1, m2, grads, tmp_planes;
  Buf records, aux, counts, rects, rowspans, cumsum, block_sums;
  // item order (view, depth16, Gaussian): sort keys, sorted keys, permutation
  Buf ikeys, ikeys_sorted, perm, item_end, isort_mem;
  SortScratch isort{};
  Buf keys, keys_sorted, vals_sorted, rec_of, flatten, fmask, partials, reached, tile_grads, gsum54;
  Buf offsets, loss_partials, color, alpha, tfinal, last, residual, targets, sort_mem;
  Buf flags, flag_scan, d_sp, d_st;
  // densification statistics (float4 per Gaussian) and multi-view scores
  Buf imp_stats, dens_accum, score_imp, score_prune, score_counts, metric_l1, metric_part,
      metric_stats, item_sums;
  bool scores_valid = false;  // scores belong to (scores_iter, current scene)
  uint64_t scores_iter = 0;
  uint32_t scores_n = 0, scores_views = 0;
  float scene_extent = 1.0f;
  SkySchedule sched{};
  uint32_t densify_runs = 0, prune_runs = 0;
  // headless viewer frame
  Buf v_splats, v_keys, v_counts, v_rects, v_order, v_ksorted, v_cum, v_csorted, v_bsums, v_misc,
      v_tkeys, v_gidx, v_tkeys_s, v_gidx_s, v_offsets, v_rgba, v_sort;
  uint32_t view_w = 0, view_h = 0;
  SortScratch sort{};
  uint32_t icap = 0;
  std::vector<SkyCamera> cams;
  std::vector<uint64_t> tgt_base;
  std::vector<uint8_t> tgt_set;
  uint64_t targets_px = 0;
  StepParams* h_sp = nullptr;
  DevStatus* h_st = nullptr;
  uint64_t iteration = 0, adam_steps = 0, last_isect = 0;
  uint64_t adam_views = 0;  // views summed over the Adam steps taken
  double last_loss = 0.0;
  uint64_t rng = 0;
  size_t device_bytes = 0;
  // shape of the last step (for readback and sky_backward)
  std::vector<uint32_t> last_views;
  uint32_t last_items = 0, last_tiles = 0, last_pixels = 0, last_groups = 0;
  bool fwd_ready = false;
  uint32_t error_flags = 0;
  uint64_t launches = 0;
  // per-stage profiling (CUDA events on the context's stream); level 2 also
  // runs the pair-counting raster variants
  bool profiling = false;
  bool count_pairs = false;
  // host <-> device bytes copied by the passes (step parameters in, status
  // out), cumulative; a captured graph's copies are counted per replay
  uint64_t step_h2d = 0, step_d2h = 0, graph_h2d = 0, graph_d2h = 0;
  cudaEvent_t ev[SKY_NUM_STAGES + 1] = {};
  double stage_ms[SKY_NUM_STAGES] = {};
  uint64_t prof_steps = 0;
  // captured training step (use_graph)
  cudaGraphExec_t gexec = nullptr;
  Shape gshape;
  bool gvalid = false;
  uint64_t graph_launches = 0, graph_captures = 0, graph_replays = 0, warm_steps = 0;
};

int dev_alloc(Context* c, Buf& b, size_t bytes, bool keep = false) {
  if (bytes <= b.bytes && b.p) return SKY_OK;
  if (inject_alloc()) return fail(SKY_ERR_INJECTED, "injected allocation failure");
  size_t want = bytes + bytes / 4 + 256;
  void* p = nullptr;
  cudaError_t e = cudaMalloc(&p, want);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return fail(SKY_ERR_OOM, "cudaMalloc(%zu) failed: %s", want, cudaGetErrorString(e));
  }
  if (keep && b.p && b.bytes) {
    CK(cudaMemcpyAsync(p, b.p, b.bytes, cudaMemcpyDeviceToDevice, c->stream));
    CK(cudaStreamSynchronize(c->stream));
  }
  if (b.p) {
    cudaFree(b.p);
    c->device_bytes -= b.bytes;
  }
  c->gvalid = false;  // a captured graph holds the old pointer
  b.p = p;
  b.bytes = want;
  c->device_bytes += want;
  return SKY_OK;
}

void dev_free(Context* c, Buf& b) {
  if (b.p) {
    cudaFree(b.p);
    c->gvalid = false;
  }
  c->device_bytes -= b.bytes;
  b.p = nullptr;
  b.bytes = 0;
}

// Zeroed densify accumulators and importance statistics for `stride`
// Gaussians (resetAccumulators / resetStats after a load, densify or prune).
int reset_stats(Context* c) {
  const size_t bytes = (size_t)c->stride * 16;
  TRY(dev_alloc(c, c->imp_stats, bytes));
  TRY(dev_alloc(c, c->dens_accum, bytes));
  CK(cudaMemsetAsync(c->imp_stats.p, 0, bytes, c->stream));
  CK(cudaMemsetAsync(c->dens_accum.p, 0, bytes, c->stream));
  return SKY_OK;
}

DevBuffers make_buffers(Context* c) {
  DevBuffers b{};
  b.params = (float*)c->params.p;
  b.m1 = (float*)c->m1.p;
  b.m2 = (float*)c->m2.p;
  b.grads = (float*)c->grads.p;
  b.records = (float4*)c->records.p;
  b.aux = (float2*)c->aux.p;
  b.counts = (uint32_t*)c->counts.p;
  b.rects = (uint2*)c->rects.p;
  b.rowspans = (uint4*)c->rowspans.p;
  b.ikeys = (uint32_t*)c->ikeys.p;
  b.perm = (uint32_t*)c->perm.p;
  b.ikeys_sorted = (uint32_t*)c->ikeys_sorted.p;
  b.item_end = (uint32_t*)c->item_end.p;
  b.cumsum = (uint32_t*)c->cumsum.p;
  b.block_sums = (uint32_t*)c->block_sums.p;
  b.keys = (uint32_t*)c->keys.p;
  b.keys_sorted = (uint32_t*)c->keys_sorted.p;
  b.vals_sorted = (uint32_t*)c->vals_sorted.p;
  b.rec_of = (uint32_t*)c->rec_of.p;
  b.flatten = (uint32_t*)c->flatten.p;
  b.fmask = (uint8_t*)c->fmask.p;
  b.reached = (uint8_t*)c->reached.p;
  b.partials = (float4*)c->partials.p;
  b.item_sums = (float4*)c->item_sums.p;
  b.tile_grads = (int32_t*)c->tile_grads.p;
  b.gsum54 = (long long*)c->gsum54.p;
  b.offsets = (uint32_t*)c->offsets.p;
  b.loss_partials = (double*)c->loss_partials.p;
  b.color = (float4*)c->color.p;
  b.alpha = (float*)c->alpha.p;
  b.tfinal = (float*)c->tfinal.p;
  b.last = (uint32_t*)c->last.p;
  b.residual = (float4*)c->residual.p;
  b.targets = (const float4*)c->targets.p;
  b.importance = (float*)c->imp_stats.p;
  b.densify_accum = (float*)c->dens_accum.p;
  b.sp = (const StepParams*)c->d_sp.p;
  b.status = (DevStatus*)c->d_st.p;
  return b;
}

uint32_t ceil_log2(uint32_t x) {
  uint32_t b = 0;
  while ((1ull << b) < (uint64_t)x) ++b;
  return b;
}

int ensure_isect(Context* c, uint32_t need) {
  if (need <= c->icap && c->keys.p) return SKY_OK;
  uint64_t cap = (uint64_t)need + need / 2 + 4096;
  if (cap > (1u << 30)) cap = 1u << 30;
  if (need > cap) return fail(SKY_ERR_CAPACITY, "%u intersections exceed the 2^30 limit", need);
  const bool ref = c->cfg.backward_mode == SKY_BWD_REFERENCE;
  TRY(dev_alloc(c, c->keys, cap * 4));
  TRY(dev_alloc(c, c->keys_sorted, cap * 4));
  TRY(dev_alloc(c, c->vals_sorted, cap * 4));
  TRY(dev_alloc(c, c->rec_of, cap * 4));
  TRY(dev_alloc(c, c->flatten, cap * 4));
  TRY(dev_alloc(c, c->fmask, cap));
  TRY(dev_alloc(c, c->partials, cap * kPartialF4 * 16));
  TRY(dev_alloc(c, c->reached, cap));
  CK(cudaMemsetAsync(c->reached.p, 0, c->reached.bytes, c->stream));
  if (ref) TRY(dev_alloc(c, c->tile_grads, cap * 54 * 4));
  TRY(dev_alloc(c, c->sort_mem, sort_scratch_bytes((uint32_t)cap)));
  c->sort = sort_scratch_carve(c->sort_mem.p, (uint32_t)cap);
  c->icap = (uint32_t)cap;
  return SKY_OK;
}

double position_lr(const SkyConfig& cfg, uint64_t iteration) {
  // computePositionLearningRate (gaussian-renderer.ts:284-298)
  const double lr0 = js_literal(cfg.lr_means), lr1 = js_literal(cfg.lr_means_final);
  if (lr0 <= 0 || lr1 <= 0) return lr0;
  const double step = (double)iteration;
  const double max_steps = std::max(1.0, (double)cfg.lr_means_max_steps);
  const double t = std::min(1.0, step / max_steps);
  const double log_lerp = std::exp(std::log(lr0) * (1 - t) + std::log(lr1) * t);
  double delay = 1.0;
  const double dm = js_literal(cfg.lr_means_delay_mult);
  if (dm < 0.999) {
    const double phase = std::min(1.0, step / std::max(1.0, std::round(0.1 * max_steps)));
    delay = dm + (1.0 - dm) * std::sin(0.5 * M_PI * phase);
  }
  return log_lerp * delay;
}

// Enqueues the pass on the context's stream.  With sizing_sync (direct
// passes only) the intersection count is read back after the scan and the
// buffers grown before emission, as the reference does with its host cumsum.
int enqueue(Context* c, const Shape& sh, bool sizing_sync, uint64_t& launches, uint64_t& h2d,
            uint64_t& d2h) {
  cudaStream_t s = c->stream;
  DevBuffers b = make_buffers(c);
  const bool prof = sh.prof;
  const bool capturing = !sizing_sync;
  auto mark = [&](int k) -> int {
    if (prof) CK(capturing ? cudaEventRecordWithFlags(c->ev[k], s, cudaEventRecordExternal)
                           : cudaEventRecord(c->ev[k], s));
    return SKY_OK;
  };
  const uint64_t items = (uint64_t)sh.nv * sh.n;
  launches = 0;
  h2d = sizeof(StepParams);
  d2h = 0;
  CK(cudaMemcpyAsync(c->d_sp.p, c->h_sp, sizeof(StepParams), cudaMemcpyHostToDevice, s));
  CK(cudaMemsetAsync(c->d_st.p, 0, sizeof(DevStatus), s));
  DevStatus* dst = (DevStatus*)c->d_st.p;
  TRY(mark(0));
  launch_preprocess(b, sh.n, sh.nv, s);
  TRY(mark(1));
  // Emission order of the items: per sort group (its items are contiguous),
  // a stable sort by depth16.  Emitting in this order lets the intersection
  // sort skip the two depth digits.
  {
    const StepParams* d_sp = (const StepParams*)c->d_sp.p;
    for (uint32_t g = 0; g < sh.ngroups; ++g) {
      // bounds = {item_begin, item_end} of the group, in device memory
      SortSegment seg{&d_sp->groups[g].item_begin, 0};
      CK(sort_pairs_launch(b.ikeys, nullptr, (uint32_t*)c->ikeys_sorted.p, b.perm, seg,
                           (uint32_t)items, 16, c->isort, &dst->error, s, 0, true));
      launches += 4;
    }
  }
  launch_scan(b, (uint32_t)items, s);
  launch_group_bounds(b, s);
  launches += 5;
  if (sizing_sync) {
    d2h += sizeof(DevStatus);
    CK(cudaMemcpyAsync(c->h_st, c->d_st.p, sizeof(DevStatus), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    // (the capacity bit is the group-bounds kernel's request to grow; after
    // a sort that gave up the later kernels of the step do nothing and the
    // count is not to be trusted: no growth)
    const uint32_t fatal = c->h_st->error & ~SKY_DEVERR_CAPACITY;
    if (fatal == 0u && c->h_st->total_isect > c->icap) {
      TRY(ensure_isect(c, c->h_st->total_isect));
      b = make_buffers(c);
      c->h_sp->icap = c->icap;
      h2d += sizeof(StepParams);
      CK(cudaMemcpyAsync(c->d_sp.p, c->h_sp, sizeof(StepParams), cudaMemcpyHostToDevice, s));
      CK(cudaMemsetAsync(c->d_st.p, 0, sizeof(DevStatus), s));
      launch_group_bounds(b, s);
      ++launches;
    }
  }
  TRY(mark(2));
  launch_emit(b, sh.n, sh.nv, s);
  TRY(mark(3));
  for (uint32_t g = 0; g < sh.ngroups; ++g) {
    // keys were emitted in depth order within each tile's items: sorting on
    // the tile field (digits 2 and 3) alone gives the full key order
    SortSegment seg{&dst->group_bounds[g][0], 0};
    CK(sort_pairs_launch(b.keys, nullptr, b.keys_sorted, b.vals_sorted, seg, c->icap, sh.key_bits[g],
                         c->sort, &dst->error, s, 2, true));
    launches += 2 + (sh.key_bits[g] + 7) / 8 - 2;
  }
  TRY(mark(4));
  launch_ranges(b, c->icap, s);
  TRY(mark(5));
  launch_forward(b, sh.max_tiles, c->cfg.tile_size, sh.fwd_batch, sh.ssim, sh.nv, sh.max_view_px,
                 sh.count, s);
  if (sh.with_loss) launch_loss_final(b, s);
  launches += 4 + (sh.with_loss ? 1 : 0) + (sh.ssim ? 1 : 0);
  TRY(mark(6));
  if (sh.mode >= kBackward) {
    if (sh.ref) CK(cudaMemsetAsync(c->gsum54.p, 0, items * 54 * 8, s));
    else CK(cudaMemsetAsync(c->reached.p, 0, c->icap, s));  // the partials this step writes
    launch_backward(b, sh.max_tiles, c->cfg.tile_size, sh.bwd_batch, sh.ref, sh.count, s);
    TRY(mark(7));
    if (!sh.ref) {
      launch_item_sums(b, items, s);
      ++launches;
    }
    launch_geom_adam(b, sh.n, s);
    launches += 2;
  } else {
    TRY(mark(7));
  }
  TRY(mark(8));
  CK(cudaGetLastError());
  d2h += sizeof(DevStatus);
  CK(cudaMemcpyAsync(c->h_st, c->d_st.p, sizeof(DevStatus), cudaMemcpyDeviceToHost, s));
  return SKY_OK;
}

void drop_graph(Context* c) {
  if (c->gexec) cudaGraphExecDestroy(c->gexec);
  c->gexec = nullptr;
  c->gvalid = false;
}

// Runs one pass over `nv` cameras.  mode: render / forward (+loss) /
// backward (gradients out, no Adam) / train (Adam step).
int run_views(Context* c, const uint32_t* cams, uint32_t nv, Mode mode, SkyStepStats* stats) {
  if (c->n == 0) return fail(SKY_ERR_STATE, "no Gaussians loaded");
  if (nv == 0 || nv > (uint32_t)kMaxViews)
    return fail(SKY_ERR_ARG, "camera count %u outside [1, %d]", nv, kMaxViews);
  if (inject_launch()) return fail(SKY_ERR_INJECTED, "injected launch failure");
  const SkyConfig& cfg = c->cfg;
  const uint32_t ts = cfg.tile_size;
  const bool with_loss = mode != kRender;
  // Training steps replay a captured graph once the intersection capacity is
  // known (the first step runs directly and sizes it).
  const bool graph = cfg.use_graph && mode == kTrain && c->icap > 0 && c->warm_steps > 0;
  StepParams& sp = *c->h_sp;
  memset(&sp, 0, sizeof(StepParams));
  uint32_t max_cam_tiles = 0, max_cam_px = 0;
  for (const SkyCamera& cam : c->cams) {
    const uint64_t vt = (uint64_t)((cam.width + ts - 1) / ts) * ((cam.height + ts - 1) / ts);
    if (vt > 65536)
      return fail(SKY_ERR_ARG, "a camera has %llu tiles; at most 65536 per view", (unsigned long long)vt);
    max_cam_tiles = std::max(max_cam_tiles, (uint32_t)vt);
    max_cam_px = std::max(max_cam_px, cam.width * cam.height);
  }
  // graph mode: fixed slot -> sort group assignment
  const uint32_t slots_per_group = std::max<uint32_t>(1, 65536 / std::max<uint32_t>(1, max_cam_tiles));
  // views, tiles, pixels, groups
  uint64_t tile_total = 0, pix_total = 0;
  uint32_t max_view_px = 0;
  uint32_t ngroups = 0;
  uint64_t group_tiles = 0;
  for (uint32_t v = 0; v < nv; ++v) {
    const uint32_t ci = cams[v];
    if (ci >= c->cams.size()) return fail(SKY_ERR_ARG, "camera %u not set", ci);
    if (with_loss && !c->tgt_set[ci]) return fail(SKY_ERR_STATE, "camera %u has no target", ci);
    const SkyCamera& cam = c->cams[ci];
    ViewInfo& vi = sp.views[v];
    memcpy(vi.view, cam.view, sizeof(vi.view));
    memcpy(vi.proj, cam.proj, sizeof(vi.proj));
    vi.focal[0] = cam.focal[0];
    vi.focal[1] = cam.focal[1];
    vi.width = cam.width;
    vi.height = cam.height;
    vi.tiles_x = (cam.width + ts - 1) / ts;
    vi.tiles_y = (cam.height + ts - 1) / ts;
    const uint64_t vt = (uint64_t)vi.tiles_x * vi.tiles_y;
    const bool new_group = graph ? (v % slots_per_group == 0) : (ngroups == 0 || group_tiles + vt > 65536);
    if (new_group) {
      if (ngroups == (uint32_t)kMaxGroups) return fail(SKY_ERR_ARG, "too many sort groups");
      GroupInfo& g = sp.groups[ngroups];
      g.tile_begin = (uint32_t)tile_total;
      g.item_begin = v * c->n;
      ++ngroups;
      group_tiles = 0;
    }
    GroupInfo& g = sp.groups[ngroups - 1];
    vi.group = ngroups - 1;
    vi.key_tile_base = (uint32_t)group_tiles;
    vi.tile_base = (uint32_t)tile_total;
    vi.pixel_base = (uint32_t)pix_total;
    vi.target_base = c->tgt_set[ci] ? (uint32_t)c->tgt_base[ci] : 0u;
    vi.has_target = c->tgt_set[ci];
    vi.camera = ci;
    group_tiles += vt;
    tile_total += vt;
    pix_total += (uint64_t)cam.width * cam.height;
    g.tile_end = (uint32_t)tile_total;
    g.item_end = (v + 1) * c->n;
    g.key_bits = 16 + ceil_log2(graph ? slots_per_group * max_cam_tiles : (uint32_t)group_tiles);
    max_view_px = std::max(max_view_px, cam.width * cam.height);
  }
  const uint64_t pix_cap = graph ? (uint64_t)nv * max_cam_px : pix_total;
  const uint64_t tile_cap = graph ? (uint64_t)nv * max_cam_tiles : tile_total;
  if (pix_cap >= (1ull << 32)) return fail(SKY_ERR_ARG, "too many pixels in one step");
  const uint64_t items = (uint64_t)nv * c->n;
  if (items >= (1ull << 32)) return fail(SKY_ERR_ARG, "views x Gaussians exceeds 2^32");
  // buffers
  TRY(dev_alloc(c, c->records, items * 48));
  TRY(dev_alloc(c, c->aux, items * 8));
  TRY(dev_alloc(c, c->counts, items * 4));
  TRY(dev_alloc(c, c->rects, items * 8));
  TRY(dev_alloc(c, c->rowspans, items * 16));
  TRY(dev_alloc(c, c->cumsum, items * 4));
  TRY(dev_alloc(c, c->ikeys, items * 4));
  TRY(dev_alloc(c, c->ikeys_sorted, items * 4));
  TRY(dev_alloc(c, c->perm, items * 4));
  TRY(dev_alloc(c, c->item_end, items * 4));
  TRY(dev_alloc(c, c->isort_mem, sort_scratch_bytes((uint32_t)items)));
  c->isort = sort_scratch_carve(c->isort_mem.p, (uint32_t)items);
  TRY(dev_alloc(c, c->block_sums, (scan_block_count((uint32_t)items) + 1) * 4));
  TRY(dev_alloc(c, c->offsets, (tile_cap + 1) * 4));
  TRY(dev_alloc(c, c->loss_partials, (tile_cap + 1) * 8));
  TRY(dev_alloc(c, c->color, pix_cap * 16));
  TRY(dev_alloc(c, c->alpha, pix_cap * 4));
  TRY(dev_alloc(c, c->tfinal, pix_cap * 4));
  TRY(dev_alloc(c, c->last, pix_cap * 4));
  TRY(dev_alloc(c, c->residual, pix_cap * 16));
  if (mode == kBackward) TRY(dev_alloc(c, c->grads, (size_t)kPlanes * c->stride * 4));
  const bool ref = cfg.backward_mode == SKY_BWD_REFERENCE;
  if (ref && mode >= kBackward) TRY(dev_alloc(c, c->gsum54, items * 54 * 8));
  if (!ref && mode >= kBackward) TRY(dev_alloc(c, c->item_sums, items * 48));
  if (c->icap == 0) TRY(ensure_isect(c, 1u << 16));
  // schedules
  uint64_t it = c->iteration + (mode == kTrain ? 1 : 0);
  uint32_t deg = cfg.sh_degree;
  if (cfg.sh_degree_interval > 0)
    deg = (uint32_t)std::min<uint64_t>(cfg.sh_degree, it / cfg.sh_degree_interval);
  sp.num_views = nv;
  sp.n = c->n;
  sp.num_tiles = (uint32_t)tile_total;
  sp.num_groups = ngroups;
  sp.sh_deg = deg;
  sp.sh_update = (mode == kTrain && cfg.sh_update_interval > 0 && it % cfg.sh_update_interval == 0) ? 1 : 0;
  sp.bwd_mode = cfg.backward_mode;
  sp.round_f16 = cfg.round_params_f16;
  sp.tile_size = ts;
  sp.has_loss = with_loss ? 1 : 0;
  sp.apply_adam = mode == kTrain ? 1 : 0;
  sp.write_grads = mode == kBackward ? 1 : 0;
  sp.icap = c->icap;
  sp.num_pixels = (uint32_t)pix_total;
  sp.plane_stride = c->stride;
  // renders and forward passes keep the reference's lists (the multi-view
  // scores walk a render's lists), and so does the reference-mode backward:
  // its batches of 64 list entries set where each pixel's walk restarts, so
  // its sums depend on the list, not only on the contributing entries
  sp.tile_cull = (cfg.tile_cull && mode >= kBackward && !ref) ? 1u : 0u;
  sp.near_plane = cfg.near_plane;
  sp.far_plane = cfg.far_plane;
  sp.radius_clip = cfg.radius_clip;
  sp.eps2d = cfg.eps2d;
  for (int k = 0; k < 3; ++k) sp.bg[k] = cfg.background[k];
  sp.w_l2 = cfg.w_l2;
  sp.w_l1 = cfg.w_l1;
  sp.w_ssim = cfg.w_ssim;
  sp.lr_pos = (float)position_lr(cfg, it);
  sp.lr_scale = cfg.lr_scale;
  sp.lr_rot = cfg.lr_rotation;
  sp.lr_opacity = cfg.lr_opacity;
  sp.lr_sh = cfg.lr_sh;
  sp.beta1 = cfg.beta1;
  sp.beta2 = cfg.beta2;
  sp.adam_eps = cfg.adam_eps;
  sp.importance_decay = 0.98f;  // DEFAULT_IMPORTANCE_CONFIG.decay (importance.ts:9)
  {
    // run_adam_on_buffer (gaussian-renderer.ts:2420-2430): t = max(1, counter)
    double t = (double)std::max<uint64_t>(1, c->adam_steps);
    if (cfg.batch_scaling && nv > 1) {
      // a step of B views: learning rates x sqrt(B), betas to the power B;
      // the bias correction's exponent counts views (max(B, views so far)
      // is t = max(1, counter) in view units, so B = 1 steps are unchanged)
      const double sq = std::sqrt((double)nv);
      sp.lr_pos = (float)(position_lr(cfg, it) * sq);
      sp.lr_scale = (float)(js_literal(cfg.lr_scale) * sq);
      sp.lr_rot = (float)(js_literal(cfg.lr_rotation) * sq);
      sp.lr_opacity = (float)(js_literal(cfg.lr_opacity) * sq);
      sp.lr_sh = (float)(js_literal(cfg.lr_sh) * sq);
      sp.beta1 = (float)std::pow(js_literal(cfg.beta1), (double)nv);
      sp.beta2 = (float)std::pow(js_literal(cfg.beta2), (double)nv);
    }
    if (cfg.batch_scaling) t = (double)std::max<uint64_t>(nv, c->adam_views);
    const double bc1 = 1.0 - std::pow(js_literal(cfg.beta1), t);
    const double bc2 = 1.0 - std::pow(js_literal(cfg.beta2), t);
    sp.bc1_rcp = (float)(1.0 / bc1);
    sp.bc2_sqrt_rcp = (float)(1.0 / std::sqrt(bc2));
  }
  Shape sh;
  sh.nv = nv;
  sh.n = c->n;
  sh.stride = c->stride;
  sh.mode = mode;
  sh.max_tiles = (uint32_t)tile_cap;
  sh.max_view_px = graph ? max_cam_px : max_view_px;
  sh.ngroups = ngroups;
  for (uint32_t g = 0; g < ngroups; ++g) sh.key_bits[g] = sp.groups[g].key_bits;
  sh.with_loss = with_loss;
  sh.ssim = with_loss && cfg.w_ssim > 0.0f;
  sh.ref = ref;
  sh.prof = c->profiling;
  sh.count = c->count_pairs;
  sh.fwd_batch = cfg.fwd_batch;
  sh.bwd_batch = cfg.bwd_batch;
  cudaStream_t s = c->stream;
  uint64_t launches = 0, h2d = 0, d2h = 0;
  for (int attempt = 0;; ++attempt) {
    sh.icap = c->icap;
    sp.icap = c->icap;
    if (!graph) {
      TRY(enqueue(c, sh, true, launches, h2d, d2h));
    } else {
      if (!c->gvalid || !c->gshape.same(sh)) {
        drop_graph(c);
        CK(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
        uint64_t l = 0, gi = 0, go = 0;
        int rc = enqueue(c, sh, false, l, gi, go);
        cudaGraph_t g = nullptr;
        cudaError_t e = cudaStreamEndCapture(s, &g);
        if (rc != SKY_OK) {
          if (g) cudaGraphDestroy(g);
          return rc;
        }
        if (e != cudaSuccess) return fail(SKY_ERR_CUDA, "graph capture: %s", cudaGetErrorString(e));
        e = cudaGraphInstantiate(&c->gexec, g, 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess) return fail(SKY_ERR_CUDA, "graph instantiate: %s", cudaGetErrorString(e));
        c->gshape = sh;
        c->gvalid = true;
        c->graph_launches = l;
        c->graph_h2d = gi;
        c->graph_d2h = go;
        c->graph_captures += 1;
      }
      CK(cudaGraphLaunch(c->gexec, s));
      launches = c->graph_launches;
      h2d = c->graph_h2d;
      d2h = c->graph_d2h;
      c->graph_replays += 1;
    }
    CK(cudaStreamSynchronize(s));
    c->launches += launches;
    c->step_h2d += h2d;
    c->step_d2h += d2h;
    if (graph && (c->h_st->error & SKY_DEVERR_CAPACITY) && attempt < 3) {
      // the failed replay changed no parameter: grow, re-capture, run again
      TRY(ensure_isect(c, c->h_st->total_isect));
      drop_graph(c);
      continue;
    }
    break;
  }
  if (sh.prof) {
    for (int k = 0; k < SKY_NUM_STAGES; ++k) {
      float ms = 0.0f;
      CK(cudaEventElapsedTime(&ms, c->ev[k], c->ev[k + 1]));
      c->stage_ms[k] += ms;
    }
    c->prof_steps += 1;
  }
  c->error_flags |= c->h_st->error;
  if (c->h_st->error & SKY_DEVERR_SORT_TIMEOUT)
    return fail(SKY_ERR_TIMEOUT, "radix sort look-back wait gave up");
  if (c->h_st->error & SKY_DEVERR_LISTS)
    return fail(SKY_ERR_STATE,
                "intersection lists inconsistent: key emission disagreed with the preprocess's "
                "tile counts, or the tile ranges met unsorted keys");
  if (c->h_st->error & SKY_DEVERR_CAPACITY)
    return fail(SKY_ERR_CAPACITY, "intersection capacity exceeded");
  c->last_views.assign(cams, cams + nv);
  c->last_items = (uint32_t)items;
  c->last_tiles = (uint32_t)tile_total;
  c->last_pixels = (uint32_t)pix_total;
  c->last_groups = ngroups;
  c->last_isect = c->h_st->total_isect;
  c->last_loss = c->h_st->loss;
  c->fwd_ready = with_loss;
  if (mode == kTrain) {
    c->iteration = it;
    c->adam_steps += 1;
    c->adam_views += nv;
    c->warm_steps += 1;
  }
  if (stats) {
    stats->iteration = c->iteration;
    stats->num_intersections = c->h_st->total_isect;
    stats->loss = c->h_st->loss;
    stats->num_gaussians = c->n;
    stats->num_views = nv;
    stats->sh_degree = deg;
    stats->sh_updated = sp.sh_update;
  }
  return SKY_OK;
}

Context* as_ctx(void* p) { return (Context*)p; }

// ---- densification, multi-view scores, scored prune ----------------------

// Device buffer released when it goes out of scope.
struct TempBuf {
  Context* c;
  Buf b;
  explicit TempBuf(Context* ctx) : c(ctx) {}
  ~TempBuf() {
    if (b.p) dev_free(c, b);
  }
  template <class T>
  T* as() const {
    return (T*)b.p;
  }
};

uint32_t stat_blocks(uint32_t n) {
  return std::max<uint32_t>(1, std::min<uint32_t>((n + 255) / 256, (uint32_t)sm_count() * 4));
}

// sampleCameraIndices (gaussian-renderer.ts:2677-2688) over the cameras that
// have a target: all of them in order when there are at most 10, else the
// first 10 of a Fisher-Yates shuffle driven by the context's generator.
std::vector<uint32_t> sample_cameras(Context* c) {
  std::vector<uint32_t> idx;
  for (uint32_t i = 0; i < (uint32_t)c->cams.size(); ++i)
    if (c->tgt_set[i]) idx.push_back(i);
  const size_t count = std::min<size_t>(10, idx.size());
  if (count >= idx.size()) return idx;
  for (size_t i = idx.size() - 1; i > 0; --i) {
    const double u = (splitmix64(c->rng) >> 11) * (1.0 / 9007199254740992.0);
    const size_t j = (size_t)(u * (double)(i + 1));
    std::swap(idx[i], idx[j]);
  }
  idx.resize(count);
  return idx;
}

// generateMultiViewScores (:2758-2788): render the views in batches, then
// per view in order: L1 map, its statistics, error-pixel hits per Gaussian.
int score_views(Context* c, const std::vector<uint32_t>& views) {
  const uint32_t n = c->n;
  for (uint32_t v : views) {
    if (v >= c->cams.size()) return fail(SKY_ERR_ARG, "camera %u not set", v);
    if (!c->tgt_set[v]) return fail(SKY_ERR_STATE, "camera %u has no target", v);
  }
  cudaStream_t s = c->stream;
  TRY(dev_alloc(c, c->score_imp, (size_t)n * 4));
  TRY(dev_alloc(c, c->score_prune, (size_t)n * 4));
  TRY(dev_alloc(c, c->score_counts, (size_t)n * 4));
  TRY(dev_alloc(c, c->metric_stats, (size_t)kMaxViews * sizeof(MetricStats)));
  CK(cudaMemsetAsync(c->score_imp.p, 0, (size_t)n * 4, s));
  CK(cudaMemsetAsync(c->score_prune.p, 0, (size_t)n * 4, s));
  CK(cudaMemsetAsync(c->score_counts.p, 0, (size_t)n * 4, s));
  MetricStats* st = (MetricStats*)c->metric_stats.p;
  for (size_t first = 0; first < views.size(); first += kMaxViews) {
    const uint32_t nb = (uint32_t)std::min<size_t>(kMaxViews, views.size() - first);
    TRY(run_views(c, views.data() + first, nb, kRender, nullptr));
    DevBuffers b = make_buffers(c);
    for (uint32_t v = 0; v < nb; ++v) {
      const ViewInfo& vi = c->h_sp->views[v];
      const uint32_t npx = vi.width * vi.height;
      const uint32_t blocks = stat_blocks(npx);
      TRY(dev_alloc(c, c->metric_l1, (size_t)npx * 4));
      // partials: blocks f32 minima, blocks f32 maxima, then blocks f64 sums
      // at byte offset 8 * blocks of the (256-byte aligned) allocation, so the
      // f64 array is 8-byte aligned for every block count
      TRY(dev_alloc(c, c->metric_part, (size_t)blocks * 16));
      float* pmin = (float*)c->metric_part.p;
      float* pmax = pmin + blocks;
      double* psum = (double*)(pmax + blocks);
      if ((reinterpret_cast<uintptr_t>(psum) & 7u) != 0u)
        return fail(SKY_ERR_STATE, "metric partials misaligned");
      launch_metric_map(b.color, b.targets, vi.pixel_base, vi.target_base, npx,
                        (float*)c->metric_l1.p, s);
      launch_metric_stats((const float*)c->metric_l1.p, npx, pmin, pmax, psum, blocks, st + v, s);
      launch_metric_accum(b, v, npx, (const float*)c->metric_l1.p, st + v, 0.1f,
                          (uint32_t*)c->score_counts.p, s);
      launch_metric_combine((uint32_t*)c->score_counts.p, n, st + v, (uint32_t*)c->score_imp.p,
                            (float*)c->score_prune.p, s);
      c->launches += 5;
    }
  }
  CK(cudaGetLastError());
  CK(cudaStreamSynchronize(s));
  c->scores_valid = true;
  c->scores_iter = c->iteration;
  c->scores_n = n;
  c->scores_views = (uint32_t)views.size();
  return SKY_OK;
}

// Scores of the current iteration and scene (getMultiViewScores cache),
// computed from a seeded camera sample when missing.  *have = false when no
// camera has a target (the reference skips densify and prune then).
int current_scores(Context* c, bool* have) {
  *have = true;
  if (c->scores_valid && c->scores_iter == c->iteration && c->scores_n == c->n) return SKY_OK;
  std::vector<uint32_t> views = sample_cameras(c);
  if (views.empty()) {
    *have = false;
    return SKY_OK;
  }
  return score_views(c, views);
}

// Stable ascending order of n 64-bit keys given as (lo, hi) halves: two LSD
// passes of 32-bit sorts.  order[k] = index of the k-th smallest key.
int sort_keys64(Context* c, const uint32_t* lo, const uint32_t* hi, uint32_t n, uint32_t* order) {
  cudaStream_t s = c->stream;
  TempBuf mem(c), kout(c), ord1(c), hperm(c), err(c);
  TRY(dev_alloc(c, mem.b, sort_scratch_bytes(n)));
  TRY(dev_alloc(c, kout.b, (size_t)n * 4));
  TRY(dev_alloc(c, ord1.b, (size_t)n * 4));
  TRY(dev_alloc(c, hperm.b, (size_t)n * 4));
  TRY(dev_alloc(c, err.b, 16));
  CK(cudaMemsetAsync(err.b.p, 0, 16, s));
  SortScratch sc = sort_scratch_carve(mem.b.p, n);
  SortSegment seg{nullptr, n};
  CK(sort_pairs_launch(lo, nullptr, kout.as<uint32_t>(), ord1.as<uint32_t>(), seg, n, 32, sc,
                       err.as<uint32_t>(), s));
  launch_gather_u32(hi, ord1.as<uint32_t>(), n, hperm.as<uint32_t>(), s);
  CK(sort_pairs_launch(hperm.as<uint32_t>(), ord1.as<uint32_t>(), kout.as<uint32_t>(), order, seg, n,
                       32, sc, err.as<uint32_t>(), s));
  uint32_t e = 0;
  CK(cudaMemcpyAsync(&e, err.b.p, 4, cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  c->launches += 11;
  if (e & SKY_DEVERR_SORT_TIMEOUT) return fail(SKY_ERR_TIMEOUT, "radix sort look-back wait gave up");
  return SKY_OK;
}

// Inclusive scan of n u32 flags into out (the hot path's scan kernels).
int scan_flags(Context* c, const uint32_t* flags, uint32_t* out, uint32_t n) {
  TempBuf bs(c);
  TRY(dev_alloc(c, bs.b, ((size_t)scan_block_count(n) + 1) * 4));
  DevBuffers sb{};
  sb.counts = (uint32_t*)flags;
  sb.cumsum = out;
  sb.block_sums = bs.as<uint32_t>();
  launch_scan(sb, n, c->stream);
  c->launches += 3;
  CK(cudaGetLastError());
  CK(cudaStreamSynchronize(c->stream));
  return SKY_OK;
}

// After a change of the scene: statistics reset, cached scores stale.
int scene_changed(Context* c, uint32_t n, uint32_t stride) {
  if (c->grads.p) dev_free(c, c->grads);
  c->n = n;
  c->stride = stride;
  c->fwd_ready = false;
  c->scores_valid = false;
  return reset_stats(c);
}

// Compacts params and moments to the survivors flagged 1 in keep
// (applyPruneMask :2917-3000).
int compact_survivors(Context* c, const uint32_t* keep, uint32_t keep_n) {
  const uint32_t n = c->n;
  cudaStream_t s = c->stream;
  TempBuf scan(c);
  TRY(dev_alloc(c, scan.b, (size_t)n * 4));
  TRY(scan_flags(c, keep, scan.as<uint32_t>(), n));
  const uint32_t new_stride = (keep_n + 255) & ~255u;
  const size_t bytes = (size_t)kPlanes * new_stride * 4;
  Buf* planes[3] = {&c->params, &c->m1, &c->m2};
  for (Buf* pl : planes) {
    Buf nb;
    TRY(dev_alloc(c, nb, bytes));
    launch_compact((const float*)pl->p, (float*)nb.p, c->stride, new_stride, kPlanes, n,
                   scan.as<uint32_t>(), s);
    ++c->launches;
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(s));
    dev_free(c, *pl);
    *pl = nb;
  }
  return scene_changed(c, keep_n, new_stride);
}

// performDensification (:3211-3433) on the device.
int densify(Context* c, const SkyDensifyParams& prm, uint32_t* cloned, uint32_t* split) {
  const uint32_t n = c->n;
  if (n == 0) return SKY_OK;
  if (n >= (1u << 30)) return fail(SKY_ERR_ARG, "densify supports fewer than 2^30 Gaussians");
  cudaStream_t s = c->stream;
  bool have = false;
  TRY(current_scores(c, &have));
  if (!have) {  // no multi-view scores: accumulators reset, nothing else
    CK(cudaMemsetAsync(c->dens_accum.p, 0, (size_t)c->stride * 16, s));
    CK(cudaStreamSynchronize(s));
    return SKY_OK;
  }
  double width = prm.pixel_width;
  if (!(width > 0.0)) {
    const uint32_t cam = c->last_views.empty() ? 0u : c->last_views[0];
    width = cam < c->cams.size() ? c->cams[cam].width : 1.0;
  }
  const double pixel_scale = std::max(width, 1.0) / 2.0;
  DensifyRule rule{};
  rule.grad_px = js_literal(prm.grad_threshold) * pixel_scale;
  rule.grad_abs_px = js_literal(prm.grad_abs_threshold) * pixel_scale;
  rule.size_threshold = prm.size_threshold > 0.0f ? (double)prm.size_threshold
                                                  : (double)c->scene_extent * 0.001;
  rule.min_visibility = std::max(1.0, (double)js_literal(prm.min_visibility));
  rule.importance_threshold = js_literal(prm.importance_threshold);
  rule.sample_count = (double)c->scores_views;
  TempBuf action(c), klo(c), khi(c), order(c), keep(c), newc(c), kscan(c), nscan(c), cnt(c);
  for (TempBuf* t : {&action, &klo, &khi, &order, &keep, &newc, &kscan, &nscan})
    TRY(dev_alloc(c, t->b, (size_t)n * 4));
  TRY(dev_alloc(c, cnt.b, 16));
  CK(cudaMemsetAsync(cnt.b.p, 0, 16, s));
  launch_densify_decide((const float*)c->params.p, c->stride, n, (const float4*)c->dens_accum.p,
                        (const uint32_t*)c->score_imp.p, rule, action.as<uint32_t>(),
                        klo.as<uint32_t>(), khi.as<uint32_t>(), cnt.as<uint32_t>(), s);
  ++c->launches;
  uint32_t ncand = 0;
  CK(cudaMemcpyAsync(&ncand, cnt.b.p, 4, cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  if (ncand == 0) {
    CK(cudaMemsetAsync(c->dens_accum.p, 0, (size_t)c->stride * 16, s));
    CK(cudaStreamSynchronize(s));
    return SKY_OK;
  }
  const uint64_t max_new = std::max<uint64_t>(1, (uint64_t)std::floor((double)n * js_literal(prm.max_new_ratio)));
  const uint32_t allowed = (uint32_t)std::min<uint64_t>(max_new, ncand);
  TRY(sort_keys64(c, klo.as<uint32_t>(), khi.as<uint32_t>(), n, order.as<uint32_t>()));
  launch_densify_select(order.as<uint32_t>(), n, allowed, action.as<uint32_t>(), keep.as<uint32_t>(),
                        newc.as<uint32_t>(), s);
  ++c->launches;
  TRY(scan_flags(c, keep.as<uint32_t>(), kscan.as<uint32_t>(), n));
  TRY(scan_flags(c, newc.as<uint32_t>(), nscan.as<uint32_t>(), n));
  uint32_t survivors = 0, added = 0;
  CK(cudaMemcpyAsync(&survivors, kscan.as<uint32_t>() + (n - 1), 4, cudaMemcpyDeviceToHost, s));
  CK(cudaMemcpyAsync(&added, nscan.as<uint32_t>() + (n - 1), 4, cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  const uint32_t splits = n - survivors, clones = added - 2 * splits;
  const uint64_t new_n = (uint64_t)survivors + added;
  if (new_n >= (1ull << 31)) return fail(SKY_ERR_CAPACITY, "densify would exceed 2^31 Gaussians");
  const uint32_t new_stride = ((uint32_t)new_n + 255) & ~255u;
  const size_t bytes = (size_t)kPlanes * new_stride * 4;
  Buf np, nm1, nm2;
  TRY(dev_alloc(c, np, bytes));
  int rc = dev_alloc(c, nm1, bytes);
  if (rc == SKY_OK) rc = dev_alloc(c, nm2, bytes);
  if (rc != SKY_OK) {
    dev_free(c, np);
    dev_free(c, nm1);
    return rc;
  }
  launch_densify_build((const float*)c->params.p, (const float*)c->m1.p, (const float*)c->m2.p,
                       c->stride, n, kscan.as<uint32_t>(), nscan.as<uint32_t>(), survivors,
                       (float*)np.p, (float*)nm1.p, (float*)nm2.p, new_stride, c->cfg.seed,
                       c->iteration, s);
  ++c->launches;
  CK(cudaGetLastError());
  CK(cudaStreamSynchronize(s));
  dev_free(c, c->params);
  dev_free(c, c->m1);
  dev_free(c, c->m2);
  c->params = np;
  c->m1 = nm1;
  c->m2 = nm2;
  TRY(scene_changed(c, (uint32_t)new_n, new_stride));
  c->densify_runs += 1;
  if (cloned) *cloned = clones;
  if (split) *split = splits;
  return SKY_OK;
}

// applyMultiViewPrune (:2800-2915) on the device.
int prune_scored(Context* c, const SkyScoredPruneParams& prm, uint32_t* removed) {
  const uint32_t n = c->n;
  if (n == 0) return SKY_OK;
  if (n >= (1u << 30)) return fail(SKY_ERR_ARG, "prune supports fewer than 2^30 Gaussians");
  cudaStream_t s = c->stream;
  const bool last_ok = prm.use_last_scores && c->scores_n > 0 && c->score_prune.p;
  if (!last_ok) {
    bool have = false;
    TRY(current_scores(c, &have));
    if (!have) return SKY_OK;
  }
  if (c->scores_views == 0) return SKY_OK;
  const uint32_t base = std::min(c->scores_n, n);
  PruneRule rule{};
  rule.min_opacity = js_literal(prm.min_opacity);
  rule.max_scale = js_literal(prm.max_scale);
  rule.max_screen_radius = js_literal(prm.max_screen_radius);
  rule.opacity_bonus = js_literal(prm.opacity_bonus);
  rule.scale_bonus = js_literal(prm.scale_bonus);
  rule.screen_bonus = js_literal(prm.screen_bonus);
  rule.use_screen = prm.use_screen_size && prm.max_screen_radius < 9999.0f ? 1u : 0u;
  const uint32_t blocks = stat_blocks(base);
  TempBuf norm(c), part(c), klo(c), khi(c), order(c), keep(c), cnt(c);
  for (TempBuf* t : {&norm, &klo, &khi, &order, &keep}) TRY(dev_alloc(c, t->b, (size_t)n * 4));
  TRY(dev_alloc(c, part.b, (size_t)blocks * 8));
  TRY(dev_alloc(c, cnt.b, 16));
  CK(cudaMemsetAsync(cnt.b.p, 0, 16, s));
  launch_prune_normalise((const float*)c->score_prune.p, base, n, norm.as<float>(), part.as<float>(),
                         part.as<float>() + blocks, blocks, s);
  launch_prune_weights((const float*)c->params.p, c->stride, n, norm.as<float>(),
                       (const float4*)c->imp_stats.p, rule, klo.as<uint32_t>(), khi.as<uint32_t>(),
                       cnt.as<uint32_t>(), c->cfg.seed, c->iteration, s);
  c->launches += 3;
  uint32_t to_remove = 0;
  CK(cudaMemcpyAsync(&to_remove, cnt.b.p, 4, cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  if (to_remove == 0) return SKY_OK;
  const uint64_t max_removals =
      std::max<uint64_t>(1, (uint64_t)std::floor((double)c->scores_n * js_literal(prm.max_ratio)));
  const uint64_t desired =
      std::max<uint64_t>(1, (uint64_t)std::floor((double)to_remove * js_literal(prm.prune_ratio)));
  const uint32_t budget = (uint32_t)std::min<uint64_t>(to_remove, std::min(desired, max_removals));
  if (budget >= n) return SKY_OK;  // applyPruneMask keeps at least one Gaussian
  TRY(sort_keys64(c, klo.as<uint32_t>(), khi.as<uint32_t>(), n, order.as<uint32_t>()));
  launch_prune_select(order.as<uint32_t>(), n, budget, keep.as<uint32_t>(), s);
  ++c->launches;
  TRY(compact_survivors(c, keep.as<uint32_t>(), n - budget));
  c->prune_runs += 1;
  if (removed) *removed = budget;
  return SKY_OK;
}

// TrainingController.getIterationActions (training-controller.ts:85-160) and
// the train loop's handling of it (gaussian-renderer.ts:3795-3829).
int run_schedule(Context* c) {
  const SkySchedule& sc = c->sched;
  const uint64_t it = c->iteration;
  const bool in_densify = it >= sc.densify_from && it <= sc.densify_until;
  const double extent = sc.scene_extent > 0.0f ? (double)sc.scene_extent : (double)c->scene_extent;
  SkyScoredPruneParams pp;
  sky_scored_prune_default(&pp);
  const bool screen = it > sc.opacity_reset_interval;
  pp.min_opacity = sc.min_opacity;
  pp.max_scale = sc.max_scale_absolute > 0.0f ? sc.max_scale_absolute
                 : sc.max_scale_ratio > 0.0f  ? (float)(extent * js_literal(sc.max_scale_ratio))
                                              : 1e6f;
  pp.use_screen_size = screen ? 1u : 0u;
  pp.max_screen_radius = screen ? sc.max_screen_size : 10000.0f;
  bool prune_attempted = false;
  if (in_densify && it % sc.densify_interval == 0) {
    bool have = false;
    TRY(current_scores(c, &have));
    if (have) {
      SkyDensifyParams dp = sc.densify;
      if (!(dp.size_threshold > 0.0f)) dp.size_threshold = (float)(extent * 0.001);
      TRY(densify(c, dp, nullptr, nullptr));
      pp.use_last_scores = 1;
      TRY(prune_scored(c, pp, nullptr));
      prune_attempted = true;
    }
  }
  if (!prune_attempted && it >= sc.prune_from && it <= sc.prune_until && it % sc.prune_interval == 0) {
    pp.use_last_scores = 0;
    TRY(prune_scored(c, pp, nullptr));
  }
  if (it != 0 && in_densify && it % sc.opacity_reset_interval == 0)
    TRY(sky_reset_opacity(c, sc.opacity_reset_value));
  return SKY_OK;
}

}  // namespace

// ===========================================================================
// C-ABI
// ===========================================================================
extern "C" {

int sky_version(void) { return 1; }

const char* sky_last_error(void) { return g_err.c_str(); }

void sky_config_default(SkyConfig* c) {
  if (!c) return;
  memset(c, 0, sizeof(*c));
  c->struct_size = sizeof(SkyConfig);
  c->tile_size = 16;
  c->sh_degree = 3;
  c->sh_degree_interval = 1000;
  c->near_plane = 0.2f;
  c->far_plane = 10000.0f;
  c->radius_clip = 512.0f;
  c->eps2d = 0.3f;
  c->w_l2 = 0.0f;
  c->w_l1 = 0.8f;
  c->w_ssim = 0.2f;
  c->lr_means = 0.00016f;
  c->lr_means_final = 0.0000016f;
  c->lr_means_delay_mult = 0.01f;
  c->lr_means_max_steps = 30000;
  c->lr_sh = 0.0025f;
  c->lr_opacity = 0.025f;
  c->lr_scale = 0.005f;
  c->lr_rotation = 0.001f;
  c->beta1 = 0.9f;
  c->beta2 = 0.999f;
  c->adam_eps = 1e-8f;
  c->sh_update_interval = 16;
  c->round_params_f16 = 1;
  c->backward_mode = SKY_BWD_EXACT;
  c->use_graph = 0;
  c->max_views_per_step = 16;
  c->seed = 0x5EEDull;
}

static int check_cfg(const SkyConfig* cfg) {
  if (!cfg) return fail(SKY_ERR_ARG, "null config");
  if (cfg->struct_size != sizeof(SkyConfig))
    return fail(SKY_ERR_ARG, "SkyConfig size %u, library expects %zu", cfg->struct_size,
                sizeof(SkyConfig));
  if (cfg->tile_size != 8 && cfg->tile_size != 16 && cfg->tile_size != 32)
    return fail(SKY_ERR_ARG, "tile_size %u not in {8, 16, 32}", cfg->tile_size);
  if (cfg->sh_degree > 3) return fail(SKY_ERR_ARG, "sh_degree %u > 3", cfg->sh_degree);
  if (cfg->backward_mode > 1) return fail(SKY_ERR_ARG, "unknown backward_mode");
  if (cfg->fwd_batch != 0 && cfg->fwd_batch != 64 && cfg->fwd_batch != 128 && cfg->fwd_batch != 256)
    return fail(SKY_ERR_ARG, "fwd_batch %u not in {0, 64, 128, 256}", cfg->fwd_batch);
  if (cfg->bwd_batch != 0 && cfg->bwd_batch != 32 && cfg->bwd_batch != 64 && cfg->bwd_batch != 128)
    return fail(SKY_ERR_ARG, "bwd_batch %u not in {0, 32, 64, 128}", cfg->bwd_batch);
  if (cfg->tile_cull > 1) return fail(SKY_ERR_ARG, "tile_cull %u not 0 or 1", cfg->tile_cull);
  if (cfg->batch_scaling > 1)
    return fail(SKY_ERR_ARG, "batch_scaling %u not 0 or 1", cfg->batch_scaling);
  return SKY_OK;
}

int sky_create(const SkyConfig* cfg, void** out) {
  if (!out) return fail(SKY_ERR_ARG, "null output pointer");
  *out = nullptr;
  TRY(check_cfg(cfg));
  Context* c = new Context();
  c->cfg = *cfg;
  c->rng = cfg->seed;
  int rc = SKY_OK;
  auto bail = [&](int r) {
    sky_destroy(c);
    return r;
  };
  cudaError_t e = cudaGetDevice(&c->device);
  if (e != cudaSuccess) return bail(fail(SKY_ERR_CUDA, "no CUDA device: %s", cudaGetErrorString(e)));
  e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) return bail(fail(SKY_ERR_CUDA, "stream: %s", cudaGetErrorString(e)));
  e = cudaMallocHost(&c->h_sp, sizeof(StepParams));
  if (e != cudaSuccess) return bail(fail(SKY_ERR_OOM, "pinned alloc: %s", cudaGetErrorString(e)));
  e = cudaMallocHost(&c->h_st, sizeof(DevStatus));
  if (e != cudaSuccess) return bail(fail(SKY_ERR_OOM, "pinned alloc: %s", cudaGetErrorString(e)));
  if ((rc = dev_alloc(c, c->d_sp, sizeof(StepParams))) != SKY_OK) return bail(rc);
  if ((rc = dev_alloc(c, c->d_st, sizeof(DevStatus))) != SKY_OK) return bail(rc);
  *out = c;
  return SKY_OK;
}

int sky_destroy(void* p) {
  Context* c = as_ctx(p);
  if (!c) return SKY_OK;
  if (c->stream) cudaStreamSynchronize(c->stream);
  Buf* all[] = {&c->params, &c->m1, &c->m2, &c->grads, &c->tmp_planes, &c->records, &c->aux,
                &c->counts, &c->rects, &c->rowspans, &c->cumsum, &c->block_sums, &c->ikeys,
                &c->ikeys_sorted, &c->perm, &c->item_end, &c->isort_mem, &c->keys,
                &c->keys_sorted, &c->vals_sorted, &c->rec_of, &c->flatten, &c->fmask, &c->partials, &c->reached,
                &c->tile_grads, &c->gsum54, &c->offsets, &c->loss_partials, &c->color,
                &c->alpha, &c->tfinal, &c->last, &c->residual, &c->targets, &c->sort_mem, &c->flags,
                &c->flag_scan, &c->d_sp, &c->d_st, &c->imp_stats, &c->dens_accum,
                &c->score_imp, &c->score_prune, &c->score_counts, &c->metric_l1,
                &c->metric_part, &c->metric_stats, &c->v_splats, &c->v_keys, &c->v_counts,
                &c->v_rects, &c->v_order, &c->v_ksorted, &c->v_cum, &c->v_csorted, &c->v_bsums,
                &c->v_misc, &c->v_tkeys, &c->v_gidx, &c->v_tkeys_s, &c->v_gidx_s, &c->v_offsets,
                &c->v_rgba, &c->v_sort, &c->item_sums};
  for (Buf* b : all) dev_free(c, *b);
  drop_graph(c);
  for (int k = 0; k <= SKY_NUM_STAGES; ++k)
    if (c->ev[k]) cudaEventDestroy(c->ev[k]);
  if (c->h_sp) cudaFreeHost(c->h_sp);
  if (c->h_st) cudaFreeHost(c->h_st);
  if (c->stream) cudaStreamDestroy(c->stream);
  delete c;
  return SKY_OK;
}

int sky_set_config(void* p, const SkyConfig* cfg) {
  Context* c = as_ctx(p);
  if (!c) return fail(SKY_ERR_ARG, "null context");
  TRY(check_cfg(cfg));
  if (cfg->tile_size != c->cfg.tile_size || cfg->backward_mode != c->cfg.backward_mode)
    return fail(SKY_ERR_ARG, "tile_size and backward_mode are fixed at creation");
  c->cfg = *cfg;
  return SKY_OK;
}

int sky_get_config(void* p, SkyConfig* out) {
  Context* c = as_ctx(p);
  if (!c || !out) return fail(SKY_ERR_ARG, "bad arguments");
  *out = c->cfg;
  return SKY_OK;
}

int sky_camera_pinhole(const float view[16], double fx, double fy, double cx, double cy,
                       uint32_t width, uint32_t height, SkyCamera* out) {
  if (!view || !out || width == 0 || height == 0) return fail(SKY_ERR_ARG, "bad camera");
  memset(out, 0, sizeof(*out));
  memcpy(out->view, view, 16 * sizeof(float));
  // get_pinhole_projection_matrix: rows (sx,0,ox,0), (0,sy,oy,0), (0,0,1,0),
  // (0,0,1,0), stored column-major.
  const double w = width, h = height;
  const double sx = 2.0 * fx / w, sy = -2.0 * fy / h;
  const double ox = 2.0 * cx / w - 1.0, oy = 1.0 - 2.0 * cy / h;
  float* P = out->proj;
  P[0 * 4 + 0] = (float)sx;
  P[1 * 4 + 1] = (float)sy;
  P[2 * 4 + 0] = (float)ox;
  P[2 * 4 + 1] = (float)oy;
  P[2 * 4 + 2] = 1.0f;
  P[2 * 4 + 3] = 1.0f;
  out->focal[0] = (float)fx;
  out->focal[1] = (float)fy;
  out->width = width;
  out->height = height;
  return SKY_OK;
}

static int load_planes(Context* c, uint32_t n) {
  uint32_t stride = (n + 255) & ~255u;
  if (stride == 0) stride = 256;
  const size_t bytes = (size_t)kPlanes * stride * 4;
  TRY(dev_alloc(c, c->params, bytes));
  TRY(dev_alloc(c, c->m1, bytes));
  TRY(dev_alloc(c, c->m2, bytes));
  CK(cudaMemsetAsync(c->m1.p, 0, bytes, c->stream));
  CK(cudaMemsetAsync(c->m2.p, 0, bytes, c->stream));
  c->n = n;
  c->stride = stride;
  c->iteration = 0;
  c->adam_steps = 0;
  c->adam_views = 0;
  c->fwd_ready = false;
  c->scores_valid = false;
  c->scores_n = 0;
  TRY(reset_stats(c));
  return SKY_OK;
}

int sky_load_points(void* p, const float* params, uint32_t n, uint64_t plane_stride) {
  Context* c = as_ctx(p);
  if (!c || !params || n == 0 || plane_stride < n) return fail(SKY_ERR_ARG, "bad points");
  TRY(load_planes(c, n));
  CK(cudaMemcpy2DAsync(c->params.p, (size_t)c->stride * 4, params, (size_t)plane_stride * 4,
                       (size_t)n * 4, kPlanes, cudaMemcpyHostToDevice, c->stream));
  // scene_extent = max bounding-box extent (pointcloud-loader.ts:103-106)
  double ext = 0.0;
  for (int k = 0; k < 3; ++k) {
    const float* v = params + (size_t)k * plane_stride;
    float lo = v[0], hi = v[0];
    for (uint32_t i = 1; i < n; ++i) {
      lo = std::min(lo, v[i]);
      hi = std::max(hi, v[i]);
    }
    ext = std::max(ext, (double)hi - (double)lo);
  }
  c->scene_extent = (float)ext;
  CK(cudaStreamSynchronize(c->stream));
  return SKY_OK;
}

static float half_to_float(uint16_t h) {
  const uint32_t s = (uint32_t)(h & 0x8000u) << 16;
  uint32_t e = (h >> 10) & 0x1Fu, m = h & 0x3FFu;
  uint32_t bits;
  if (e == 0) {
    if (m == 0) {
      bits = s;
    } else {
      e = 127 - 15 + 1;
      while (!(m & 0x400u)) {
        m <<= 1;
        --e;
      }
      m &= 0x3FFu;
      bits = s | (e << 23) | (m << 13);
    }
  } else if (e == 31) {
    bits = s | 0x7F800000u | (m << 13);
  } else {
    bits = s | ((e + 112) << 23) | (m << 13);
  }
  float f;
  memcpy(&f, &bits, 4);
  return f;
}

int sky_load_packed(void* p, const uint32_t* gaussians, const uint32_t* sh, uint32_t n) {
  Context* c = as_ctx(p);
  if (!c || !gaussians || n == 0) return fail(SKY_ERR_ARG, "bad packed points");
  // training_init_params (training-params.wgsl:35-79): halves
  // [x, y | z, opacity | rot0, rot1 | rot2, rot3 | s0, s1 | s2, pad];
  // train_rotation = (rot1, rot2, rot3, rot0).
  std::vector<float> planes((size_t)kPlanes * n, 0.0f);
  for (uint32_t i = 0; i < n; ++i) {
    const uint16_t* h = (const uint16_t*)(gaussians + (size_t)i * 6);
    float f[12];
    for (int k = 0; k < 12; ++k) f[k] = half_to_float(h[k]);
    const float vals[11] = {f[0], f[1], f[2], f[8], f[9], f[10], f[5], f[6], f[7], f[4], f[3]};
    for (int k = 0; k < 11; ++k) planes[(size_t)k * n + i] = vals[k];
    if (sh) {
      const uint16_t* hs = (const uint16_t*)(sh + (size_t)i * 24);
      for (int k = 0; k < 48; ++k) planes[(size_t)(11 + k) * n + i] = half_to_float(hs[k]);
    }
  }
  return sky_load_points(p, planes.data(), n, n);
}

int sky_load_ply(void* p, const char* path, uint32_t* n_out, uint32_t* deg_out) {
  Context* c = as_ctx(p);
  if (!c || !path) return fail(SKY_ERR_ARG, "bad PLY arguments");
  PlyScene sc;
  std::string err;
  if (ply_read(path, sc, err) != 0) return fail(SKY_ERR_ARG, "%s", err.c_str());
  TRY(sky_load_points(p, sc.planes.data(), sc.n, sc.n));
  c->scene_extent = (float)sc.extent;
  if (n_out) *n_out = sc.n;
  if (deg_out) *deg_out = sc.sh_deg;
  return SKY_OK;
}

int sky_ply_read_host(const char* path, uint32_t* n_out, uint32_t* deg_out, float* planes,
                      uint64_t capacity, double* extent_out) {
  if (!path) return fail(SKY_ERR_ARG, "null path");
  PlyScene sc;
  std::string err;
  if (ply_read(path, sc, err) != 0) return fail(SKY_ERR_ARG, "%s", err.c_str());
  if (n_out) *n_out = sc.n;
  if (deg_out) *deg_out = sc.sh_deg;
  if (extent_out) *extent_out = sc.extent;
  if (planes) {
    if (capacity < sc.planes.size())
      return fail(SKY_ERR_ARG, "planes hold %llu floats, need %zu", (unsigned long long)capacity,
                  sc.planes.size());
    memcpy(planes, sc.planes.data(), sc.planes.size() * sizeof(float));
  }
  return SKY_OK;
}

int sky_save_ply(void* p, const char* path, uint32_t sh_degree) {
  Context* c = as_ctx(p);
  if (!c || !path) return fail(SKY_ERR_ARG, "bad PLY arguments");
  if (c->n == 0) return fail(SKY_ERR_STATE, "no Gaussians loaded");
  std::vector<float> planes((size_t)kPlanes * c->n);
  TRY(sky_get_params(p, planes.data(), c->n));
  std::string err;
  if (ply_write(path, planes.data(), c->n, c->n, sh_degree, err) != 0)
    return fail(SKY_ERR_ARG, "%s", err.c_str());
  return SKY_OK;
}

namespace {
struct CkptHeader {
  char magic[8];  // "SKYCKPT1"
  uint32_t version, n, planes, reserved0;
  uint64_t iteration, adam_steps, rng;
  float scene_extent;
  uint32_t densify_runs, prune_runs;
  uint32_t adam_views;  // saturating; 0 in files written before it was kept
};
}  // namespace

int sky_save_checkpoint(void* p, const char* path) {
  Context* c = as_ctx(p);
  if (!c || !path) return fail(SKY_ERR_ARG, "bad checkpoint arguments");
  if (c->n == 0) return fail(SKY_ERR_STATE, "no Gaussians loaded");
  const uint32_t n = c->n;
  CkptHeader h{};
  memcpy(h.magic, "SKYCKPT1", 8);
  h.version = 1;
  h.n = n;
  h.planes = kPlanes;
  h.iteration = c->iteration;
  h.adam_steps = c->adam_steps;
  h.rng = c->rng;
  h.scene_extent = c->scene_extent;
  h.densify_runs = c->densify_runs;
  h.prune_runs = c->prune_runs;
  h.adam_views = (uint32_t)std::min<uint64_t>(c->adam_views, 0xFFFFFFFFu);
  std::vector<float> P((size_t)kPlanes * n), M1(P.size()), M2(P.size()), I4((size_t)n * 4), G4(I4.size());
  TRY(sky_get_params(p, P.data(), n));
  TRY(sky_get_moments(p, M1.data(), M2.data(), n));
  TRY(sky_densify_stats(p, G4.data(), I4.data()));
  FILE* f = fopen(path, "wb");
  if (!f) return fail(SKY_ERR_ARG, "cannot create %s", path);
  bool ok = fwrite(&h, sizeof(h), 1, f) == 1;
  for (const std::vector<float>* v : {&P, &M1, &M2, &I4, &G4})
    ok = ok && fwrite(v->data(), 4, v->size(), f) == v->size();
  if (fclose(f) != 0) ok = false;
  if (!ok) return fail(SKY_ERR_ARG, "write failed: %s", path);
  return SKY_OK;
}

int sky_load_checkpoint(void* p, const char* path) {
  Context* c = as_ctx(p);
  if (!c || !path) return fail(SKY_ERR_ARG, "bad checkpoint arguments");
  FILE* f = fopen(path, "rb");
  if (!f) return fail(SKY_ERR_ARG, "cannot open %s", path);
  CkptHeader h{};
  bool ok = fread(&h, sizeof(h), 1, f) == 1;
  if (!ok || memcmp(h.magic, "SKYCKPT1", 8) != 0 || h.version != 1 || h.planes != (uint32_t)kPlanes ||
      h.n == 0 || h.n >= (1u << 31)) {
    fclose(f);
    return fail(SKY_ERR_ARG, "%s is not a version-1 skyfall checkpoint", path);
  }
  const uint32_t n = h.n;
  std::vector<float> P((size_t)kPlanes * n), M1(P.size()), M2(P.size()), I4((size_t)n * 4), G4(I4.size());
  for (std::vector<float>* v : {&P, &M1, &M2, &I4, &G4}) ok = ok && fread(v->data(), 4, v->size(), f) == v->size();
  fclose(f);
  if (!ok) return fail(SKY_ERR_ARG, "%s is truncated", path);
  TRY(load_planes(c, n));
  cudaStream_t s = c->stream;
  const size_t pitch = (size_t)c->stride * 4;
  CK(cudaMemcpy2DAsync(c->params.p, pitch, P.data(), (size_t)n * 4, (size_t)n * 4, kPlanes,
                       cudaMemcpyHostToDevice, s));
  CK(cudaMemcpy2DAsync(c->m1.p, pitch, M1.data(), (size_t)n * 4, (size_t)n * 4, kPlanes,
                       cudaMemcpyHostToDevice, s));
  CK(cudaMemcpy2DAsync(c->m2.p, pitch, M2.data(), (size_t)n * 4, (size_t)n * 4, kPlanes,
                       cudaMemcpyHostToDevice, s));
  CK(cudaMemcpyAsync(c->imp_stats.p, I4.data(), (size_t)n * 16, cudaMemcpyHostToDevice, s));
  CK(cudaMemcpyAsync(c->dens_accum.p, G4.data(), (size_t)n * 16, cudaMemcpyHostToDevice, s));
  CK(cudaStreamSynchronize(s));
  c->iteration = h.iteration;
  c->adam_steps = h.adam_steps;
  c->adam_views = h.adam_views ? h.adam_views : h.adam_steps;
  c->rng = h.rng;
  c->scene_extent = h.scene_extent;
  c->densify_runs = h.densify_runs;
  c->prune_runs = h.prune_runs;
  return SKY_OK;
}

int sky_knn_init(void* p, float scene_extent, float* density_out) {
  Context* c = as_ctx(p);
  if (!c) return fail(SKY_ERR_ARG, "null context");
  if (c->n == 0) return fail(SKY_ERR_STATE, "no Gaussians loaded");
  if (c->n >= (1u << 30)) return fail(SKY_ERR_ARG, "k-NN init supports fewer than 2^30 Gaussians");
  const uint32_t n = c->n;
  cudaStream_t s = c->stream;
  const float extent = scene_extent > 0.0f ? scene_extent : c->scene_extent;
  TempBuf bounds(c), keys(c), ksorted(c), order(c), cstart(c), logs(c), dens(c), smem(c);
  TRY(dev_alloc(c, bounds.b, 64));
  uint32_t init[6];
  for (int k = 0; k < 6; ++k) init[k] = knn_bounds_init(k);
  CK(cudaMemcpyAsync(bounds.b.p, init, sizeof(init), cudaMemcpyHostToDevice, s));
  launch_knn_bounds((const float*)c->params.p, c->stride, n, bounds.as<uint32_t>(), s);
  uint32_t bw[6];
  CK(cudaMemcpyAsync(bw, bounds.b.p, sizeof(bw), cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  // grid: about two points per cell over the bounding box, at most 2^22
  // cells and 1024 per axis
  KnnGrid g{};
  double ext[3], big = 0.0;
  for (int k = 0; k < 3; ++k) {
    g.lo[k] = knn_bounds_decode(bw[k]);
    const float hi = knn_bounds_decode(bw[3 + k]);
    ext[k] = std::isfinite(g.lo[k]) && std::isfinite(hi) ? std::max(0.0, (double)hi - (double)g.lo[k]) : 0.0;
    if (!std::isfinite(g.lo[k])) g.lo[k] = 0.0f;
    big = std::max(big, ext[k]);
  }
  double h = big > 0.0 ? big / 1024.0 : 1.0;
  if (big > 0.0) {
    const double floor_e = big / 1024.0;
    const double vol = std::max(ext[0], floor_e) * std::max(ext[1], floor_e) * std::max(ext[2], floor_e);
    const double want = std::min<double>(std::max<double>(n / 2.0, 1.0), (double)(1u << 22));
    h = std::max(h, std::cbrt(vol / want));
  }
  for (;;) {
    uint64_t cells = 1;
    for (int k = 0; k < 3; ++k) {
      g.dims[k] = (uint32_t)std::min(1024.0, std::max(1.0, std::ceil(ext[k] / h)));
      cells *= g.dims[k];
    }
    if (cells <= (1u << 22)) {
      g.cells = (uint32_t)cells;
      break;
    }
    h *= 1.25;
  }
  g.h = (float)h;
  TRY(dev_alloc(c, keys.b, (size_t)n * 4));
  TRY(dev_alloc(c, ksorted.b, (size_t)n * 4));
  TRY(dev_alloc(c, order.b, (size_t)n * 4));
  TRY(dev_alloc(c, cstart.b, ((size_t)g.cells + 1) * 4));
  TRY(dev_alloc(c, logs.b, (size_t)n * 4));
  if (density_out) TRY(dev_alloc(c, dens.b, (size_t)n * 4));
  TRY(dev_alloc(c, smem.b, sort_scratch_bytes(n)));
  launch_knn_keys((const float*)c->params.p, c->stride, n, g, keys.as<uint32_t>(), s);
  SortScratch sc = sort_scratch_carve(smem.b.p, n);
  SortSegment seg{nullptr, n};
  uint32_t* err = bounds.as<uint32_t>() + 8;
  CK(cudaMemsetAsync(err, 0, 4, s));
  CK(sort_pairs_launch(keys.as<uint32_t>(), nullptr, ksorted.as<uint32_t>(), order.as<uint32_t>(), seg,
                       n, std::max<uint32_t>(1, ceil_log2(g.cells)), sc, err, s));
  launch_knn_cell_ranges(ksorted.as<uint32_t>(), n, g.cells, cstart.as<uint32_t>(), s);
  launch_knn_query((float*)c->params.p, c->stride, n, g, order.as<uint32_t>(), cstart.as<uint32_t>(),
                   extent, dens.as<float>(), logs.as<float>(), s);
  launch_knn_write((float*)c->params.p, c->stride, n, logs.as<float>(), s);
  c->launches += 10;
  CK(cudaGetLastError());
  uint32_t e = 0;
  CK(cudaMemcpyAsync(&e, err, 4, cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  if (e & SKY_DEVERR_SORT_TIMEOUT) return fail(SKY_ERR_TIMEOUT, "radix sort look-back wait gave up");
  if (density_out) CK(cudaMemcpy(density_out, dens.b.p, (size_t)n * 4, cudaMemcpyDeviceToHost));
  c->fwd_ready = false;
  c->scores_valid = false;
  return SKY_OK;
}

int sky_set_cameras(void* p, const SkyCamera* cams, uint32_t n) {
  Context* c = as_ctx(p);
  if (!c || (!cams && n)) return fail(SKY_ERR_ARG, "bad cameras");
  for (uint32_t i = 0; i < n; ++i)
    if (cams[i].width == 0 || cams[i].height == 0 || cams[i].focal[0] <= 0 || cams[i].focal[1] <= 0)
      return fail(SKY_ERR_ARG, "camera %u has an empty image or non-positive focal", i);
  c->cams.assign(cams, cams + n);
  c->tgt_base.assign(n, 0);
  c->tgt_set.assign(n, 0);
  c->targets_px = 0;
  c->fwd_ready = false;
  return SKY_OK;
}

int sky_set_target(void* p, uint32_t cam, const float* rgb, uint32_t width, uint32_t height) {
  Context* c = as_ctx(p);
  if (!c || !rgb) return fail(SKY_ERR_ARG, "bad target");
  if (cam >= c->cams.size()) return fail(SKY_ERR_ARG, "camera %u not set", cam);
  if (width != c->cams[cam].width || height != c->cams[cam].height)
    return fail(SKY_ERR_ARG, "target %ux%u does not match camera %ux%u", width, height,
                c->cams[cam].width, c->cams[cam].height);
  const uint64_t px = (uint64_t)width * height;
  uint64_t base;
  if (c->tgt_set[cam]) {
    base = c->tgt_base[cam];
  } else {
    base = c->targets_px;
    if (base + px >= (1ull << 32)) return fail(SKY_ERR_ARG, "target images exceed 2^32 pixels");
    TRY(dev_alloc(c, c->targets, (base + px) * 16, true));
    c->targets_px = base + px;
  }
  std::vector<float> rgba(px * 4);
  for (uint64_t i = 0; i < px; ++i) {
    rgba[i * 4 + 0] = rgb[i * 3 + 0];
    rgba[i * 4 + 1] = rgb[i * 3 + 1];
    rgba[i * 4 + 2] = rgb[i * 3 + 2];
    rgba[i * 4 + 3] = 1.0f;
  }
  CK(cudaMemcpyAsync((char*)c->targets.p + base * 16, rgba.data(), px * 16,
                     cudaMemcpyHostToDevice, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  c->tgt_base[cam] = base;
  c->tgt_set[cam] = 1;
  return SKY_OK;
}

int sky_render(void* p, const uint32_t* cams, uint32_t n, float* rgba, float* alpha) {
  Context* c = as_ctx(p);
  if (!c || !cams) return fail(SKY_ERR_ARG, "bad render arguments");
  TRY(run_views(c, cams, n, kRender, nullptr));
  if (rgba) CK(cudaMemcpy(rgba, c->color.p, (size_t)c->last_pixels * 16, cudaMemcpyDeviceToHost));
  if (alpha) CK(cudaMemcpy(alpha, c->alpha.p, (size_t)c->last_pixels * 4, cudaMemcpyDeviceToHost));
  return SKY_OK;
}

int sky_forward(void* p, const uint32_t* cams, uint32_t n, double* loss) {
  Context* c = as_ctx(p);
  if (!c || !cams) return fail(SKY_ERR_ARG, "bad forward arguments");
  TRY(run_views(c, cams, n, kForward, nullptr));
  if (loss) *loss = c->last_loss;
  return SKY_OK;
}

int sky_backward(void* p, float* grads, uint64_t plane_stride) {
  Context* c = as_ctx(p);
  if (!c) return fail(SKY_ERR_ARG, "null context");
  if (!c->fwd_ready) return fail(SKY_ERR_STATE, "sky_backward needs a preceding sky_forward");
  std::vector<uint32_t> views = c->last_views;
  TRY(run_views(c, views.data(), (uint32_t)views.size(), kBackward, nullptr));
  if (grads) {
    if (plane_stride < c->n) return fail(SKY_ERR_ARG, "plane_stride < number of Gaussians");
    CK(cudaMemcpy2D(grads, plane_stride * 4, c->grads.p, (size_t)c->stride * 4, (size_t)c->n * 4,
                    kPlanes, cudaMemcpyDeviceToHost));
  }
  return SKY_OK;
}

int sky_step(void* p, const uint32_t* cams, uint32_t n, SkyStepStats* stats) {
  Context* c = as_ctx(p);
  if (!c || !cams) return fail(SKY_ERR_ARG, "bad step arguments");
  return run_views(c, cams, n, kTrain, stats);
}

int sky_train(void* p, uint32_t iterations, uint32_t views_per_step, SkyStepStats* last) {
  Context* c = as_ctx(p);
  if (!c) return fail(SKY_ERR_ARG, "null context");
  if (c->cams.empty()) return fail(SKY_ERR_STATE, "no cameras");
  if (views_per_step == 0) views_per_step = 1;
  std::vector<uint32_t> v(views_per_step);
  for (uint32_t i = 0; i < iterations; ++i) {
    // Math.floor(Math.random() * numCameras) with a seeded generator
    for (uint32_t k = 0; k < views_per_step; ++k)
      v[k] = (uint32_t)(((splitmix64(c->rng) >> 11) * (1.0 / 9007199254740992.0)) * c->cams.size());
    TRY(run_views(c, v.data(), views_per_step, kTrain, last));
    if (c->sched.enabled) TRY(run_schedule(c));
  }
  return SKY_OK;
}

int sky_get_params(void* p, float* out, uint64_t plane_stride) {
  Context* c = as_ctx(p);
  if (!c || !out || plane_stride < c->n) return fail(SKY_ERR_ARG, "bad readback");
  if (c->n == 0) return SKY_OK;
  CK(cudaStreamSynchronize(c->stream));
  CK(cudaMemcpy2D(out, plane_stride * 4, c->params.p, (size_t)c->stride * 4, (size_t)c->n * 4,
                  kPlanes, cudaMemcpyDeviceToHost));
  return SKY_OK;
}

int sky_get_moments(void* p, float* m1, float* m2, uint64_t plane_stride) {
  Context* c = as_ctx(p);
  if (!c || plane_stride < c->n) return fail(SKY_ERR_ARG, "bad readback");
  if (c->n == 0) return SKY_OK;
  CK(cudaStreamSynchronize(c->stream));
  if (m1)
    CK(cudaMemcpy2D(m1, plane_stride * 4, c->m1.p, (size_t)c->stride * 4, (size_t)c->n * 4,
                    kPlanes, cudaMemcpyDeviceToHost));
  if (m2)
    CK(cudaMemcpy2D(m2, plane_stride * 4, c->m2.p, (size_t)c->stride * 4, (size_t)c->n * 4,
                    kPlanes, cudaMemcpyDeviceToHost));
  return SKY_OK;
}

int sky_get_count(void* p, uint32_t* n) {
  Context* c = as_ctx(p);
  if (!c || !n) return fail(SKY_ERR_ARG, "bad arguments");
  *n = c->n;
  return SKY_OK;
}

int sky_get_status(void* p, SkyStatus* st) {
  Context* c = as_ctx(p);
  if (!c || !st) return fail(SKY_ERR_ARG, "bad arguments");
  memset(st, 0, sizeof(*st));
  st->iteration = c->iteration;
  st->adam_steps = c->adam_steps;
  st->last_intersections = c->last_isect;
  st->device_bytes = c->device_bytes;
  st->num_gaussians = c->n;
  st->capacity = c->stride;
  st->num_cameras = (uint32_t)c->cams.size();
  st->error_flags = c->error_flags;
  st->kernel_launches = c->launches;
  st->graph_replays = c->graph_replays;
  st->graph_captures = c->graph_captures;
  st->scene_extent = c->scene_extent;
  st->scored_views = c->scores_views;
  st->densify_runs = c->densify_runs;
  st->prune_runs = c->prune_runs;
  st->step_h2d_bytes = c->step_h2d;
  st->step_d2h_bytes = c->step_d2h;
  return SKY_OK;
}

int sky_read_buffer(void* p, int which, void* dst, uint64_t bytes, uint64_t* size_out) {
  Context* c = as_ctx(p);
  if (!c) return fail(SKY_ERR_ARG, "null context");
  const uint64_t items = c->last_items, I = std::min<uint64_t>(c->last_isect, c->icap);
  const uint64_t T = c->last_tiles, P = c->last_pixels;
  const void* src = nullptr;
  uint64_t sz = 0, pitch_src = 0, rows = 0, row_bytes = 0;
  switch (which) {
    case SKY_BUF_RECORDS: src = c->records.p; sz = items * 48; break;
    case SKY_BUF_DEPTH_RADIUS: src = c->aux.p; sz = items * 8; break;
    case SKY_BUF_COUNTS: src = c->counts.p; sz = items * 4; break;
    case SKY_BUF_CUMSUM: src = c->cumsum.p; sz = items * 4; break;
    case SKY_BUF_ITEM_ORDER: src = c->perm.p; sz = items * 4; break;
    case SKY_BUF_KEYS_EMIT: src = c->keys.p; sz = I * 4; break;
    case SKY_BUF_KEYS_SORTED: src = c->keys_sorted.p; sz = I * 4; break;
    case SKY_BUF_VALS_SORTED: src = c->vals_sorted.p; sz = I * 4; break;
    case SKY_BUF_FLATTEN: src = c->flatten.p; sz = I * 4; break;
    case SKY_BUF_TILE_OFFSETS: src = c->offsets.p; sz = (T + 1) * 4; break;
    case SKY_BUF_COLOR: src = c->color.p; sz = P * 16; break;
    case SKY_BUF_ALPHA: src = c->alpha.p; sz = P * 4; break;
    case SKY_BUF_LAST_IDS: src = c->last.p; sz = P * 4; break;
    case SKY_BUF_RESIDUAL: src = c->residual.p; sz = P * 16; break;
    case SKY_BUF_PARTIALS: src = c->partials.p; sz = I * kPartialF4 * 16; break;
    case SKY_BUF_TILE_GRADS: src = c->tile_grads.p; sz = c->tile_grads.p ? I * 54 * 4 : 0; break;
    case SKY_BUF_VIEW_RGBA: src = c->v_rgba.p; sz = (uint64_t)c->view_w * c->view_h * 16; break;
    case SKY_BUF_GRADS:
      src = c->grads.p;
      sz = c->grads.p ? (uint64_t)kPlanes * c->n * 4 : 0;
      pitch_src = (uint64_t)c->stride * 4;
      rows = kPlanes;
      row_bytes = (uint64_t)c->n * 4;
      break;
    case SKY_BUF_STEP_SCALARS: {
      const StepParams& q = *c->h_sp;
      const float v[12] = {q.lr_pos, q.lr_scale, q.lr_rot, q.lr_opacity, q.lr_sh, q.beta1,
                           q.beta2, q.adam_eps, q.bc1_rcp, q.bc2_sqrt_rcp, (float)q.sh_deg,
                           (float)q.sh_update};
      if (size_out) *size_out = sizeof(v);
      if (dst && bytes >= sizeof(v)) memcpy(dst, v, sizeof(v));
      return SKY_OK;
    }
    case SKY_BUF_PAIR_COUNTS: {
      if (size_out) *size_out = sizeof(c->h_st->pairs);
      if (dst && bytes >= sizeof(c->h_st->pairs)) memcpy(dst, c->h_st->pairs, sizeof(c->h_st->pairs));
      return SKY_OK;
    }
    case SKY_BUF_GROUPS: {
      if (size_out) *size_out = (uint64_t)c->last_groups * 8;
      if (dst && bytes >= (uint64_t)c->last_groups * 8)
        memcpy(dst, c->h_st->group_bounds, (size_t)c->last_groups * 8);
      return SKY_OK;
    }
    default: return fail(SKY_ERR_ARG, "unknown buffer %d", which);
  }
  if (size_out) *size_out = sz;
  if (!dst || sz == 0) return SKY_OK;
  if (bytes < sz) return fail(SKY_ERR_ARG, "destination holds %llu bytes, need %llu",
                              (unsigned long long)bytes, (unsigned long long)sz);
  if (which == SKY_BUF_PARTIALS) {
    // the exact backward writes only the partials it flags; the rest are zero
    launch_partials_fill(make_buffers(c), (uint32_t)I, c->stream);
    CK(cudaGetLastError());
  }
  if (which == SKY_BUF_FLATTEN) {
    // the step resolved only the staged batches; complete it for the reader
    launch_flatten_fill(make_buffers(c), (uint32_t)I, c->stream);
    CK(cudaGetLastError());
  }
  CK(cudaStreamSynchronize(c->stream));
  if (rows)
    CK(cudaMemcpy2D(dst, row_bytes, src, pitch_src, row_bytes, rows, cudaMemcpyDeviceToHost));
  else
    CK(cudaMemcpy(dst, src, sz, cudaMemcpyDeviceToHost));
  return SKY_OK;
}

int sky_sync(void* p) {
  Context* c = as_ctx(p);
  if (!c) return fail(SKY_ERR_ARG, "null context");
  CK(cudaStreamSynchronize(c->stream));
  return SKY_OK;
}

int sky_get_stream(void* p, void** stream) {
  Context* c = as_ctx(p);
  if (!c || !stream) return fail(SKY_ERR_ARG, "bad arguments");
  *stream = (void*)c->stream;
  return SKY_OK;
}

int sky_set_profiling(void* p, int enabled) {
  Context* c = as_ctx(p);
  if (!c) return fail(SKY_ERR_ARG, "null context");
  if (enabled < 0 || enabled > 2) return fail(SKY_ERR_ARG, "profiling level %d not 0, 1 or 2", enabled);
  if (enabled && !c->ev[0])
    for (int k = 0; k <= SKY_NUM_STAGES; ++k) CK(cudaEventCreate(&c->ev[k]));
  c->profiling = enabled != 0;
  c->count_pairs = enabled == 2;
  for (int k = 0; k < SKY_NUM_STAGES; ++k) c->stage_ms[k] = 0.0;
  c->prof_steps = 0;
  return SKY_OK;
}

int sky_get_stage_times(void* p, double* ms, uint32_t n, uint64_t* steps) {
  Context* c = as_ctx(p);
  if (!c) return fail(SKY_ERR_ARG, "null context");
  for (uint32_t k = 0; k < n && k < (uint32_t)SKY_NUM_STAGES; ++k) ms[k] = c->stage_ms[k];
  if (steps) *steps = c->prof_steps;
  return SKY_OK;
}

// ---- device-pointer sort ---------------------------------------------------
static std::mutex g_sort_mu;
struct SortCache {
  void* mem = nullptr;
  size_t bytes = 0;
  uint32_t max_n = 0;
  uint32_t* err = nullptr;
};
static SortCache g_sort_cache[64];

int sky_sort_pairs(const uint32_t* keys_in, const uint32_t* vals_in, uint32_t* keys_out,
                   uint32_t* vals_out, uint32_t n, uint32_t key_bits, void* stream) {
  if (!keys_in || !keys_out || !vals_out) return fail(SKY_ERR_ARG, "null device pointer");
  if (key_bits == 0 || key_bits > 32) return fail(SKY_ERR_ARG, "key_bits %u outside 1..32", key_bits);
  if (n >= (1u << 30)) return fail(SKY_ERR_ARG, "n = %u exceeds 2^30 - 1", n);
  if (keys_in == keys_out || (vals_in && vals_in == vals_out))
    return fail(SKY_ERR_ARG, "input and output arrays must differ");
  if (n == 0) return SKY_OK;
  int dev = 0;
  CK(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) return fail(SKY_ERR_ARG, "device index %d unsupported", dev);
  std::lock_guard<std::mutex> lock(g_sort_mu);
  SortCache& sc = g_sort_cache[dev];
  cudaStream_t s = (cudaStream_t)stream;
  if (n > sc.max_n) {
    if (sc.mem) {
      CK(cudaDeviceSynchronize());
      cudaFree(sc.mem);
      sc.mem = nullptr;
    }
    const size_t bytes = sort_scratch_bytes(n) + 256;
    if (inject_alloc()) return fail(SKY_ERR_INJECTED, "injected allocation failure");
    CK(cudaMalloc(&sc.mem, bytes));
    sc.bytes = bytes;
    sc.max_n = n;
    sc.err = (uint32_t*)((char*)sc.mem + bytes - 256);
  }
  SortScratch scr = sort_scratch_carve(sc.mem, sc.max_n);
  CK(cudaMemsetAsync(sc.err, 0, 4, s));
  SortSegment seg{nullptr, n};
  CK(sort_pairs_launch(keys_in, vals_in, keys_out, vals_out, seg, n, key_bits, scr, sc.err, s, 0,
                       true));
  uint32_t err = 0;
  CK(cudaMemcpyAsync(&err, sc.err, 4, cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  if (err & SKY_DEVERR_SORT_TIMEOUT) return fail(SKY_ERR_TIMEOUT, "radix sort look-back wait gave up");
  return SKY_OK;
}

int sky_densify_stats(void* p, float* grad_accum, float* importance) {
  Context* c = as_ctx(p);
  if (!c) return fail(SKY_ERR_ARG, "null context");
  if (c->n == 0) return SKY_OK;
  CK(cudaStreamSynchronize(c->stream));
  if (grad_accum)
    CK(cudaMemcpy(grad_accum, c->dens_accum.p, (size_t)c->n * 16, cudaMemcpyDeviceToHost));
  if (importance)
    CK(cudaMemcpy(importance, c->imp_stats.p, (size_t)c->n * 16, cudaMemcpyDeviceToHost));
  return SKY_OK;
}

void sky_densify_default(SkyDensifyParams* p) {
  if (!p) return;
  memset(p, 0, sizeof(*p));
  p->grad_threshold = 0.003f;
  p->grad_abs_threshold = 0.015f;
  p->size_threshold = 0.0f;  // 0: 0.001 * scene extent
  p->min_visibility = 25.0f;
  p->importance_threshold = 5.0f;
  p->max_new_ratio = 0.1f;
  p->pixel_width = 0.0f;
}

void sky_scored_prune_default(SkyScoredPruneParams* p) {
  if (!p) return;
  memset(p, 0, sizeof(*p));
  p->min_opacity = 0.005f;
  p->max_scale = 1.0f;
  p->max_screen_radius = 20.0f;
  p->use_screen_size = 0;
  p->prune_ratio = 0.5f;
  p->max_ratio = 0.02f;
  p->opacity_bonus = 0.35f;
  p->scale_bonus = 0.25f;
  p->screen_bonus = 0.25f;
  p->use_last_scores = 0;
}

void sky_schedule_default(SkySchedule* s) {
  if (!s) return;
  memset(s, 0, sizeof(*s));
  s->enabled = 1;
  s->densify_from = 500;
  s->densify_until = 15000;
  s->densify_interval = 100;
  s->prune_from = 500;
  s->prune_until = 25000;
  s->prune_interval = 100;
  s->opacity_reset_interval = 3000;
  s->opacity_reset_value = 0.01f;
  s->min_opacity = 0.005f;
  s->max_screen_size = 20.0f;
  s->max_scale_ratio = 0.0f;
  s->max_scale_absolute = 1.0f;
  s->scene_extent = 0.0f;
  sky_densify_default(&s->densify);
}

int sky_set_schedule(void* p, const SkySchedule* s) {
  Context* c = as_ctx(p);
  if (!c || !s) return fail(SKY_ERR_ARG, "bad schedule arguments");
  if (s->enabled && (s->densify_interval == 0 || s->prune_interval == 0 || s->opacity_reset_interval == 0))
    return fail(SKY_ERR_ARG, "schedule intervals must be positive");
  c->sched = *s;
  return SKY_OK;
}

int sky_score_views(void* p, const uint32_t* cams, uint32_t n, uint32_t* importance, float* pruning) {
  Context* c = as_ctx(p);
  if (!c) return fail(SKY_ERR_ARG, "null context");
  if (c->n == 0) return fail(SKY_ERR_STATE, "no Gaussians loaded");
  std::vector<uint32_t> list;
  if (cams) {
    if (n == 0) return fail(SKY_ERR_ARG, "no cameras to score");
    list.assign(cams, cams + n);
  } else {
    list = sample_cameras(c);
  }
  if (list.empty()) return fail(SKY_ERR_STATE, "no cameras to score");
  TRY(score_views(c, list));
  if (importance)
    CK(cudaMemcpy(importance, c->score_imp.p, (size_t)c->scores_n * 4, cudaMemcpyDeviceToHost));
  if (pruning)
    CK(cudaMemcpy(pruning, c->score_prune.p, (size_t)c->scores_n * 4, cudaMemcpyDeviceToHost));
  return SKY_OK;
}

int sky_densify(void* p, const SkyDensifyParams* prm, uint32_t* cloned, uint32_t* split) {
  Context* c = as_ctx(p);
  if (cloned) *cloned = 0;
  if (split) *split = 0;
  if (!c || !prm) return fail(SKY_ERR_ARG, "bad densify arguments");
  if (!(prm->max_new_ratio >= 0.0f) || !(prm->min_visibility >= 0.0f))
    return fail(SKY_ERR_ARG, "negative densify ratio or visibility");
  return densify(c, *prm, cloned, split);
}

int sky_prune_scored(void* p, const SkyScoredPruneParams* prm, uint32_t* removed) {
  Context* c = as_ctx(p);
  if (removed) *removed = 0;
  if (!c || !prm) return fail(SKY_ERR_ARG, "bad prune arguments");
  return prune_scored(c, *prm, removed);
}

int sky_reset_opacity(void* p, float max_opacity);

void sky_view_settings_default(SkyViewSettings* s) {
  if (!s) return;
  memset(s, 0, sizeof(*s));
  s->gaussian_scaling = 1.0f;
  s->sh_degree = 3;
  s->round_params_f16 = 1;
}

int sky_view_render(void* p, const SkyCamera* cam, const SkyViewSettings* vs, float* rgba,
                    uint8_t* rgba8) {
  Context* c = as_ctx(p);
  if (!c || !cam || !vs) return fail(SKY_ERR_ARG, "bad view arguments");
  if (cam->width == 0 || cam->height == 0 || cam->width > 65535u * kViewTile ||
      cam->height > 65535u * kViewTile)
    return fail(SKY_ERR_ARG, "viewport %ux%u out of range", cam->width, cam->height);
  if (c->n == 0) return fail(SKY_ERR_STATE, "no Gaussians loaded");
  const uint32_t n = c->n;
  cudaStream_t s = c->stream;
  ViewerParams vp{};
  memcpy(vp.view, cam->view, sizeof(vp.view));
  memcpy(vp.proj, cam->proj, sizeof(vp.proj));
  vp.focal[0] = cam->focal[0];
  vp.focal[1] = cam->focal[1];
  vp.viewport[0] = (float)cam->width;
  vp.viewport[1] = (float)cam->height;
  vp.gaussian_scaling = vs->gaussian_scaling;
  vp.sh_deg = vs->sh_degree;
  vp.round_f16 = vs->round_params_f16;
  vp.n = n;
  vp.plane_stride = c->stride;
  vp.width = cam->width;
  vp.height = cam->height;
  vp.tiles_x = (cam->width + kViewTile - 1) / kViewTile;
  vp.tiles_y = (cam->height + kViewTile - 1) / kViewTile;
  const uint32_t tiles = vp.tiles_x * vp.tiles_y;
  const uint64_t px = (uint64_t)cam->width * cam->height;
  // per Gaussian: project, sort by depth key, counts in depth order, scan
  TRY(dev_alloc(c, c->v_splats, (size_t)n * 48));
  TRY(dev_alloc(c, c->v_keys, (size_t)n * 4));
  TRY(dev_alloc(c, c->v_counts, (size_t)n * 4));
  TRY(dev_alloc(c, c->v_rects, (size_t)n * 8));
  TRY(dev_alloc(c, c->v_order, (size_t)n * 4));
  TRY(dev_alloc(c, c->v_ksorted, (size_t)n * 4));
  TRY(dev_alloc(c, c->v_cum, (size_t)n * 4));
  TRY(dev_alloc(c, c->v_csorted, (size_t)n * 4));
  TRY(dev_alloc(c, c->v_bsums, ((size_t)scan_block_count(n) + 1) * 4));
  TRY(dev_alloc(c, c->v_misc, 64));
  TRY(dev_alloc(c, c->v_offsets, ((size_t)tiles + 1) * 4));
  TRY(dev_alloc(c, c->v_rgba, px * 16));
  unsigned long long* d_total = (unsigned long long*)c->v_misc.p;
  uint32_t* d_err = (uint32_t*)((char*)c->v_misc.p + 8);
  CK(cudaMemsetAsync(c->v_misc.p, 0, 64, s));
  launch_viewer_project(vp, (const float*)c->params.p, (float4*)c->v_splats.p, (uint32_t*)c->v_keys.p,
                        (uint32_t*)c->v_counts.p, (uint2*)c->v_rects.p, d_total, s);
  unsigned long long total = 0;
  CK(cudaMemcpyAsync(&total, d_total, 8, cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  if (total >= (1ull << 30)) return fail(SKY_ERR_CAPACITY, "%llu quad-tile pairs exceed 2^30", total);
  const uint32_t I = (uint32_t)total;
  TRY(dev_alloc(c, c->v_sort, sort_scratch_bytes(std::max(n, std::max(I, 1u)))));
  SortScratch sc = sort_scratch_carve(c->v_sort.p, std::max(n, std::max(I, 1u)));
  SortSegment seg_n{nullptr, n};
  CK(sort_pairs_launch((const uint32_t*)c->v_keys.p, nullptr, (uint32_t*)c->v_ksorted.p,
                       (uint32_t*)c->v_order.p, seg_n, n, 32, sc, d_err, s));
  launch_viewer_gather_counts((const uint32_t*)c->v_order.p, (const uint32_t*)c->v_counts.p, n,
                              (uint32_t*)c->v_csorted.p, s);
  DevBuffers sb{};
  sb.counts = (uint32_t*)c->v_csorted.p;
  sb.cumsum = (uint32_t*)c->v_cum.p;
  sb.block_sums = (uint32_t*)c->v_bsums.p;
  launch_scan(sb, n, s);
  c->launches += 8;
  // per quad-tile pair: emit in depth order, stable sort by tile, ranges
  if (I > 0) {
    TRY(dev_alloc(c, c->v_tkeys, (size_t)I * 4));
    TRY(dev_alloc(c, c->v_gidx, (size_t)I * 4));
    TRY(dev_alloc(c, c->v_tkeys_s, (size_t)I * 4));
    TRY(dev_alloc(c, c->v_gidx_s, (size_t)I * 4));
    launch_viewer_emit(vp, (const uint32_t*)c->v_order.p, (const uint32_t*)c->v_cum.p,
                       (const uint32_t*)c->v_csorted.p, (const uint2*)c->v_rects.p, n,
                       (uint32_t*)c->v_tkeys.p, (uint32_t*)c->v_gidx.p, s);
    SortSegment seg_i{nullptr, I};
    const uint32_t bits = std::max<uint32_t>(1, ceil_log2(tiles));
    CK(sort_pairs_launch((const uint32_t*)c->v_tkeys.p, (const uint32_t*)c->v_gidx.p,
                         (uint32_t*)c->v_tkeys_s.p, (uint32_t*)c->v_gidx_s.p, seg_i, I, bits, sc,
                         d_err, s));
    c->launches += 6;
  }
  launch_viewer_ranges(I ? (const uint32_t*)c->v_tkeys_s.p : nullptr, I, tiles,
                       (uint32_t*)c->v_offsets.p, s);
  launch_viewer_raster(vp, (const float4*)c->v_splats.p, (const uint32_t*)c->v_offsets.p,
                       I ? (const uint32_t*)c->v_gidx_s.p : nullptr, (float4*)c->v_rgba.p, s);
  c->launches += 2;
  CK(cudaGetLastError());
  uint32_t err = 0;
  CK(cudaMemcpyAsync(&err, d_err, 4, cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  if (err & SKY_DEVERR_SORT_TIMEOUT) return fail(SKY_ERR_TIMEOUT, "radix sort look-back wait gave up");
  c->view_w = cam->width;
  c->view_h = cam->height;
  if (rgba || rgba8) {
    std::vector<float> tmp;
    float* dst = rgba;
    if (!dst) {
      tmp.resize(px * 4);
      dst = tmp.data();
    }
    CK(cudaMemcpy(dst, c->v_rgba.p, px * 16, cudaMemcpyDeviceToHost));
    if (rgba8)
      for (uint64_t i = 0; i < px * 4; ++i) {
        const float v = std::min(std::max(dst[i], 0.0f), 1.0f);
        rgba8[i] = (uint8_t)std::lround(v * 255.0f);
      }
  }
  return SKY_OK;
}

}  // extern "C"

// ---- prune / opacity reset (compact.cu kernels) ---------------------------
extern "C" int sky_prune(void* p, const SkyPruneParams* prm, const uint8_t* mask,
                         uint32_t* removed) {
  Context* c = as_ctx(p);
  if (removed) *removed = 0;
  if (!c || (!prm && !mask)) return fail(SKY_ERR_ARG, "bad prune arguments");
  if (c->n == 0) return SKY_OK;
  const uint32_t n = c->n;
  cudaStream_t s = c->stream;
  Buf dmask;
  if (mask) {
    TRY(dev_alloc(c, dmask, n));
    CK(cudaMemcpyAsync(dmask.p, mask, n, cudaMemcpyHostToDevice, s));
  }
  TRY(dev_alloc(c, c->flags, (size_t)n * 4));
  const float min_op = prm ? prm->min_opacity : 0.0f;
  const float max_scale = prm ? prm->max_scale : INFINITY;
  launch_prune_flags((const float*)c->params.p, c->stride, n, min_op, max_scale,
                     (const uint8_t*)dmask.p, (uint32_t*)c->flags.p, s);
  // flags hold 1 for survivors; optional cap on the removal count
  std::vector<uint32_t> keep(n);
  CK(cudaMemcpyAsync(keep.data(), c->flags.p, (size_t)n * 4, cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  if (dmask.p) dev_free(c, dmask);
  uint64_t remove = 0;
  for (uint32_t i = 0; i < n; ++i) remove += keep[i] == 0;
  if (prm && prm->max_remove_ratio > 0.0f && remove > 0) {
    const uint64_t cap = std::max<uint64_t>(1, (uint64_t)std::floor(n * (double)prm->max_remove_ratio));
    if (remove > cap) {
      uint64_t seen = 0;
      for (uint32_t i = 0; i < n; ++i)
        if (keep[i] == 0 && ++seen > cap) keep[i] = 1;
      remove = cap;
      CK(cudaMemcpyAsync(c->flags.p, keep.data(), (size_t)n * 4, cudaMemcpyHostToDevice, s));
    }
  }
  // applyPruneMask (gaussian-renderer.ts:2917-2925): nothing to do when no
  // Gaussian or every Gaussian would be removed.
  if (remove == 0 || remove >= n) return SKY_OK;
  TRY(compact_survivors(c, (const uint32_t*)c->flags.p, (uint32_t)(n - remove)));
  c->prune_runs += 1;
  if (removed) *removed = (uint32_t)remove;
  return SKY_OK;
}

extern "C" int sky_reset_opacity(void* p, float max_opacity) {
  Context* c = as_ctx(p);
  if (!c) return fail(SKY_ERR_ARG, "null context");
  if (!(max_opacity > 0.0f && max_opacity < 1.0f)) return fail(SKY_ERR_ARG, "max_opacity outside (0, 1)");
  if (c->n == 0) return SKY_OK;
  const float logit = (float)std::log((double)max_opacity / (1.0 - (double)max_opacity));
  launch_reset_opacity((float*)c->params.p, c->stride, c->n, logit, c->stream);
  CK(cudaGetLastError());
  CK(cudaStreamSynchronize(c->stream));
  return SKY_OK;
}

namespace sky {
// Sets the calling thread's sky_last_error() message; returns `code`.  Lets
// entry points defined in other translation units report errors.
int record_error(int code, const char* msg) {
  g_err = msg;
  return code;
}
}  // namespace sky
