// Hot-path kernels of the skyfall library: preprocess, scan, key emission,
// tile ranges, the tiled forward rasterizer with the fused loss, the tiled
// backward (exact and reference modes), and the fused geometry adjoint +
// Adam.  Sort lives in sort.cu.  See kernels.cuh for the launch interface.
#include "kernels.cuh"
#include "project.cuh"

#include <atomic>

namespace sky {
namespace {

constexpr uint32_t kFull = 0xFFFFFFFFu;

SKY_DEV float load_plane(const float* __restrict__ P, uint32_t stride, int plane, uint32_t g,
                         bool r16) {
  float v = __ldg(&P[(size_t)plane * stride + g]);
  return r16 ? round_f16(v) : v;
}

SKY_DEV float load_plane_rw(const float* P, uint32_t stride, int plane, uint32_t g, bool r16) {
  float v = P[(size_t)plane * stride + g];
  return r16 ? round_f16(v) : v;
}

// Asynchronous global -> shared copies (16 bytes through L2; 8 and 4 through
// L1), and their group fences.
SKY_DEV void cp_async16(void* smem, const void* gmem) {
  const uint32_t s = (uint32_t)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem) : "memory");
}
SKY_DEV void cp_async8(void* smem, const void* gmem) {
  const uint32_t s = (uint32_t)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(s), "l"(gmem) : "memory");
}
SKY_DEV void cp_async4(void* smem, const void* gmem) {
  const uint32_t s = (uint32_t)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(s), "l"(gmem) : "memory");
}
SKY_DEV void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
SKY_DEV void cp_async_wait1() { asm volatile("cp.async.wait_group 1;\n" ::: "memory"); }
SKY_DEV void cp_async_wait0() { asm volatile("cp.async.wait_group 0;\n" ::: "memory"); }

SKY_DEV int find_view(const StepParams& sp, uint32_t tile) {
  int v = 0;
  for (int k = 1; k < (int)sp.num_views; ++k)
    if (sp.views[k].tile_base <= tile) v = k;
  return v;
}

// Any error earlier in the step (capacity overflow, a sort that gave up, keys
// out of order) makes every later kernel of the step a no-op, so no kernel
// indexes with data that failed its checks.
SKY_DEV bool capacity_failed(const DevStatus* st) {
  return *(volatile const uint32_t*)&st->error != 0u;
}

// Raster pre-filter bound of a Gaussian with this opacity (see write_projection).
SKY_DEV float alpha_skip_bound(float opacity) { return __logf(255.0f * opacity) + 1e-3f; }

// The depth field of an intersection key: u32(clamp(depth, 0, 65535)) & 0xFFFF
// (encode_isect_key, training-tiles.wgsl:193-199).
SKY_DEV uint32_t depth_key(float depth) {
  return wgsl_u32(clampf_(depth, 0.0f, 65535.0f)) & 0xFFFFu;
}

// Tiles of an item's rectangle (packed as in b.rects).
SKY_DEV uint32_t rect_area(uint2 rc) {
  const uint32_t x0 = rc.x & 0xFFFFu, y0 = rc.x >> 16, x1 = rc.y & 0xFFFFu, y1 = rc.y >> 16;
  return (x1 <= x0 || y1 <= y0) ? 0u : (x1 - x0) * (y1 - y0);
}

// The ellipse E = {s <= L}, L = 1.001 smax, of a splat's raster pre-filter
// s = 0.5 (a dx^2 + c dy^2) + b dx dy <= smax, row by row, to skip tiles and
// pixel blocks where no pixel can pass it.  Relative to the mean, E's rows
// span |v| <= V = sqrt(2 a L / det) (det = a c - b^2), its rightmost point is
// (U, -b U / c) with U = sqrt(2 c L / det) (the leftmost the mirror image),
// and at height v it spans u in [(-b v - sqrt(D)) / a, (-b v + sqrt(D)) / a],
// D = 2 a L - det v^2.  Rounding: for a conic with b^2 <= 0.98 a c,
// |a dx^2| + |c dy^2| + 2 |b dx dy| <= 400 s, so the rasterisers' f32
// evaluation of s is within 3e-4 s of the exact value at their f32 offsets
// (dx, dy): every pixel that passes the pre-filter has those offsets inside E.
// Worse-conditioned conics (and smax <= 0) get no EllipseRows.
// Culled lists: an item whose rectangle has at most kSpanRows tile rows and
// at most 255 tile columns keeps its rows' spans (as the preprocess counted
// them) for the key emission, two bytes per row.
constexpr uint32_t kSpanRows = 8;

struct EllipseRows {
  float mx, my, a, b, det, two_a_l;
  float V, v_margin;  // V, and 1.01 V + 0.05: the rows listed
  float u_margin;     // 0.01 U + 0.05, added to each row's extent
  float v_right;      // -b U / c
};

// Square root and quotient of the ellipse arithmetic.  Tile lists and
// per-block masks only have to be conservative, so they take sqrt.approx
// (relative error below 2^-22) and the fast reciprocal division (2 ulp),
// errors far inside the margins above (the CPU tests check the extents with
// every square root and quotient moved adversarially by 2e-6).  The
// preprocess's counts and the emission's tiles come from the same code, so
// they agree bit for bit.
SKY_DEV float e_sqrt(float x) {
  float r;
  asm("sqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}
SKY_DEV float e_div(float x, float y) { return __fdividef(x, y); }

SKY_DEV bool ellipse_rows(float mx, float my, float a, float bq, float c, float smax, EllipseRows& r) {
  if (!(a > 0.0f) || !(c > 0.0f) || !(bq * bq <= 0.98f * (a * c)) || !(smax > 0.0f)) return false;
  const float L = 1.001f * smax;
  const float det = a * c - bq * bq;
  const float U = e_sqrt(e_div(2.0f * c * L, det));
  r.mx = mx;
  r.my = my;
  r.a = a;
  r.b = bq;
  r.det = det;
  r.two_a_l = 2.0f * a * L;
  r.V = e_sqrt(e_div(r.two_a_l, det));
  r.v_margin = 1.01f * r.V + 0.05f;
  r.u_margin = 0.01f * U + 0.05f;
  r.v_right = e_div(-bq * U, c);
  return true;
}

// E's extent [ul, ur] (relative to the mean, margins included) within a band
// of pixel-centre rows whose f32 dy run over [v0, v1] (the rasterisers' own
// dy at the band's first and last rows); false when the band misses E.  Over
// the band the right edge (-b v + sqrt(D)) / a is concave in v, so its
// maximum is at v_right clamped into the band, and the left edge's minimum at
// -v_right clamped likewise.  f32 error: det carries up to 6e-6 relative
// error (b^2 <= 0.98 a c), so D is within 6.2e-6 (2 a L) and each extent
// within 2.5e-3 U of the exact one; V within 1e-5 V.  The margins (1 % plus
// 0.05 px) cover that with room, so a pixel column outside [mx + ul, mx + ur]
// holds no pixel of the band that can pass the pre-filter; a column kept in
// excess only costs time.  A band that lies wholly beyond E's top or bottom
// row but within v_margin of it (w0 > w1) can only hold pixels that pass
// through that rounding, within 1e-5 V of the extreme row, so it gets the
// extent of that row (the tip -b v / a at v = +-V, plus the margins).
SKY_DEV bool band_extent(const EllipseRows& r, float v0, float v1, float& ul, float& ur) {
  if (v1 < -r.v_margin || v0 > r.v_margin) return false;
  const float w0 = fmaxf(v0, -r.V), w1 = fminf(v1, r.V);
  float vr, vl;
  if (w0 > w1) {
    vr = vl = v0 > 0.0f ? r.V : -r.V;
  } else {
    vr = fminf(fmaxf(r.v_right, w0), w1);
    vl = fminf(fmaxf(-r.v_right, w0), w1);
  }
  const float dr = fmaxf(r.two_a_l - r.det * vr * vr, 0.0f);
  const float dl = fmaxf(r.two_a_l - r.det * vl * vl, 0.0f);
  ur = e_div(-r.b * vr + e_sqrt(dr), r.a) + r.u_margin;
  ul = e_div(-r.b * vl - e_sqrt(dl), r.a) - r.u_margin;
  return true;
}

// Row ty's listed tiles [lo, lo + len) of the rectangle [x0, x1): those
// whose pixel-centre columns meet E's extent within the row's band.
SKY_DEV uint32_t row_span(const EllipseRows& r, uint32_t ty, uint32_t x0, uint32_t x1, uint32_t ts,
                          uint32_t& lo) {
  lo = x0;
  const float cy = (float)(ty * ts) + 0.5f;
  const float v0 = cy - r.my, v1 = (cy + (float)(ts - 1u)) - r.my;
  float ul, ur;
  if (!band_extent(r, v0, v1, ul, ur)) return 0u;
  // tiles whose centre columns [tx ts + 0.5, tx ts + ts - 0.5] meet [mx + ul, mx + ur]
  const float fts = (float)ts;
  const float t_lo = ceilf(e_div((r.mx + ul) - (fts - 0.5f), fts));
  const float t_hi = floorf(e_div((r.mx + ur) - 0.5f, fts));
  const float flo = fmaxf(t_lo, (float)x0), fhi = fminf(t_hi, (float)x1 - 1.0f);
  if (!(fhi >= flo)) return 0u;
  lo = (uint32_t)flo;
  return (uint32_t)fhi - lo + 1u;
}

// Writes the raster record, depth/radius, tile count, rectangle and item sort
// key (min(count, 0xFFFF) << 16) | depth16 of one item (the sort orders by the
// depth field; the count rides along for the scan in emission order);
// smax_g = alpha_skip_bound(o.opacity), the same for every view.  With
// tile_cull the count is that of the rectangle's tiles in the row spans of
// the splat's ellipse (row_span; all of them for a conic the test cannot
// bound, none when smax <= 0), and k_emit lists those same tiles; the
// rectangle is kept.
SKY_DEV void write_projection(const DevBuffers& b, const ProjOut& o, bool ok, float smax_g,
                              size_t item) {
  // Raster pre-filter: a pair with s > smax has opacity * exp(-s) < 1/255
  // whatever the rounding of exp (|error| < 1e-6 << 1e-3), so skipping it
  // there decides as the reference does.  The pixels with s <= smax lie in
  // the ellipse d^T conic d <= 2 smax, whose bounding box has half-widths
  // sqrt(2 smax cov00), sqrt(2 smax cov11).  The f32 evaluation of s has a
  // relative error below 20 ulp x cond(conic) <= 0.12 (cond <= 1e5 because
  // eps2d >= 0.3 and radius <= 512), so the box is computed for
  // 1.25 smax + 0.01: no pixel it excludes can pass the alpha test.
  float smax = -1.0f, hx = -1.0f, hy = -1.0f;
  if (ok) {
    smax = smax_g;
    if (smax > 0.0f) {
      const float sb = 2.0f * (1.25f * smax + 0.01f);
      hx = e_sqrt(sb * o.cov00) + 0.01f;  // (only masks read the box: 25 % margin)
      hy = e_sqrt(sb * o.cov11) + 0.01f;
    }
  }
  float4* rec = b.records + item * 3;
  rec[0] = make_float4(o.mx, o.my, o.ca, o.cb);
  rec[1] = make_float4(o.cc, o.opacity, o.col[0], o.col[1]);
  rec[2] = make_float4(o.col[2], smax, hx, hy);
  uint32_t count = o.count;
  const StepParams& sp = *b.sp;
  if (sp.tile_cull && count > 0u) {
    EllipseRows e;
    if (!(smax > 0.0f)) {
      count = 0u;
    } else if (ellipse_rows(o.mx, o.my, o.ca, o.cb, o.cc, smax, e)) {
      count = 0u;
      const bool keep = o.y1 - o.y0 <= kSpanRows && o.x1 - o.x0 <= 255u;
      uint32_t w[4] = {0u, 0u, 0u, 0u};
#pragma unroll
      for (uint32_t r = 0; r < kSpanRows; ++r) {
        const uint32_t ty = o.y0 + r;
        if (ty >= o.y1) break;
        uint32_t lo;
        const uint32_t len = row_span(e, ty, o.x0, o.x1, sp.tile_size, lo);
        count += len;
        w[r >> 1] |= ((lo - o.x0) | (len << 8)) << (16u * (r & 1u));
      }
      if (keep) {
        b.rowspans[item] = make_uint4(w[0], w[1], w[2], w[3]);
      } else {
        uint32_t lo;
        for (uint32_t ty = o.y0 + kSpanRows; ty < o.y1; ++ty)
          count += row_span(e, ty, o.x0, o.x1, sp.tile_size, lo);
      }
    }
  }
  b.aux[item] = make_float2(o.depth, o.radius);
  b.counts[item] = count;
  b.rects[item] = make_uint2(o.x0 | (o.y0 << 16), o.x1 | (o.y1 << 16));
  b.ikeys[item] = (min(count, 0xFFFFu) << 16) | depth_key(o.depth);
}

// ---------------------------------------------------------------------------
// Preprocess: one thread per Gaussian; its parameters are read (and rounded
// to f16) once and projected into every view of the step.
// ---------------------------------------------------------------------------
// The SH coefficients live in shared memory (one column per thread,
// conflict-free), the 11 geometry parameters in registers: 8 CTAs of 128
// threads per multiprocessor.
constexpr int kPrepThreads = 128;
__global__ void __launch_bounds__(kPrepThreads, 8) k_preprocess(DevBuffers b) {
  __shared__ float s_sh[48][kPrepThreads];
  extern __shared__ ViewInfo s_views[];  // the step's cameras (num_views)
  const StepParams& sp = *b.sp;
  {
    uint32_t dyn;
    asm("mov.u32 %0, %%dynamic_smem_size;" : "=r"(dyn));
    if (sp.num_views * (uint32_t)sizeof(ViewInfo) > dyn) {  // launched for fewer views
      if (threadIdx.x == 0) atomicOr(&b.status->error, SKY_DEVERR_CAPACITY);
      return;
    }
    const uint32_t words = sp.num_views * (uint32_t)(sizeof(ViewInfo) / 4);
    const uint32_t* src = reinterpret_cast<const uint32_t*>(sp.views);
    uint32_t* dst = reinterpret_cast<uint32_t*>(s_views);
    for (uint32_t i = threadIdx.x; i < words; i += blockDim.x) dst[i] = src[i];
  }
  __syncthreads();
  const int t = threadIdx.x;
  const uint32_t g = blockIdx.x * blockDim.x + t;
  if (g >= sp.n) return;
  const bool r16 = sp.round_f16 != 0;
  const uint32_t stride = sp.plane_stride;
  const int deg = (int)sp.sh_deg;
  const int nsh = 3 * (deg + 1) * (deg + 1);
  // the SH coefficients go to this thread's column of s_sh by asynchronous
  // copies, all in flight at once and holding no registers (loads into
  // registers would have to be stored in groups of a few), then rounded in
  // place
#pragma unroll
  for (int k = 0; k < 48; ++k) {
    if (k < nsh) cp_async4(&s_sh[k][t], &b.params[(size_t)(11 + k) * stride + g]);
    else s_sh[k][t] = 0.0f;
  }
  cp_async_commit();
  float prm[11];
#pragma unroll
  for (int k = 0; k < 11; ++k) prm[k] = load_plane(b.params, stride, k, g, r16);
  cp_async_wait0();
  if (r16) {
#pragma unroll
    for (int k = 0; k < 48; ++k) s_sh[k][t] = round_f16(s_sh[k][t]);
  }
  auto get = [&](int plane) { return plane < 11 ? prm[plane] : s_sh[plane - 11][t]; };
  // the covariance, opacity and skip bound do not depend on the view
  GaussCov3 gc;
  gauss_cov3(get, gc);
  const float smax_g = alpha_skip_bound(gc.opacity);
  for (uint32_t v = 0; v < sp.num_views; ++v) {
    const ViewInfo& vi = s_views[v];
    ProjOut o;
    const bool ok = project_gaussian(get, gc, vi, sp, deg, true, o);
    const size_t item = (size_t)v * sp.n + g;
    write_projection(b, o, ok, smax_g, item);
  }
}

// ---------------------------------------------------------------------------
// Scan of the tile counts (reduce, scan of block sums, scan + add).
// ---------------------------------------------------------------------------
constexpr int kScanThreads = 256;
constexpr int kScanItems = 16;
constexpr int kScanTile = kScanThreads * kScanItems;

SKY_DEV uint32_t block_excl_scan(uint32_t x, uint32_t* s_warp, uint32_t& total) {
  const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t y = x;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    uint32_t t = __shfl_up_sync(kFull, y, o);
    if (lane >= (uint32_t)o) y += t;
  }
  if (lane == 31) s_warp[warp] = y;
  __syncthreads();
  uint32_t add = 0, tot = 0;
  const uint32_t nw = blockDim.x >> 5;
  for (uint32_t w = 0; w < nw; ++w) {
    if (w < warp) add += s_warp[w];
    tot += s_warp[w];
  }
  total = tot;
  __syncthreads();
  return y - x + add;
}

// Count at scan position i: the counts are scanned in perm order when a
// permutation is given, read from the sorted item keys (which carry them up
// to 0xFFFF; larger ones are gathered).
SKY_DEV uint32_t scan_count(const DevBuffers& b, uint32_t i) {
  if (!b.perm) return b.counts[i];
  const uint32_t c = b.ikeys_sorted[i] >> 16;
  return c < 0xFFFFu ? c : b.counts[b.perm[i]];
}

// A scan of a step (b.status set) after a sort that gave up does nothing:
// the permutation may hold stale words, which must not be used as indices.
SKY_DEV bool scan_skipped(const DevBuffers& b) { return b.status && capacity_failed(b.status); }

__global__ void __launch_bounds__(kScanThreads) k_scan_reduce(DevBuffers b, uint32_t n_items) {
  __shared__ uint32_t s_warp[kScanThreads / 32];
  if (scan_skipped(b)) return;
  const uint32_t base = blockIdx.x * kScanTile;
  uint32_t sum = 0;
  for (int k = 0; k < kScanItems; ++k) {
    uint32_t i = base + k * kScanThreads + threadIdx.x;
    if (i < n_items) sum += scan_count(b, i);
  }
  uint32_t total;
  block_excl_scan(sum, s_warp, total);
  if (threadIdx.x == 0) b.block_sums[blockIdx.x] = total;
}

__global__ void __launch_bounds__(1024) k_scan_blocks(DevBuffers b, uint32_t nblocks) {
  __shared__ uint32_t s_warp[32];
  if (scan_skipped(b)) return;
  uint32_t carry = 0;
  for (uint32_t base = 0; base < nblocks; base += 1024) {
    uint32_t i = base + threadIdx.x;
    uint32_t v = i < nblocks ? b.block_sums[i] : 0u;
    uint32_t total;
    uint32_t ex = block_excl_scan(v, s_warp, total);
    if (i < nblocks) b.block_sums[i] = carry + ex;
    carry += total;
  }
}

__global__ void __launch_bounds__(kScanThreads) k_scan_final(DevBuffers b, uint32_t n_items) {
  __shared__ uint32_t s_warp[kScanThreads / 32];
  if (scan_skipped(b)) return;
  const uint32_t base = blockIdx.x * kScanTile + threadIdx.x * kScanItems;
  uint32_t v[kScanItems], pi[kScanItems];
  uint32_t sum = 0;
#pragma unroll
  for (int k = 0; k < kScanItems; ++k) {
    uint32_t i = base + k;
    v[k] = i < n_items ? scan_count(b, i) : 0u;
    // the items of the scatter below, loaded ahead: a load after a store
    // would wait for it (the arrays may alias as far as the compiler knows)
    pi[k] = (b.perm && i < n_items) ? b.perm[i] : 0u;
    sum += v[k];
  }
  uint32_t total;
  uint32_t run = block_excl_scan(sum, s_warp, total) + b.block_sums[blockIdx.x];
#pragma unroll
  for (int k = 0; k < kScanItems; ++k) {
    run += v[k];
    uint32_t i = base + k;
    if (i < n_items) {
      b.cumsum[i] = run;
      if (b.perm) b.item_end[pi[k]] = run;
    }
  }
}

// Group bounds of the sort segments and the capacity check.
// After an earlier error (the item sort gave up, so the scan was skipped)
// the step has no intersections: every group is empty.
__global__ void k_group_bounds(DevBuffers b) {
  const StepParams& sp = *b.sp;
  const uint32_t items = sp.num_views * sp.n;
  const bool failed = capacity_failed(b.status);
  const uint32_t total = (items && !failed) ? b.cumsum[items - 1] : 0u;
  if (threadIdx.x == 0) {
    b.status->total_isect = total;
    if (total > sp.icap) atomicOr(&b.status->error, SKY_DEVERR_CAPACITY);
  }
  for (uint32_t g = threadIdx.x; g < sp.num_groups; g += blockDim.x) {
    const GroupInfo& gi = sp.groups[g];
    uint32_t lo = (gi.item_begin && !failed) ? b.cumsum[gi.item_begin - 1] : 0u;
    uint32_t hi = (gi.item_end && !failed) ? b.cumsum[gi.item_end - 1] : 0u;
    b.status->group_bounds[g][0] = min(lo, sp.icap);
    b.status->group_bounds[g][1] = min(hi, sp.icap);
  }
}

// ---------------------------------------------------------------------------
// Key emission: (key_tile << 16) | depth16 in row-major tile order per item
// -- emit_intersections (training-tiles.wgsl:202-247) with a per-group tile
// field.  Items are emitted in perm order -- per sort group, by depth16, ties
// in (view, Gaussian) order -- not in (view, Gaussian) order.  A tile belongs
// to one view, so a stable sort of these keys on the tile field alone yields
// the order of the reference's stable sort of the full keys over (view,
// Gaussian) emission: within a tile by depth16, ties by Gaussian.
//
// One thread per item in item order, so every read is coalesced: the
// item's tile count, its emission end (scattered into item order by the
// scan), its depth field (the item key the preprocess wrote), its rectangle
// and, with culled lists, its record.  Each thread writes its item's
// contiguous range [end - count, end) of the emission order.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256, 6) k_emit(DevBuffers b) {
  const StepParams& sp = *b.sp;
  const uint32_t g = blockIdx.x * blockDim.x + threadIdx.x;
  const uint32_t v = blockIdx.y;
  if (g >= sp.n || v >= sp.num_views) return;
  if (capacity_failed(b.status)) return;  // item_end / cumsum are not to be trusted
  const uint32_t item = v * sp.n + g;
  // every load the item needs is issued before the first branch, so their
  // latencies overlap (most items are emitted)
  const uint32_t cnt = b.counts[item];  // the rectangle's area, or the culled count
  const uint32_t end = b.perm ? b.item_end[item] : b.cumsum[item];
  const uint32_t ikey = b.ikeys[item];
  const uint2 rc = b.rects[item];
  const uint4 spans = sp.tile_cull ? b.rowspans[item] : make_uint4(0u, 0u, 0u, 0u);
  if (cnt == 0u) return;
  if (end > sp.icap || cnt > end) {
    atomicOr(&b.status->error, SKY_DEVERR_LISTS);
    return;
  }
  const uint32_t dq = ikey & 0xFFFFu;  // depth16 (depth_key of the item's depth)
  const uint32_t x0 = rc.x & 0xFFFFu, y0 = rc.x >> 16, x1 = rc.y & 0xFFFFu, y1 = rc.y >> 16;
  const uint32_t area = (x1 <= x0 || y1 <= y0) ? 0u : (x1 - x0) * (y1 - y0);
  uint32_t cur = end - cnt;
  const ViewInfo& vi = sp.views[v];
  // the keys of tiles [lo, lo + len) of tile row ty; false: the row holds
  // more tiles than the item's range has left (lists counted differently)
  auto emit_row = [&](uint32_t ty, uint32_t lo, uint32_t len) {
    if (len > end - cur) return false;
    for (uint32_t tx = lo; tx < lo + len; ++tx) {
      const uint32_t kt = vi.key_tile_base + ty * vi.tiles_x + tx;
      b.keys[cur] = (kt << 16) | dq;
      b.rec_of[cur] = item;
      ++cur;
    }
    return true;
  };
  bool ok = true;
  if (cnt == area) {
    for (uint32_t ty = y0; ty < y1; ++ty) emit_row(ty, x0, x1 - x0);
    return;
  }
  // culled: the tiles the preprocess counted -- its row spans where it kept
  // them, else the same test on the same record values
  if (!sp.tile_cull) {
    ok = false;
  } else if (y1 - y0 <= kSpanRows && x1 - x0 <= 255u) {
    for (uint32_t r = 0; ok && r < y1 - y0; ++r) {
      const uint32_t wv = r < 2u ? spans.x : (r < 4u ? spans.y : (r < 6u ? spans.z : spans.w));
      const uint32_t h = (wv >> (16u * (r & 1u))) & 0xFFFFu;
      ok = emit_row(y0 + r, x0 + (h & 0xFFu), h >> 8);
    }
  } else {
    const float4 r0 = b.records[(size_t)item * 3 + 0];
    const float cc = b.records[(size_t)item * 3 + 1].x;
    const float smax = b.records[(size_t)item * 3 + 2].y;
    EllipseRows e;
    ok = ellipse_rows(r0.x, r0.y, r0.z, r0.w, cc, smax, e);
    for (uint32_t ty = y0; ok && ty < y1; ++ty) {
      uint32_t lo;
      const uint32_t len = row_span(e, ty, x0, x1, sp.tile_size, lo);
      ok = emit_row(ty, lo, len);
    }
  }
  // counted differently from the preprocess: corrupt lists
  if (!ok || cur != end) atomicOr(&b.status->error, SKY_DEVERR_LISTS);
}

// ---------------------------------------------------------------------------
// Tile ranges: offsets[t] = first sorted intersection of tile t, empty tiles
// take the start of the next non-empty one (build_tile_offsets +
// host backward min-fill, training-tiles.wgsl:250-271 and
// gaussian-renderer.ts:1966-2020).
//
// The item of each sorted intersection (flatten[i] = rec_of[vals_sorted[i]])
// is resolved by the forward as it stages a batch: every later reader in the
// exact mode (backward, multi-view scores) stays within each tile's staged
// batches, since a pixel's last contributor lies in them.  The
// reference-mode backward walks every list to its end, so for it this kernel
// resolves them all; a read-back of the buffer completes it (flatten_fill).
// ---------------------------------------------------------------------------
// Grid-stride over chunks of four sorted intersections (one 16-byte key
// load where the chunk lies inside the group; the key before the chunk comes
// from the cache line the neighbouring thread loaded); the grid is sized for
// the capacity's order of magnitude, not the capacity itself.  The sort
// groups' bounds and tile ranges are read once per block into shared memory,
// and each group's chunks are walked within its bounds (a chunk straddling
// two groups is split).  Each group writes offsets[tile_end], the end of its
// last tile (the next group writes the same value there, the start of its
// first; the last group's is the final sentinel).
__global__ void __launch_bounds__(256) k_ranges(DevBuffers b) {
  __shared__ uint32_t s_gb[kMaxGroups][2];
  __shared__ uint32_t s_gt[kMaxGroups][2];
  const StepParams& sp = *b.sp;
  if (capacity_failed(b.status)) return;
  const int ng = (int)sp.num_groups;
  for (int k = (int)threadIdx.x; k < ng; k += (int)blockDim.x) {
    s_gb[k][0] = b.status->group_bounds[k][0];
    s_gb[k][1] = b.status->group_bounds[k][1];
    s_gt[k][0] = sp.groups[k].tile_begin;
    s_gt[k][1] = sp.groups[k].tile_end;
  }
  __syncthreads();
  const bool resolve = sp.bwd_mode != 0;
  for (int g = 0; g < ng; ++g) {
    const uint32_t gb = s_gb[g][0], ge = s_gb[g][1], tb = s_gt[g][0], te = s_gt[g][1];
    if (gb >= ge) continue;  // empty: k_ranges_empty
    const uint32_t c_lo = gb / 4u, c_hi = (ge + 3u) / 4u;
    for (uint32_t c = c_lo + blockIdx.x * blockDim.x + threadIdx.x; c < c_hi;
         c += gridDim.x * blockDim.x) {
      const uint32_t i0 = 4u * c;
      uint32_t kk[4];
      if (i0 >= gb && i0 + 4u <= ge) {
        const uint4 v = reinterpret_cast<const uint4*>(b.keys_sorted)[c];
        kk[0] = v.x; kk[1] = v.y; kk[2] = v.z; kk[3] = v.w;
      } else {
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          const uint32_t i = i0 + (uint32_t)j;
          kk[j] = (i >= gb && i < ge) ? b.keys_sorted[i] : 0u;
        }
      }
      uint32_t prev = i0 > gb ? b.keys_sorted[i0 - 1u] : 0u;
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const uint32_t i = i0 + (uint32_t)j;
        if (i < gb || i >= ge) continue;
        const uint32_t t = tb + (kk[j] >> 16);
        const uint32_t tp = tb + (prev >> 16);  // the key before, when in the group (i > gb)
        prev = kk[j];
        if (t >= te || (i > gb && tp > t)) {
          atomicOr(&b.status->error, SKY_DEVERR_LISTS);  // unsorted or corrupt keys
          return;
        }
        if (i == gb) {
          for (uint32_t u = tb; u <= t; ++u) b.offsets[u] = i;
        } else {
          for (uint32_t u = tp + 1; u <= t; ++u) b.offsets[u] = i;
        }
        if (i + 1 == ge)
          for (uint32_t u = t + 1; u <= te; ++u) b.offsets[u] = ge;
        if (resolve) b.flatten[i] = b.rec_of[b.vals_sorted[i]];
      }
    }
  }
}

// flatten[i] = rec_of[vals_sorted[i]] for every sorted intersection of the
// last step (the forward resolved only its staged batches); idempotent.
__global__ void __launch_bounds__(256) k_flatten_fill(DevBuffers b, uint32_t total) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < total; i += gridDim.x * blockDim.x) {
    const uint32_t e = b.vals_sorted[i];
    if (e < total) b.flatten[i] = b.rec_of[e];
  }
}

// Empty groups: every tile's range, and the group's offsets[tile_end], start
// at the group's bound.
__global__ void k_ranges_empty(DevBuffers b) {
  const StepParams& sp = *b.sp;
  if (capacity_failed(b.status)) return;
  for (uint32_t g = 0; g < sp.num_groups; ++g) {
    const uint32_t gb = b.status->group_bounds[g][0], ge = b.status->group_bounds[g][1];
    if (gb != ge) continue;
    const GroupInfo& gi = sp.groups[g];
    for (uint32_t u = gi.tile_begin + threadIdx.x; u <= gi.tile_end; u += blockDim.x)
      b.offsets[u] = gb;
  }
}

// ---------------------------------------------------------------------------
// Forward: training_tiled_forward (training-forward-tiles.wgsl:107-215), one
// CTA per tile, one thread per pixel, splat records staged in shared memory
// one batch of FB (the splat-batch depth: 64, 128 or 256) at a time,
// whole-CTA early exit once every pixel has reached the transmittance
// threshold.  The loss of training-loss.wgsl:86-126 (without its SSIM term)
// is fused into the epilogue.  The batch depth changes no result.
// ---------------------------------------------------------------------------
constexpr int kFwdBatch = 256;  // default splat-batch depth of the forward

// Bit w set when warp w of the tile (pixel rows [w * RPW, (w + 1) * RPW),
// RPW = 32/TS unless the warp's lanes hold several pixels) has a pixel centre
// inside the splat's alpha >= 1/255 bounding box (half-widths r2.z, r2.w
// around the mean r0.xy; negative = no pixel).
// Warps covering BW x BH pixel blocks of the tile, numbered row-major over
// the TS/BW x TS/BH block grid: bit w set when block w has a pixel centre in
// the splat's alpha >= 1/255 bounding box.
template <int TS, int BW, int BH>
SKY_DEV uint32_t block_mask(float4 r0, float4 r2, uint32_t x0, uint32_t y0) {
  constexpr int NCOL = TS / BW;
  const float hx = r2.z, hy = r2.w;
  if (!(hx > 0.0f) || !(hy > 0.0f)) return 0u;
  const float xlo = r0.x - hx - (float)x0 - 0.5f, xhi = r0.x + hx - (float)x0 - 0.5f;
  const float ylo = r0.y - hy - (float)y0 - 0.5f, yhi = r0.y + hy - (float)y0 - 0.5f;
  if (!(xhi >= 0.0f) || !(xlo <= (float)(TS - 1))) return 0u;
  if (!(yhi >= 0.0f) || !(ylo <= (float)(TS - 1))) return 0u;
  const int clo = xlo <= 0.0f ? 0 : (int)ceilf(xlo);
  const int chi = xhi >= (float)(TS - 1) ? TS - 1 : (int)floorf(xhi);
  const int rlo = ylo <= 0.0f ? 0 : (int)ceilf(ylo);
  const int rhi = yhi >= (float)(TS - 1) ? TS - 1 : (int)floorf(yhi);
  if (clo > chi || rlo > rhi) return 0u;
  const uint32_t cols = ((1u << (chi / BW + 1)) - 1u) & ~((1u << (clo / BW)) - 1u);
  uint32_t mask = 0u;
  for (int br = rlo / BH; br <= rhi / BH; ++br) mask |= cols << (br * NCOL);
  return mask;
}

// block_mask with the bounding box replaced by the ellipse itself, band by
// band (band_extent): per row of BW x BH blocks, E's x-extent within the
// row's BH pixel rows, and block c kept when its pixel-centre columns meet
// it.  A cleared bit means no pixel of the block can pass the raster
// pre-filter, so the block's warp would do nothing with the splat.
// Worse-conditioned conics keep the bounding-box mask.
template <int TS, int BW, int BH>
SKY_DEV uint32_t ellipse_band_mask(float4 r0, float4 r1, float4 r2, uint32_t x0, uint32_t y0) {
  constexpr int NCOL = TS / BW, NROW = TS / BH;
  const uint32_t m = block_mask<TS, BW, BH>(r0, r2, x0, y0);
  EllipseRows e;
  if (m == 0u || !ellipse_rows(r0.x, r0.y, r0.z, r0.w, r1.x, r2.y, e)) return m;
  uint32_t keep = 0u;
#pragma unroll 1
  for (int br = 0; br < NROW; ++br) {
    if (((m >> (br * NCOL)) & ((1u << NCOL) - 1u)) == 0u) continue;
    const float cy = (float)(y0 + (uint32_t)(br * BH)) + 0.5f;
    float ul, ur;
    if (!band_extent(e, cy - e.my, (cy + (float)(BH - 1)) - e.my, ul, ur)) continue;
    const float xl = e.mx + ul, xr = e.mx + ur;
#pragma unroll
    for (int bc = 0; bc < NCOL; ++bc) {
      const float cx = (float)(x0 + (uint32_t)(bc * BW)) + 0.5f;
      if (xr >= cx && xl <= cx + (float)(BW - 1)) keep |= 1u << (br * NCOL + bc);
    }
  }
  return m & keep;
}

template <int TS, int RPW = 32 / TS>
SKY_DEV uint32_t warp_mask(float4 r0, float4 r2, uint32_t x0, uint32_t y0) {
  const float hx = r2.z, hy = r2.w;
  if (!(hx > 0.0f) || !(hy > 0.0f)) return 0u;
  const float cx0 = (float)x0 + 0.5f, cx1 = (float)x0 + ((float)TS - 0.5f);
  if (cx1 < r0.x - hx || cx0 > r0.x + hx) return 0u;
  const float ylo = r0.y - hy - (float)y0 - 0.5f;  // rows r with r >= ylo ...
  const float yhi = r0.y + hy - (float)y0 - 0.5f;  // ... and r <= yhi
  if (!(yhi >= 0.0f) || !(ylo <= (float)(TS - 1))) return 0u;
  const int rlo = ylo <= 0.0f ? 0 : (int)ceilf(ylo);
  const int rhi = yhi >= (float)(TS - 1) ? TS - 1 : (int)floorf(yhi);
  if (rlo > rhi) return 0u;
  const int wlo = rlo / RPW, whi = rhi / RPW;
  const uint32_t upto = whi >= 31 ? 0xFFFFFFFFu : ((1u << (whi + 1)) - 1u);
  return upto & ~((1u << wlo) - 1u);
}

// A raster record as the tiled kernels keep it in shared memory: the conic's
// a and c halved, so that (a/2 dx) dx + (c/2 dy) dy is the reference's
// 0.5 (a dx^2 + c dy^2) bit for bit (halving is exact, and for the emitted
// conics, a, c >= 1e-6 and |dx|, |dy| = 0 or >= 2^-26, no product comes near
// the subnormal range), one multiply fewer per pixel and splat.
SKY_DEV void stage_record(float4* dst, const float4& q0, const float4& q1, const float4& q2) {
  dst[0] = make_float4(q0.x, q0.y, 0.5f * q0.z, q0.w);
  dst[1] = make_float4(0.5f * q1.x, q1.y, q1.z, q1.w);
  dst[2] = q2;
}

// !(0 <= s <= smax) for smax > 0 (every listed splat's) in one unsigned
// compare: a negative s has the sign bit set, and s is never -0 (it is
// (+0 or positive) + (b dx) dy, and +0 + -0 = +0).
SKY_DEV bool outside_smax(float s, float smax) { return __float_as_uint(s) > __float_as_uint(smax); }

// Warp sums of the counting variants' per-lane tallies of evaluated and
// contributing pairs, and lane 0's count of the warp's list entries, added
// to the step's status counters pairs[base..base+2].
SKY_DEV void add_pair_counts(const DevBuffers& b, int base, uint32_t eval, uint32_t contrib,
                             uint32_t entries) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    eval += __shfl_xor_sync(kFull, eval, o);
    contrib += __shfl_xor_sync(kFull, contrib, o);
  }
  if ((threadIdx.x & 31) == 0) {
    atomicAdd(&b.status->pairs[base + 0], (unsigned long long)eval);
    atomicAdd(&b.status->pairs[base + 1], (unsigned long long)contrib);
    atomicAdd(&b.status->pairs[base + 2], (unsigned long long)entries);
  }
}

// CNT: the counting variant (profiling level 2) also tallies the pairs it
// evaluates and composites and the list entries its warps walk; the
// arithmetic and every result are those of the plain variant.
template <int TS, int FB, bool CNT = false>
__global__ void __launch_bounds__(TS* TS, TS == 16 ? 6 : 1) k_forward(DevBuffers b) {
  static_assert(FB <= 256, "list entries are bytes");
  constexpr int NT = TS * TS;
  constexpr int NW = NT / 32;
  __shared__ float4 s_rec[FB * 3];
  __shared__ uint32_t s_mask[FB];
  __shared__ uint8_t s_list[NW][FB];
  __shared__ double s_loss[NW];
  __shared__ float4 s_tgt[NT];  // this thread's target pixel, copied in during the loop
  const StepParams& sp = *b.sp;
  const uint32_t tile = blockIdx.x;
  if (tile >= sp.num_tiles) return;
  if (capacity_failed(b.status)) return;
  const int v = find_view(sp, tile);
  const ViewInfo& vi = sp.views[v];
  const uint32_t local = tile - vi.tile_base;
  const uint32_t tx = local % vi.tiles_x, ty = local / vi.tiles_x;
  const uint32_t tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  // warp w covers the 8x4 pixel block (w % (TS/8), w / (TS/8)) of the tile:
  // compact blocks meet fewer splats than full-width strips
  const uint32_t x = tx * TS + 8u * (warp % (TS / 8)) + (lane & 7u);
  const uint32_t y = ty * TS + 4u * (warp / (TS / 8)) + (lane >> 3);
  const bool inside = x < vi.width && y < vi.height;
  const uint32_t start = b.offsets[tile], end = b.offsets[tile + 1];
  const float pxf = (float)x + 0.5f, pyf = (float)y + 0.5f;
  const bool want_tgt = inside && sp.has_loss && vi.has_target;
  if (want_tgt) cp_async16(&s_tgt[tid], &b.targets[(size_t)vi.target_base + (size_t)y * vi.width + x]);
  cp_async_commit();
  float C0 = 0.0f, C1 = 0.0f, C2 = 0.0f, A = 0.0f, Tp = 1.0f;
  // the reference's loop visits every intersection of the tile up to the
  // one that ends it (training-forward-tiles.wgsl:168-207)
  uint32_t last = end - 1;
  bool done = !inside;
  const uint32_t wbit = 1u << warp;
  const uint32_t lt = (1u << lane) - 1u;
  uint32_t n_eval = 0, n_contrib = 0, n_entries = 0;  // counting variant only
  for (uint32_t bs = start; bs < end; bs += FB) {
    const uint32_t cnt = min((uint32_t)FB, end - bs);
    __syncthreads();
    for (uint32_t k = tid; k < cnt; k += NT) {
      // the batch's items, resolved here for the later readers (k_ranges)
      const uint32_t item = b.rec_of[b.vals_sorted[bs + k]];
      b.flatten[bs + k] = item;
      const size_t r = item;
      const float4 q0 = b.records[r * 3 + 0];
      const float4 q1 = b.records[r * 3 + 1];
      const float4 q2 = b.records[r * 3 + 2];
      stage_record(s_rec + k * 3, q0, q1, q2);
      const uint32_t m = ellipse_band_mask<TS, 8, 4>(q0, q1, q2, tx * TS, ty * TS);
      s_mask[k] = m;
      if constexpr (TS == 16) b.fmask[bs + k] = (uint8_t)m;  // for the 16x16 backward
    }
    __syncthreads();
    // this warp's splats of the batch, in order (skipped splats cannot pass
    // the alpha test at any pixel of the warp)
    uint32_t nlist = 0;
    const bool warp_live = !__all_sync(kFull, done);  // a finished warp lists nothing
    for (uint32_t base = 0; warp_live && base < cnt; base += 32) {
      const uint32_t j = base + lane;
      const bool in = j < cnt && (s_mask[j] & wbit);
      const uint32_t m = __ballot_sync(kFull, in);
      if (in) s_list[warp][nlist + __popc(m & lt)] = (uint8_t)j;
      nlist += __popc(m);
    }
    __syncwarp();
    if constexpr (CNT) n_entries += nlist;
    if (!done) {
      for (uint32_t li = 0; li < nlist; ++li) {
        const uint32_t j = s_list[warp][li];
        const float4 r0 = s_rec[j * 3 + 0];
        const float4 r2 = s_rec[j * 3 + 2];
        const float dx = pxf - r0.x, dy = pyf - r0.y;
        const float s1 = (r0.z * dx) * dx;  // halved conic: s1 + s2 = 0.5 (a dx^2 + c dy^2)
        const float4 r1 = s_rec[j * 3 + 1];
        const float s2 = (r1.x * dy) * dy;
        float so2 = s1 + s2;
        so2 = so2 + (r0.w * dx) * dy;
        if constexpr (CNT) ++n_eval;
        if (outside_smax(so2, r2.y)) continue;
        // emitted records have finite means and conics, so 0 <= s <= s_max
        const float G = sky_expf_inrange(-so2);
        const float al = r1.y * G;
        const float a = fmin_(al, MAX_ALPHA);
        if (a < MIN_ALPHA) continue;
        if constexpr (CNT) ++n_contrib;
        const float om = 1.0f - A;
        const float ca = a * om;
        C0 = C0 + r1.z * ca;
        C1 = C1 + r1.w * ca;
        C2 = C2 + r2.x * ca;
        A = A + ca;
        Tp = Tp * (1.0f - a);
        if (1.0f - A < T_THRESH) {
          last = bs + j;
          done = true;
          break;
        }
      }
    }
    if (__syncthreads_and(done)) break;
  }
  if constexpr (CNT) add_pair_counts(b, 0, n_eval, n_contrib, n_entries);
  double lpx = 0.0;
  if (inside) {
    const size_t p = (size_t)vi.pixel_base + (size_t)y * vi.width + x;
    const float T = 1.0f - A;
    const float o0 = C0 + T * sp.bg[0], o1 = C1 + T * sp.bg[1], o2 = C2 + T * sp.bg[2];
    if (start >= end) last = 0xFFFFFFFFu;
    b.color[p] = make_float4(o0, o1, o2, 1.0f);
    b.alpha[p] = A;
    b.tfinal[p] = Tp;
    b.last[p] = last;
    cp_async_wait0();
    if (want_tgt) {
      const float4 tg = s_tgt[tid];
      const float d0 = o0 - tg.x, d1 = o1 - tg.y, d2 = o2 - tg.z;
      auto sgn = [](float d) { return d > 0.0f ? 1.0f : (d < 0.0f ? -1.0f : 0.0f); };
      const float g0 = sp.w_l2 * d0 + sp.w_l1 * sgn(d0);
      const float g1 = sp.w_l2 * d1 + sp.w_l1 * sgn(d1);
      const float g2 = sp.w_l2 * d2 + sp.w_l1 * sgn(d2);
      b.residual[p] = make_float4(g0, g1, g2, 0.0f);
      const double hl2 = 0.5 * (double)sp.w_l2, wl1 = (double)sp.w_l1;
      lpx = hl2 * (double)d0 * (double)d0 + wl1 * fabs((double)d0);
      lpx += hl2 * (double)d1 * (double)d1 + wl1 * fabs((double)d1);
      lpx += hl2 * (double)d2 * (double)d2 + wl1 * fabs((double)d2);
    }
  }
  if (sp.has_loss) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) lpx += __shfl_xor_sync(kFull, lpx, o);
    if ((tid & 31) == 0) s_loss[tid >> 5] = lpx;
    __syncthreads();
    if (tid == 0) {
      double s = 0.0;
      for (int w = 0; w < NT / 32; ++w) s += s_loss[w];
      b.loss_partials[tile] = s;
    }
  }
}

// SSIM pseudo-gradient term (training-loss.wgsl:33-84), added to the
// residual after the forward when w_ssim > 0.  One thread per pixel of the
// step (grid-stride over views).
__global__ void __launch_bounds__(256) k_ssim(DevBuffers b) {
  const StepParams& sp = *b.sp;
  if (capacity_failed(b.status)) return;
  const uint32_t v = blockIdx.y;
  if (v >= sp.num_views) return;
  const ViewInfo& vi = sp.views[v];
  if (!vi.has_target) return;
  const uint32_t np = vi.width * vi.height;
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= np) return;
  const int W = (int)vi.width, H = (int)vi.height;
  const int x = (int)(i % vi.width), y = (int)(i / vi.width);
  auto P = [&](int xx, int yy) {
    xx = min(max(xx, 0), W - 1);
    yy = min(max(yy, 0), H - 1);
    return b.color[(size_t)vi.pixel_base + (size_t)yy * W + xx];
  };
  auto Tg = [&](int xx, int yy) {
    xx = min(max(xx, 0), W - 1);
    yy = min(max(yy, 0), H - 1);
    return b.targets[(size_t)vi.target_base + (size_t)yy * W + xx];
  };
  const float C1 = 0.0001f, C2 = 0.0009f, nwin = 25.0f;  // f32(0.01^2), f32(0.03^2)
  float out[3];
  for (int c = 0; c < 3; ++c) {
    auto comp = [c](float4 f) { return c == 0 ? f.x : (c == 1 ? f.y : f.z); };
    float mx = 0.0f, my = 0.0f;
    for (int dy = -2; dy <= 2; ++dy)
      for (int dx = -2; dx <= 2; ++dx) {
        mx = mx + comp(P(x + dx, y + dy));
        my = my + comp(Tg(x + dx, y + dy));
      }
    mx = mx / nwin;
    my = my / nwin;
    float sx = 0.0f, sy = 0.0f, sxy = 0.0f;
    for (int dy = -2; dy <= 2; ++dy)
      for (int dx = -2; dx <= 2; ++dx) {
        float a = comp(P(x + dx, y + dy)) - mx;
        float bb = comp(Tg(x + dx, y + dy)) - my;
        sx = sx + a * a;
        sy = sy + bb * bb;
        sxy = sxy + a * bb;
      }
    sx = sx / nwin;
    sy = sy / nwin;
    sxy = sxy / nwin;
    float num1 = (2.0f * mx) * my + C1;
    float num2 = 2.0f * sxy + C2;
    float den1 = (mx * mx + my * my) + C1;
    float den2 = (sx + sy) + C2;
    float ssim = (num1 * num2) / (den1 * den2);
    float dssim = (1.0f - ssim) * 0.5f;
    out[c] = dssim * (comp(P(x, y)) - comp(Tg(x, y)));
  }
  const size_t p = (size_t)vi.pixel_base + i;
  float4 r = b.residual[p];
  r.x = r.x + sp.w_ssim * out[0];
  r.y = r.y + sp.w_ssim * out[1];
  r.z = r.z + sp.w_ssim * out[2];
  b.residual[p] = r;
}

__global__ void __launch_bounds__(1024) k_loss_final(DevBuffers b) {
  __shared__ double s[32];
  const StepParams& sp = *b.sp;
  double acc = 0.0;
  // fixed assignment of tiles to threads, then a fixed tree; a thread's
  // partials are loaded 16 at a time and added in order (one load, one add
  // after another would wait on every load)
  constexpr uint32_t kAhead = 16;
  const uint32_t nt = sp.num_tiles, step = blockDim.x;
  uint32_t t = threadIdx.x;
  for (; t + (kAhead - 1) * step < nt; t += kAhead * step) {
    double v[kAhead];
#pragma unroll
    for (uint32_t k = 0; k < kAhead; ++k) v[k] = b.loss_partials[t + k * step];
#pragma unroll
    for (uint32_t k = 0; k < kAhead; ++k) acc += v[k];
  }
  for (; t < nt; t += step) acc += b.loss_partials[t];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(kFull, acc, o);
  if ((threadIdx.x & 31) == 0) s[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += s[w];
    b.status->loss = t;
  }
}

// ---------------------------------------------------------------------------
// Backward, exact mode.  One CTA per tile; each pixel walks its composited
// splats back to front from its last contributor, recomputing transmittance
// from the final product transmittance (T_before = T / (1 - alpha); the
// product keeps relative precision where 1 - alpha_final would cancel); per
// pair it forms the nine quantities of backward-tiles-local.wgsl:333-359
// (dL/dcolour replaces the 48 SH products: the SH chain is applied once per
// Gaussian later).  A warp skips a splat whose alpha >= 1/255 box misses all
// of its pixels or that lies beyond all of its pixels' last contributors.
// Each batch's per-pair values are reduced over the warp by a fixed
// reduce-scatter (12 shuffles for 9 values; column first, 10 shuffles, in
// the 16x16 kernel), then over the warps in index order, and written per
// intersection to partials[emission index] -- so every Gaussian's partials
// are contiguous and the later per-Gaussian sum has a fixed order.
// ---------------------------------------------------------------------------

// Sum of v[0..8] over the warp, scattered: on return the lane with bit 0
// clear and slot() == k holds the warp total of v[k] (slot() >= 9: none).
SKY_DEV float warp_reduce_scatter9(const float v[9], uint32_t lane) {
  const bool b4 = lane & 16u, b3 = lane & 8u, b2 = lane & 4u, b1 = lane & 2u;
  float w[5];
#pragma unroll
  for (int i = 0; i < 5; ++i) {
    const float lo = v[i], hi = (i + 5 < 9) ? v[i + 5] : 0.0f;
    w[i] = (b4 ? hi : lo) + __shfl_xor_sync(kFull, b4 ? lo : hi, 16);
  }
  float x3[3];
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    const float lo = w[i], hi = (i + 3 < 5) ? w[i + 3] : 0.0f;
    x3[i] = (b3 ? hi : lo) + __shfl_xor_sync(kFull, b3 ? lo : hi, 8);
  }
  float y2[2];
#pragma unroll
  for (int i = 0; i < 2; ++i) {
    const float lo = x3[i], hi = (i + 2 < 3) ? x3[i + 2] : 0.0f;
    y2[i] = (b2 ? hi : lo) + __shfl_xor_sync(kFull, b2 ? lo : hi, 4);
  }
  float z = (b1 ? y2[1] : y2[0]) + __shfl_xor_sync(kFull, b1 ? y2[0] : y2[1], 2);
  return z + __shfl_xor_sync(kFull, z, 1);
}

// The partial of a sorted intersection, at its emission index e, flagged in
// b.reached; one whose nine sums are all zero is not written (it counts as
// zero, like the intersections no pixel reaches).
SKY_DEV void write_partial(const DevBuffers& b, uint32_t e, const float sum[9], float dlogit, float dca,
                           float dcb, float dcc, float dmx, float dmy) {
  bool nz = false;
#pragma unroll
  for (int k = 0; k < 9; ++k) nz = nz || sum[k] != 0.0f;
  if (!nz) return;
  float4* dst = b.partials + (size_t)e * kPartialF4;
  dst[0] = make_float4(sum[0], sum[1], sum[2], dlogit);
  dst[1] = make_float4(dca, dcb, dcc, dmx);
  dst[2] = make_float4(dmy, 0.0f, 0.0f, 0.0f);
  b.reached[e] = 1u;
}

// Value index a lane holds after warp_reduce_scatter9, or 9 for none.
SKY_DEV int scatter9_slot(uint32_t lane) {
  if (lane & 1u) return 9;
  const int xi = (int)(((lane >> 2) & 1u) * 2 + ((lane >> 1) & 1u));  // x3 index, 3 = pad
  if (xi >= 3) return 9;
  const int wi = (int)((lane >> 3) & 1u) * 3 + xi;                     // w index, >= 5 = pad
  if (wi >= 5) return 9;
  const int vi = (int)((lane >> 4) & 1u) * 5 + wi;
  return vi < 9 ? vi : 9;
}

template <int TS>
__global__ void __launch_bounds__(TS* TS) k_backward_exact(DevBuffers b) {
  constexpr int NT = TS * TS;
  constexpr int NW = NT / 32;
  constexpr int kBwdBatch = NW <= 8 ? 64 : 16;
  __shared__ float4 s_rec[kBwdBatch * 3];
  __shared__ uint32_t s_mask[kBwdBatch];
  __shared__ float s_part[NW][kBwdBatch][9];
  __shared__ int s_hi[NW];
  __shared__ uint8_t s_list[NW][kBwdBatch];
  const StepParams& sp = *b.sp;
  const uint32_t tile = blockIdx.x;
  if (tile >= sp.num_tiles) return;
  if (capacity_failed(b.status)) return;
  const uint32_t start = b.offsets[tile], end = b.offsets[tile + 1];
  if (start >= end) return;
  const int v = find_view(sp, tile);
  const ViewInfo& vi = sp.views[v];
  const uint32_t local = tile - vi.tile_base;
  const uint32_t tx = local % vi.tiles_x, ty = local / vi.tiles_x;
  const uint32_t tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const uint32_t x = tx * TS + (tid % TS), y = ty * TS + (tid / TS);
  const bool inside = x < vi.width && y < vi.height;
  float T = 1.0f, acc0 = sp.bg[0], acc1 = sp.bg[1], acc2 = sp.bg[2];
  float r0 = 0.0f, r1 = 0.0f, r2 = 0.0f;
  int myhi = (int)start - 1;
  const float pxf = (float)x + 0.5f, pyf = (float)y + 0.5f;
  if (inside) {
    const size_t p = (size_t)vi.pixel_base + (size_t)y * vi.width + x;
    const uint32_t lst = b.last[p];
    if (lst >= start) myhi = (int)min(lst, end - 1);
    T = b.tfinal[p];
    const float4 rs = b.residual[p];
    r0 = rs.x; r1 = rs.y; r2 = rs.z;
  }
  int whi = myhi;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) whi = max(whi, __shfl_xor_sync(kFull, whi, o));
  if (lane == 0) s_hi[warp] = whi;
  __syncthreads();
  int hi = s_hi[0];
  for (int w = 1; w < NW; ++w) hi = max(hi, s_hi[w]);
  const int slot = scatter9_slot(lane);
  const uint32_t wbit = 1u << warp;
  const uint32_t lt = (1u << lane) - 1u;
  // intersections beyond every pixel's last contributor are not written:
  // their emission slots stay unflagged in b.reached and count as zero
  for (int bhi = hi; bhi >= (int)start; bhi -= kBwdBatch) {
    const int cnt = min(kBwdBatch, bhi - (int)start + 1);
    __syncthreads();
    for (int k = (int)tid; k < cnt; k += NT) {
      const size_t r = b.flatten[bhi - k];
      const float4 q0 = b.records[r * 3 + 0];
      const float4 q2 = b.records[r * 3 + 2];
      s_rec[k * 3 + 0] = q0;
      s_rec[k * 3 + 1] = b.records[r * 3 + 1];
      s_rec[k * 3 + 2] = q2;
      s_mask[k] = warp_mask<TS>(q0, q2, tx * TS, ty * TS);
    }
    __syncthreads();
    // this warp's splats of the batch (box overlaps a pixel of the warp and
    // some pixel of the warp has not stopped before it), back to front
    uint32_t nlist = 0;
    for (int base = 0; base < cnt; base += 32) {
      const int j = base + (int)lane;
      const bool in = j < cnt && (s_mask[j] & wbit) && bhi - j <= whi;
      const uint32_t m = __ballot_sync(kFull, in);
      if (in) s_list[warp][nlist + __popc(m & lt)] = (uint8_t)j;
      nlist += __popc(m);
    }
    __syncwarp();
    for (uint32_t li = 0; li < nlist; ++li) {
      const int j = s_list[warp][li];
      const int i = bhi - j;
      float val[9];
#pragma unroll
      for (int k = 0; k < 9; ++k) val[k] = 0.0f;
      bool contrib = false;
      if (i <= myhi) {
        const float4 q0 = s_rec[j * 3 + 0], q1 = s_rec[j * 3 + 1], q2 = s_rec[j * 3 + 2];
        const float dx = pxf - q0.x, dy = pyf - q0.y;
        const float s1 = (q0.z * dx) * dx;
        const float s2 = (q1.x * dy) * dy;
        float so2 = 0.5f * (s1 + s2);
        so2 = so2 + (q0.w * dx) * dy;
        if (so2 >= 0.0f && so2 <= q2.y) {
          const float G = sky_expf_inrange(-so2);
          const float al = q1.y * G;
          const float a = fmin_(al, MAX_ALPHA);
          if (a >= MIN_ALPHA) {
            // The decision above repeats the forward's bit for bit; the
            // gradient arithmetic below only has to be accurate, so it uses
            // fused multiply-adds and the fast reciprocal division.  Per
            // pair it forms raw moments; the per-splat factors (1 - opacity
            // for the logit, -1/2 and -1 for the conic, the conic matrix for
            // the mean) are applied once per splat after the reduction:
            //   v3 = dL/dalpha * alpha          (dL/dlogit / (1 - opacity))
            //   g  = dL/dalpha * opacity * G    (= -dL/ds)
            //   v4..v8 = g dx^2, g dx dy, g dy^2, g dx, g dy.
            contrib = true;
            const float om = fmax_(1.0f - a, 0.0001f);
            const float Tb = __fdividef(T, om);
            const float ctb = a * Tb;
            const float d0 = q1.z - acc0, d1 = q1.w - acc1, d2 = q2.x - acc2;
            const float dLda = __fmaf_rn(r2, d2, __fmaf_rn(r1, d1, r0 * d0)) * Tb;
            const float dl = al > MAX_ALPHA ? 0.0f : dLda;  // the alpha clamp has zero slope
            const float g = dl * al;
            const float gdx = g * dx, gdy = g * dy;
            val[0] = r0 * ctb;
            val[1] = r1 * ctb;
            val[2] = r2 * ctb;
            val[3] = dl * a;
            val[4] = gdx * dx;
            val[5] = gdx * dy;
            val[6] = gdy * dy;
            val[7] = gdx;
            val[8] = gdy;
            acc0 = __fmaf_rn(a, d0, acc0);
            acc1 = __fmaf_rn(a, d1, acc1);
            acc2 = __fmaf_rn(a, d2, acc2);
            T = Tb;
          }
        }
      }
      const uint32_t who = __ballot_sync(kFull, contrib);
      if (who == 0u) {
        if (slot < 9) s_part[warp][j][slot] = 0.0f;
      } else if ((who & (who - 1u)) == 0u) {
        // a single contributing pixel: its values are the warp's sums
        if (contrib) {
#pragma unroll
          for (int k = 0; k < 9; ++k) s_part[warp][j][k] = val[k];
        }
      } else {
        const float tot = warp_reduce_scatter9(val, lane);
        if (slot < 9) s_part[warp][j][slot] = tot;
      }
    }
    __syncthreads();
    for (int j = (int)tid; j < cnt; j += NT) {
      const int i = bhi - j;
      const uint32_t m = s_mask[j];
      float sum[9];
#pragma unroll
      for (int k = 0; k < 9; ++k) sum[k] = 0.0f;
      for (int w = 0; w < NW; ++w) {
        if (!((m >> w) & 1u) || i > s_hi[w]) continue;  // warp w skipped this splat
#pragma unroll
        for (int k = 0; k < 9; ++k) sum[k] = sum[k] + s_part[w][j][k];
      }
      // moments -> dL/dlogit, dL/dconic (a, b, c), dL/dmean (x, y)
      const float4 q0 = s_rec[j * 3 + 0], q1 = s_rec[j * 3 + 1];
      const float dlogit = sum[3] * (1.0f - q1.y);
      const float dca = -0.5f * sum[4], dcb = -sum[5], dcc = -0.5f * sum[6];
      const float dmx = __fmaf_rn(q0.z, sum[7], q0.w * sum[8]);
      const float dmy = __fmaf_rn(q0.w, sum[7], q1.x * sum[8]);
      write_partial(b, b.vals_sorted[i], sum, dlogit, dca, dcb, dcc, dmx, dmy);
    }
  }
}

// ---------------------------------------------------------------------------
// Backward, exact mode, 16x16 tiles with two pixels per thread: 128 threads;
// warp w covers the 8x8 block (w & 1, w >> 1) of the tile, lane l holds
// column l & 7 of block rows 2(l >> 3) and the row below.  A splat reaches
// about half as many warps as with 16x2 strips, and each (warp, splat) pays
// its shared loads, list entry and nine-value reduction once for 64 pixels
// (the two pixels' values are added in the lane first).  Per pixel the
// arithmetic is that of k_backward_exact; the per-(tile, intersection) sums
// differ only in summation order.
// ---------------------------------------------------------------------------
// racc = r . acc: the residual dotted with the colour accumulated behind the
// current splat (starting from the background), the only use of that colour.
struct BwdPix {
  float px, py, T, racc, r[3];
  int hi;
};

// exp(-s) for 0 <= s <= ln(255) + 1e-3 by the ex2.approx instruction
// (relative error below 1e-6 here, including the rounding of -s log2 e).
SKY_DEV float exp_neg_approx(float s) {
  float r;
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(s * -1.44269504f));
  return r;
}

// The s below which a pair surely contributes, unclamped: for a splat with
// opacity <= 0.9989 (alpha = opacity exp(-s) rounds to at most 0.99890018 <
// 0.999, never clamped) it is the raster pre-filter bound smax =
// __logf(255 opacity) + 1e-3 less 1.1e-3.  smax - 1e-3 is within 2e-6 of
// ln(opacity / f32(1/255)) (3 ulp of __logf, f32 roundings), so at s <=
// smax - 1.1e-3 the exact alpha is at least f32(1/255) (1 + 9e-5), far
// beyond the forward exponential's 1-ulp error: the forward composited the
// pair.  -1 (no pair is sure) for opacities that can reach the clamp.
SKY_DEV float sure_bound(const float4& q1, const float4& q2) {
  return q1.y > 0.9989f ? -1.0f : q2.y - 1.1e-3f;
}

// One (pixel, splat) pair of the exact backward: adds the pair's raw moments
// to val and steps the pixel's transmittance and accumulated colour back past
// the splat.  val[0..3] are the colour-weighted and opacity moments; since
// a lane's two pixels share dx, val[4..6] hold sum g, sum g dy and sum g dy^2
// (g = dL/dalpha alpha), and the entry forms g dx^2, g dx dy, g dy^2, g dx,
// g dy from them (lane_moments).  Returns whether the splat contributes at the pixel.
// Which pairs contribute (alpha >= 1/255) and which are clamped (alpha >
// 0.999) must be decided exactly as the forward decided them; the gradient
// values only have to be accurate.  A pair with s <= s_sure (sure_bound)
// contributes unclamped; above it, alpha comes from the fast exponential,
// and from sky_expf (the forward's) only when it lies within 2e-6 relative of
// either threshold, where the two could decide differently.  In both cases
// the gradient uses the fast exponential's alpha.
// dx = px - mx, s1 = (a/2 dx) dx (q0, q1 are staged records, conic halved)
// and bdx = b dx belong to the pixel column and are shared by the lane's two
// pixels.
SKY_DEV bool bwd_pair(BwdPix& p, float dx, float s1, float bdx, const float4& q0, const float4& q1,
                      const float4& q2, float s_sure, float val[9]) {
  const float dy = p.py - q0.y;
  const float s2 = (q1.x * dy) * dy;  // staged record: halved conic
  float so2 = s1 + s2;
  so2 = so2 + bdx * dy;
  if (outside_smax(so2, q2.y)) return false;
  float G = exp_neg_approx(so2);
  float al = q1.y * G;
  float a = al;
  bool clamped = false;
  if (so2 > s_sure) {
    if (fabsf(al - MIN_ALPHA) <= 2e-6f * MIN_ALPHA || fabsf(al - MAX_ALPHA) <= 2e-6f) {
      G = sky_expf_inrange(-so2);
      al = q1.y * G;
    }
    a = fmin_(al, MAX_ALPHA);
    if (!(a >= MIN_ALPHA)) return false;
    clamped = al > MAX_ALPHA;  // the clamp has zero slope
  }
  const float om = 1.0f - a;  // >= 0.001 (a <= 0.999): the reference's max(1 - a, 1e-4)
  const float Tb = __fdividef(p.T, om);
  const float ctb = a * Tb;
  // dL/dalpha = r . (colour - acc) T_before, with r . acc carried as racc
  const float rcol = __fmaf_rn(p.r[2], q2.x, __fmaf_rn(p.r[1], q1.w, p.r[0] * q1.z));
  const float dd = rcol - p.racc;
  const float dLda = dd * Tb;
  const float dl = clamped ? 0.0f : dLda;
  const float g = dl * al;
  const float gdy = g * dy;
  val[0] = __fmaf_rn(p.r[0], ctb, val[0]);
  val[1] = __fmaf_rn(p.r[1], ctb, val[1]);
  val[2] = __fmaf_rn(p.r[2], ctb, val[2]);
  val[3] = __fmaf_rn(dl, a, val[3]);
  val[4] = val[4] + g;                     // sum g      (dx is the lane's)
  val[5] = val[5] + gdy;                   // sum g dy
  val[6] = __fmaf_rn(gdy, dy, val[6]);     // sum g dy^2
  p.racc = __fmaf_rn(a, dd, p.racc);  // acc += a (colour - acc), dotted with r
  p.T = Tb;
  return true;
}

// The nine moments of a lane from its accumulators (bwd_pair) and its dx.
SKY_DEV void lane_moments(float val[9], float dx) {
  const float gs = val[4], gy = val[5], gyy = val[6];
  const float gdx = gs * dx;
  val[4] = gdx * dx;
  val[5] = gy * dx;
  val[6] = gyy;
  val[7] = gdx;
  val[8] = gy;
}

// The warp's nine moment sums of an entry from the lanes' raw sums (bwd_pair's
// val[0..6]), column first: the four lanes of a pixel column (lane & 7) share
// dx, so the seven raw sums are added over the column (lanes l ^ 8, l ^ 16)
// before the g sums are expanded by dx, and only then over the eight columns
// (10 shuffles instead of 12, and the expansion once per column).  After the
// column step a lane of row group (lane >> 3) & 3 holds two sums u0, u1
// ({c0, c1}, {c2, g}, {o, g dy}, {g dy^2, -}) and forms u0, u1 f1, u1 f2 from
// its factors f1 = a1 + dx (b1 + dx c1), f2 = a2 + dx b2.  On return the lane
// with cols9_slot(lane) == k < 9 holds the warp total of lane_moments' k-th
// value.
struct ColFactors {
  float a1, b1, c1, a2, b2;
};
// The row group's outputs u0, u1 f1, u1 f2 per case:
SKY_DEV ColFactors col_factors(uint32_t lane) {
  switch ((lane >> 3) & 3u) {
    case 0: return {1.0f, 0.0f, 0.0f, 0.0f, 0.0f};  // c0, c1, (0)
    case 1: return {0.0f, 0.0f, 1.0f, 0.0f, 1.0f};  // c2, g dx^2, g dx
    case 2: return {0.0f, 1.0f, 0.0f, 1.0f, 0.0f};  // o, g dy dx, g dy
    default: return {0.0f, 0.0f, 0.0f, 0.0f, 0.0f};  // g dy^2, (0), (0)
  }
}
SKY_DEV int cols9_slot(uint32_t lane) {
  if (lane & 1u) return 9;
  const int xi = (int)((lane >> 2) & 1u) * 2 + (int)((lane >> 1) & 1u);
  switch ((lane >> 3) & 3u) {
    case 0: return xi == 0 ? 0 : (xi == 1 ? 1 : 9);
    case 1: return xi == 0 ? 2 : (xi == 1 ? 4 : (xi == 2 ? 7 : 9));
    case 2: return xi == 0 ? 3 : (xi == 1 ? 5 : (xi == 2 ? 8 : 9));
    default: return xi == 0 ? 6 : 9;
  }
}
SKY_DEV float warp_reduce_cols9(const float val[9], float dx, uint32_t lane, const ColFactors& f) {
  const bool b4 = lane & 16u, b3 = lane & 8u, b2 = lane & 4u, b1 = lane & 2u;
  const float v[8] = {val[0], val[1], val[2], val[4], val[3], val[5], val[6], 0.0f};
  float w[4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
    w[i] = (b4 ? v[i + 4] : v[i]) + __shfl_xor_sync(kFull, b4 ? v[i] : v[i + 4], 16);
  float u[2];
#pragma unroll
  for (int i = 0; i < 2; ++i)
    u[i] = (b3 ? w[i + 2] : w[i]) + __shfl_xor_sync(kFull, b3 ? w[i] : w[i + 2], 8);
  const float f1 = __fmaf_rn(dx, __fmaf_rn(dx, f.c1, f.b1), f.a1);
  const float f2 = __fmaf_rn(dx, f.b2, f.a2);
  const float x0 = u[0], x1 = u[1] * f1, x2 = u[1] * f2;
  const float y0 = (b2 ? x2 : x0) + __shfl_xor_sync(kFull, b2 ? x0 : x2, 4);
  const float y1 = (b2 ? 0.0f : x1) + __shfl_xor_sync(kFull, b2 ? x1 : 0.0f, 4);
  const float z = (b1 ? y1 : y0) + __shfl_xor_sync(kFull, b1 ? y0 : y1, 2);
  return z + __shfl_xor_sync(kFull, z, 1);
}

// BB: the splat-batch depth (32, 64 or 128 staged splats); the per-splat sums
// do not depend on it.
template <int BB, bool CNT = false>
__global__ void __launch_bounds__(128, 8) k_backward_exact2(DevBuffers b) {
  constexpr int TS = 16, NT = 128, NW = 4, kBatch = BB;
  static_assert(BB <= NT, "one staged splat per thread and batch");
  __shared__ float4 s_rec[kBatch * 3];
  __shared__ uint32_t s_mask[kBatch];
  __shared__ float s_part[NW][kBatch][9];
  __shared__ int s_hi[NW];
  __shared__ uint8_t s_list[NW][kBatch];
  const StepParams& sp = *b.sp;
  const uint32_t tile = blockIdx.x;
  if (tile >= sp.num_tiles) return;
  if (capacity_failed(b.status)) return;
  const uint32_t start = b.offsets[tile], end = b.offsets[tile + 1];
  if (start >= end) return;
  const int v = find_view(sp, tile);
  const ViewInfo& vi = sp.views[v];
  const uint32_t local = tile - vi.tile_base;
  const uint32_t tx = local % vi.tiles_x, ty = local / vi.tiles_x;
  const uint32_t tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const uint32_t x = tx * TS + 8u * (warp & 1u) + (lane & 7u);
  const uint32_t y0 = ty * TS + 8u * (warp >> 1) + 2u * (lane >> 3);
  BwdPix pix[2];
#pragma unroll
  for (int h = 0; h < 2; ++h) {
    BwdPix& p = pix[h];
    const uint32_t y = y0 + (uint32_t)h;
    p.px = (float)x + 0.5f;
    p.py = (float)y + 0.5f;
    p.T = 1.0f;
    p.r[0] = p.r[1] = p.r[2] = 0.0f;
    p.hi = (int)start - 1;
    if (x < vi.width && y < vi.height) {
      const size_t q = (size_t)vi.pixel_base + (size_t)y * vi.width + x;
      const uint32_t lst = b.last[q];
      if (lst >= start) p.hi = (int)min(lst, end - 1);
      p.T = b.tfinal[q];
      const float4 rs = b.residual[q];
      p.r[0] = rs.x; p.r[1] = rs.y; p.r[2] = rs.z;
    }
    p.racc = __fmaf_rn(p.r[2], sp.bg[2], __fmaf_rn(p.r[1], sp.bg[1], p.r[0] * sp.bg[0]));
  }
  int whi = max(pix[0].hi, pix[1].hi);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) whi = max(whi, __shfl_xor_sync(kFull, whi, o));
  if (lane == 0) s_hi[warp] = whi;
  __syncthreads();
  int hi = s_hi[0];
  for (int w = 1; w < NW; ++w) hi = max(hi, s_hi[w]);
  const int slot = cols9_slot(lane);
  const ColFactors cf = col_factors(lane);
  const uint32_t wbit = 1u << warp;
  const uint32_t lt = (1u << lane) - 1u;
  uint32_t n_eval = 0, n_contrib = 0, n_entries = 0, n_idle = 0;  // counting variant only
  // intersections beyond every pixel's last contributor are not written:
  // their emission slots stay unflagged in b.reached and count as zero
  for (int bhi = hi; bhi >= (int)start; bhi -= kBatch) {
    const int cnt = min(kBatch, bhi - (int)start + 1);
    __syncthreads();
    // thread k stages splat k and later writes its partial: its emission
    // index is loaded here, off the write's path
    uint32_t e_mine = 0;
    for (int k = (int)tid; k < cnt; k += NT) {
      e_mine = b.vals_sorted[bhi - k];
      const size_t r = b.flatten[bhi - k];
      const float4 q0 = b.records[r * 3 + 0];
      const float4 q1 = b.records[r * 3 + 1];
      const float4 q2 = b.records[r * 3 + 2];
      // the forward's 8x4-block ellipse mask of this intersection (it staged
      // every intersection up to the tile's last contributor): an 8x8 block
      // is kept when either of its two 8x4 halves is
      const uint32_t m8 = b.fmask[bhi - k];
      s_mask[k] = ((m8 | (m8 >> 2)) & 3u) | ((((m8 >> 4) | (m8 >> 6)) & 3u) << 2);
      // the box half-widths are only needed for the mask: the staged record
      // carries the splat's sure bound in their place
      stage_record(s_rec + k * 3, q0, q1, make_float4(q2.x, q2.y, sure_bound(q1, q2), q2.w));
    }
    __syncthreads();
    uint32_t nlist = 0;
    for (int base = 0; base < cnt; base += 32) {
      const int j = base + (int)lane;
      const bool in = j < cnt && (s_mask[j] & wbit) && bhi - j <= whi;
      const uint32_t m = __ballot_sync(kFull, in);
      if (in) s_list[warp][nlist + __popc(m & lt)] = (uint8_t)j;
      nlist += __popc(m);
    }
    __syncwarp();
    for (uint32_t li = 0; li < nlist; ++li) {
      const int j = s_list[warp][li];
      const int i = bhi - j;
      float val[9];
#pragma unroll
      for (int k = 0; k < 9; ++k) val[k] = 0.0f;
      const float4 q0 = s_rec[j * 3 + 0], q1 = s_rec[j * 3 + 1], q2 = s_rec[j * 3 + 2];
      const float dx = pix[0].px - q0.x;
      const float s1 = (q0.z * dx) * dx, bdx = q0.w * dx;
      const float s_sure = q2.z;  // sure_bound, staged
      bool contrib = false;
      if constexpr (CNT) {
        ++n_entries;
        bool c0 = false, c1 = false;
        if (i <= pix[0].hi) { ++n_eval; c0 = bwd_pair(pix[0], dx, s1, bdx, q0, q1, q2, s_sure, val); }
        if (i <= pix[1].hi) { ++n_eval; c1 = bwd_pair(pix[1], dx, s1, bdx, q0, q1, q2, s_sure, val); }
        n_contrib += (uint32_t)c0 + (uint32_t)c1;
        contrib = c0 || c1;
      } else {
        if (i <= pix[0].hi) contrib = bwd_pair(pix[0], dx, s1, bdx, q0, q1, q2, s_sure, val);
        if (i <= pix[1].hi) contrib = bwd_pair(pix[1], dx, s1, bdx, q0, q1, q2, s_sure, val) || contrib;
      }
      const uint32_t who = __ballot_sync(kFull, contrib);
      if constexpr (CNT) n_idle += who == 0u ? 1u : 0u;
      if (who == 0u) {
        if (slot < 9) s_part[warp][j][slot] = 0.0f;
      } else if ((who & (who - 1u)) == 0u) {
        if (contrib) {
          lane_moments(val, dx);
#pragma unroll
          for (int k = 0; k < 9; ++k) s_part[warp][j][k] = val[k];
        }
      } else {
        const float tot = warp_reduce_cols9(val, dx, lane, cf);
        if (slot < 9) s_part[warp][j][slot] = tot;
      }
    }
    __syncthreads();
    for (int j = (int)tid; j < cnt; j += NT) {  // (j = tid: the thread that staged it)
      const int i = bhi - j;
      const uint32_t m = s_mask[j];
      float sum[9];
#pragma unroll
      for (int k = 0; k < 9; ++k) sum[k] = 0.0f;
      for (int w = 0; w < NW; ++w) {
        if (!((m >> w) & 1u) || i > s_hi[w]) continue;  // warp w skipped this splat
#pragma unroll
        for (int k = 0; k < 9; ++k) sum[k] = sum[k] + s_part[w][j][k];
      }
      const float4 q0 = s_rec[j * 3 + 0], q1 = s_rec[j * 3 + 1];
      const float ca = q0.z + q0.z, cc = q1.x + q1.x;  // the conic (exact doubling)
      const float dlogit = sum[3] * (1.0f - q1.y);
      const float dca = -0.5f * sum[4], dcb = -sum[5], dcc = -0.5f * sum[6];
      const float dmx = __fmaf_rn(ca, sum[7], q0.w * sum[8]);
      const float dmy = __fmaf_rn(q0.w, sum[7], cc * sum[8]);
      write_partial(b, e_mine, sum, dlogit, dca, dcb, dcc, dmx, dmy);
    }
  }
  // (every lane walks the warp's list: lane 0's n_entries and n_idle are
  // the warp's)
  if constexpr (CNT) {
    add_pair_counts(b, 3, n_eval, n_contrib, n_entries);
    if (lane == 0) atomicAdd(&b.status->pairs[6], (unsigned long long)n_idle);
  }
}

// ---------------------------------------------------------------------------
// Backward, reference mode: backward-tiles-local.wgsl:185-382 as written --
// batches of 64 intersections in ascending order, each walked back to front
// per pixel, alpha > 0.98 skipped, 54 values per pair truncated to i32 fixed
// point (x65536) and summed per (tile, intersection); then per item the 54
// sums are added exactly in i64 (backward-reduce.wgsl:35-71 without its
// order-dependent float CAS).
// ---------------------------------------------------------------------------
constexpr int kRefBatch = 64;

template <int TS>
__global__ void __launch_bounds__(TS* TS) k_backward_ref(DevBuffers b) {
  constexpr int NT = TS * TS;
  __shared__ float4 s_rec[kRefBatch * 3];
  __shared__ float s_dir[kRefBatch * 3];
  __shared__ int s_tg[kRefBatch][54];
  const StepParams& sp = *b.sp;
  const uint32_t tile = blockIdx.x;
  if (tile >= sp.num_tiles) return;
  if (capacity_failed(b.status)) return;
  const uint32_t start = b.offsets[tile], end = b.offsets[tile + 1];
  if (start >= end) return;
  const int v = find_view(sp, tile);
  const ViewInfo& vi = sp.views[v];
  const uint32_t local = tile - vi.tile_base;
  const uint32_t tx = local % vi.tiles_x, ty = local / vi.tiles_x;
  const uint32_t tid = threadIdx.x, lane = tid & 31;
  const uint32_t x = tx * TS + (tid % TS), y = ty * TS + (tid / TS);
  const bool inside = x < vi.width && y < vi.height;
  const int deg = (int)sp.sh_deg;
  float T = 1.0f, acc0 = sp.bg[0], acc1 = sp.bg[1], acc2 = sp.bg[2];
  float r0 = 0.0f, r1 = 0.0f, r2 = 0.0f;
  uint32_t binf = 0;
  bool valid = false;
  const float pxf = (float)x + 0.5f, pyf = (float)y + 0.5f;
  if (inside) {
    const size_t p = (size_t)vi.pixel_base + (size_t)y * vi.width + x;
    binf = b.last[p];
    T = 1.0f - b.alpha[p];
    const float4 rs = b.residual[p];
    r0 = rs.x; r1 = rs.y; r2 = rs.z;
    valid = binf >= start && binf != 0xFFFFFFFFu;
  }
  const bool r16 = sp.round_f16 != 0;
  for (uint32_t bs = start; bs < end; bs += kRefBatch) {
    const uint32_t be = min(bs + kRefBatch, end);
    const int cnt = (int)(be - bs);
    __syncthreads();
    for (int k = tid; k < kRefBatch * 54; k += NT) (&s_tg[0][0])[k] = 0;
    if ((int)tid < cnt) {
      const size_t r = b.flatten[bs + tid];
      s_rec[tid * 3 + 0] = b.records[r * 3 + 0];
      s_rec[tid * 3 + 1] = b.records[r * 3 + 1];
      s_rec[tid * 3 + 2] = b.records[r * 3 + 2];
      // view direction normalize(-(view * p)), as the projection computes it
      const uint32_t g = (uint32_t)(r % sp.n);
      const float px = load_plane(b.params, sp.plane_stride, 0, g, r16);
      const float py = load_plane(b.params, sp.plane_stride, 1, g, r16);
      const float pz = load_plane(b.params, sp.plane_stride, 2, g, r16);
      const float c0 = -mat4_row(vi.view, 0, px, py, pz, 1.0f);
      const float c1 = -mat4_row(vi.view, 1, px, py, pz, 1.0f);
      const float c2 = -mat4_row(vi.view, 2, px, py, pz, 1.0f);
      float vv = c0 * c0 + c1 * c1;
      vv = vv + c2 * c2;
      const float vl = sqrtf(vv);
      s_dir[tid * 3 + 0] = c0 / vl;
      s_dir[tid * 3 + 1] = c1 / vl;
      s_dir[tid * 3 + 2] = c2 / vl;
    }
    __syncthreads();
    const uint32_t pe = valid ? min(be, binf + 1) : bs;
    for (int jj = cnt - 1; jj >= 0; --jj) {
      const uint32_t i = bs + (uint32_t)jj;
      int val[54];
#pragma unroll
      for (int k = 0; k < 54; ++k) val[k] = 0;
      bool contrib = false;
      if (i < pe) {
        const float4 q0 = s_rec[jj * 3 + 0], q1 = s_rec[jj * 3 + 1], q2 = s_rec[jj * 3 + 2];
        const float dx = pxf - q0.x, dy = pyf - q0.y;
        const float s1 = (q0.z * dx) * dx;
        const float s2 = (q1.x * dy) * dy;
        float so2 = 0.5f * (s1 + s2);
        so2 = so2 + (q0.w * dx) * dy;
        if (so2 >= 0.0f && so2 <= q2.y) {
          const float G = sky_expf(-so2);
          const float op = q1.y;
          const float a = fmin_(op * G, MAX_ALPHA);
          if (a >= MIN_ALPHA && !(a > 0.98f)) {
            contrib = true;
            const float cr = q1.z, cg = q1.w, cbl = q2.x;
            const float om = fmax_(1.0f - a, 0.0001f);
            const float Tb = T / om;
            const float ctb = a * Tb;
            const float rs0 = r0 * ctb, rs1 = r1 * ctb, rs2 = r2 * ctb;
            const float xd = s_dir[jj * 3 + 0], yd = s_dir[jj * 3 + 1], zd = s_dir[jj * 3 + 2];
            float Y[16];
            sh_basis(xd, yd, zd, deg, Y);
            const int ncoef = (deg + 1) * (deg + 1);
#pragma unroll
            for (int k = 0; k < 16; ++k) {
              if (k < ncoef) {
                val[6 + 3 * k + 0] = wgsl_i32((Y[k] * rs0) * 65536.0f);
                val[6 + 3 * k + 1] = wgsl_i32((Y[k] * rs1) * 65536.0f);
                val[6 + 3 * k + 2] = wgsl_i32((Y[k] * rs2) * 65536.0f);
              }
            }
            float fg = r0 * cr + r1 * cg;
            fg = fg + r2 * cbl;
            float bgt = r0 * acc0 + r1 * acc1;
            bgt = bgt + r2 * acc2;
            const float dLda = (fg - bgt) * Tb;
            const float dlogit = (dLda * a) * (1.0f - op);
            const float dLdG = dLda * op;
            const float dLds = dLdG * (-G);
            val[0] = wgsl_i32(dlogit * 65536.0f);
            val[1] = wgsl_i32((((dLds * 0.5f) * dx) * dx) * 65536.0f);
            val[2] = wgsl_i32(((dLds * dx) * dy) * 65536.0f);
            val[3] = wgsl_i32((((dLds * 0.5f) * dy) * dy) * 65536.0f);
            val[4] = wgsl_i32((-(dLds * ((q0.z * dx) + (q0.w * dy)))) * 65536.0f);
            val[5] = wgsl_i32((-(dLds * ((q0.w * dx) + (q1.x * dy)))) * 65536.0f);
            acc0 = a * cr + (1.0f - a) * acc0;
            acc1 = a * cg + (1.0f - a) * acc1;
            acc2 = a * cbl + (1.0f - a) * acc2;
            T = Tb;
          }
        }
      }
      if (__any_sync(kFull, contrib)) {
#pragma unroll
        for (int k = 0; k < 54; ++k) {
          int s = val[k];
#pragma unroll
          for (int o = 16; o > 0; o >>= 1)
            s = (int)((uint32_t)s + (uint32_t)__shfl_xor_sync(kFull, s, o));
          val[k] = s;
        }
        // lane k adds slot k and k + 32 (integer, order-independent)
#pragma unroll
        for (int k = 0; k < 54; ++k)
          if ((k & 31) == (int)lane && val[k] != 0) atomicAdd(&s_tg[jj][k], val[k]);
      }
    }
    __syncthreads();
    for (int k = tid; k < cnt * 54; k += NT) {
      const int jj = k / 54, slot = k % 54;
      const int s = s_tg[jj][slot];
      const uint32_t i = bs + (uint32_t)jj;
      b.tile_grads[(size_t)i * 54 + slot] = s;
      if (s != 0) atomicAdd((unsigned long long*)&b.gsum54[(size_t)b.flatten[i] * 54 + slot],
                            (unsigned long long)(long long)s);
    }
  }
}

// ---------------------------------------------------------------------------
// Geometry adjoint + SH chain + Adam, one thread per Gaussian.  For each view
// of the step: sum the Gaussian's per-intersection partials (contiguous in
// emission order, summed in order), then back-propagate dL/d(colour, logit,
// conic, mean2d) through the projection as implemented (training-tiles.wgsl:
// 40-180) to position, log sigma, quaternion, opacity logit and SH.  The
// per-view gradients are added in view order.  Then adam.wgsl:18-38 per
// plane with the group's learning rate.
// ---------------------------------------------------------------------------
struct Grad11 {
  float pos[3], ls[3], q[4], logit;
};

// One view of the adjoint, up to the 3D covariance: adds the view's dL/dmean
// and dL/dlogit to gr and its dL/dC3 to g3 (the symmetric V^T GW V, entries
// 00 01 02 11 12 22).  The chain from C3 to the scales and the quaternion is
// linear in dL/dC3, so it runs once per Gaussian on the sum over views
// (geom_cov_final).  pc is the camera-space mean, o.dir / o.raw the view
// direction and the unclamped SH colour.
SKY_DEV void geom_view(const float pc[4], const ProjOut& o, const ViewInfo& vi, const StepParams& sp,
                       const float (&C3)[3][3], const float in9[9], bool color_dir,
                       const float* sh /*48 values at sh[k * sh_stride]*/, int sh_stride, int deg,
                       Grad11& gr, float g3[6]) {
  // mean -> camera space
  float dpc[3] = {0.f, 0.f, 0.f};
  float clip[4];
#pragma unroll
  for (int r = 0; r < 4; ++r) clip[r] = mat4_row(vi.proj, r, pc[0], pc[1], pc[2], pc[3]);
  // (gradient arithmetic only -- no decision depends on it -- so quotients
  // take the fast reciprocal: 2 ulp)
  const float rw = __fdividef(1.0f, clip[3]);
  const float ndx = clip[0] * rw, ndy = clip[1] * rw;
  const float gx = in9[7] * (0.5f * (float)vi.width) * rw, gy = in9[8] * (0.5f * (float)vi.height) * rw;
#pragma unroll
  for (int j = 0; j < 3; ++j) {
    dpc[j] += gx * (vi.proj[j * 4 + 0] - ndx * vi.proj[j * 4 + 3]);
    dpc[j] += gy * (vi.proj[j * 4 + 1] - ndy * vi.proj[j * 4 + 3]);
  }
  // covariance
  float V3[3][3];  // math rows
#pragma unroll
  for (int r = 0; r < 3; ++r)
#pragma unroll
    for (int j = 0; j < 3; ++j) V3[r][j] = vi.view[j * 4 + r];
  float tmp[3][3], Wm[2][2];
#pragma unroll
  for (int a = 0; a < 2; ++a)
#pragma unroll
    for (int c = 0; c < 3; ++c) tmp[a][c] = V3[a][0] * C3[0][c] + V3[a][1] * C3[1][c] + V3[a][2] * C3[2][c];
#pragma unroll
  for (int a = 0; a < 2; ++a)
#pragma unroll
    for (int c = 0; c < 2; ++c) Wm[a][c] = tmp[a][0] * V3[c][0] + tmp[a][1] * V3[c][1] + tmp[a][2] * V3[c][2];
  const float tz = pc[2];
  const float rtz = __fdividef(1.0f, tz);
  const float kx = vi.focal[0] * rtz, ky = vi.focal[1] * rtz;
  const float C00 = kx * kx * Wm[0][0], C01 = kx * ky * Wm[0][1], C11 = ky * ky * Wm[1][1];
  const float e00 = C00 + sp.eps2d, e11 = C11 + sp.eps2d;
  const float det = e00 * e11 - C01 * C01;
  const float rdet = __fdividef(1.0f, det);
  const float Qa = e11 * rdet, Qb = -C01 * rdet, Qc = e00 * rdet;
  const float ga = in9[4], gb = 0.5f * in9[5], gc = in9[6];
  // dC = -Q GQ Q (2x2 symmetric)
  const float t00 = ga * Qa + gb * Qb, t01 = ga * Qb + gb * Qc;
  const float t10 = gb * Qa + gc * Qb, t11 = gb * Qb + gc * Qc;
  const float dC00 = -(Qa * t00 + Qb * t10);
  const float dC01a = -(Qa * t01 + Qb * t11);
  const float dC10a = -(Qb * t00 + Qc * t10);
  const float dC11 = -(Qb * t01 + Qc * t11);
  const float dC01 = dC01a + dC10a;
  const float dW00 = dC00 * kx * kx, dW01 = dC01 * kx * ky, dW11 = dC11 * ky * ky;
  dpc[2] += -2.0f * rtz * (dC00 * C00 + dC01 * C01 + dC11 * C11);
  // G3 = V3^T GW V3 with GW = [[dW00, dW01/2, 0], [dW01/2, dW11, 0], [0, 0, 0]]
  const float hW01 = 0.5f * dW01;
  float u0[3], u1[3];  // GW V3, rows 0 and 1
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    u0[c] = dW00 * V3[0][c] + hW01 * V3[1][c];
    u1[c] = hW01 * V3[0][c] + dW11 * V3[1][c];
  }
  g3[0] += V3[0][0] * u0[0] + V3[1][0] * u1[0];
  g3[1] += V3[0][0] * u0[1] + V3[1][0] * u1[1];
  g3[2] += V3[0][0] * u0[2] + V3[1][0] * u1[2];
  g3[3] += V3[0][1] * u0[1] + V3[1][1] * u1[1];
  g3[4] += V3[0][1] * u0[2] + V3[1][1] * u1[2];
  g3[5] += V3[0][2] * u0[2] + V3[1][2] * u1[2];
  gr.logit += in9[3];
  // colour -> view direction
  if (color_dir && deg > 0 && sh) {
    const float X = o.dir[0], Yv = o.dir[1], Z = o.dir[2];
    float draw[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) draw[c] = o.raw[c] > 0.0f ? in9[c] : 0.0f;
    float ddir[3] = {0.f, 0.f, 0.f};
    auto addk = [&](int k, float gx, float gy, float gz) {
      float s = draw[0] * sh[(3 * k) * sh_stride] + draw[1] * sh[(3 * k + 1) * sh_stride] +
                draw[2] * sh[(3 * k + 2) * sh_stride];
      ddir[0] += s * gx;
      ddir[1] += s * gy;
      ddir[2] += s * gz;
    };
    addk(1, 0.f, -SH_C1, 0.f);
    addk(2, 0.f, 0.f, SH_C1);
    addk(3, -SH_C1, 0.f, 0.f);
    if (deg > 1) {
      addk(4, SH_C2_0 * Yv, SH_C2_0 * X, 0.f);
      addk(5, 0.f, SH_C2_1 * Z, SH_C2_1 * Yv);
      addk(6, -2.f * SH_C2_2 * X, -2.f * SH_C2_2 * Yv, 4.f * SH_C2_2 * Z);
      addk(7, SH_C2_3 * Z, 0.f, SH_C2_3 * X);
      addk(8, 2.f * SH_C2_4 * X, -2.f * SH_C2_4 * Yv, 0.f);
    }
    if (deg > 2) {
      const float xx = X * X, yy = Yv * Yv, zz = Z * Z;
      addk(9, SH_C3_0 * 6.f * X * Yv, SH_C3_0 * (3.f * xx - 3.f * yy), 0.f);
      addk(10, SH_C3_1 * Yv * Z, SH_C3_1 * X * Z, SH_C3_1 * X * Yv);
      addk(11, SH_C3_2 * (-2.f * X * Yv), SH_C3_2 * (4.f * zz - xx - 3.f * yy), SH_C3_2 * 8.f * Yv * Z);
      addk(12, SH_C3_3 * (-6.f * X * Z), SH_C3_3 * (-6.f * Yv * Z), SH_C3_3 * (6.f * zz - 3.f * xx - 3.f * yy));
      addk(13, SH_C3_4 * (4.f * zz - 3.f * xx - yy), SH_C3_4 * (-2.f * X * Yv), SH_C3_4 * 8.f * X * Z);
      addk(14, SH_C3_5 * 2.f * X * Z, SH_C3_5 * (-2.f * Yv * Z), SH_C3_5 * (xx - yy));
      addk(15, SH_C3_6 * (3.f * xx - 3.f * yy), SH_C3_6 * (-6.f * X * Yv), 0.f);
    }
    const float rvl = rsqrtf(pc[0] * pc[0] + pc[1] * pc[1] + pc[2] * pc[2]);
    const float dd = X * ddir[0] + Yv * ddir[1] + Z * ddir[2];
    dpc[0] += -(ddir[0] - X * dd) * rvl;
    dpc[1] += -(ddir[1] - Yv * dd) * rvl;
    dpc[2] += -(ddir[2] - Z * dd) * rvl;
  }
#pragma unroll
  for (int j = 0; j < 3; ++j) gr.pos[j] += V3[0][j] * dpc[0] + V3[1][j] * dpc[1] + V3[2][j] * dpc[2];
}

// dL/dC3 summed over the views (g3, entries 00 01 02 11 12 22) through
// C3 = M M^T, M = R diag(sigma), to log sigma (zero slope where the clamp to
// [-10, 10] is active) and the quaternion (through the normalisation).
SKY_DEV void geom_cov_final(const float* prm /*11 geometry params*/, const float g3[6], Grad11& gr) {
  float sig[3], lsg[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const float raw = prm[3 + k];
    sig[k] = sky_expf(clampf_(raw, -10.0f, 10.0f));
    lsg[k] = (raw > -10.0f && raw < 10.0f) ? 1.0f : 0.0f;
  }
  float R[3][3], qn[4], ql;
  gauss_rotation([&](int plane) { return prm[plane]; }, R, qn, ql);
  const float x = qn[0], y = qn[1], z = qn[2], w = qn[3];
  const float G3[3][3] = {{g3[0], g3[1], g3[2]}, {g3[1], g3[3], g3[4]}, {g3[2], g3[4], g3[5]}};
  float dR[3][3], dsig[3] = {0.f, 0.f, 0.f};
#pragma unroll
  for (int a = 0; a < 3; ++a)
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      // dL/dM = 2 G3 M
      const float dM = 2.0f * sig[c] * (G3[a][0] * R[0][c] + G3[a][1] * R[1][c] + G3[a][2] * R[2][c]);
      dR[a][c] = dM * sig[c];
      dsig[c] += dM * R[a][c];
    }
  float dq[4];
  dq[0] = 2 * y * (dR[0][1] + dR[1][0]) + 2 * z * (dR[0][2] + dR[2][0]) +
          2 * w * (dR[2][1] - dR[1][2]) - 4 * x * (dR[1][1] + dR[2][2]);
  dq[1] = -4 * y * (dR[0][0] + dR[2][2]) + 2 * x * (dR[0][1] + dR[1][0]) +
          2 * w * (dR[0][2] - dR[2][0]) + 2 * z * (dR[1][2] + dR[2][1]);
  dq[2] = -4 * z * (dR[0][0] + dR[1][1]) + 2 * w * (dR[1][0] - dR[0][1]) +
          2 * x * (dR[0][2] + dR[2][0]) + 2 * y * (dR[1][2] + dR[2][1]);
  dq[3] = -2 * z * dR[0][1] + 2 * y * dR[0][2] + 2 * z * dR[1][0] - 2 * x * dR[1][2] -
          2 * y * dR[2][0] + 2 * x * dR[2][1];
  const float qd = x * dq[0] + y * dq[1] + z * dq[2] + w * dq[3];
#pragma unroll
  for (int k = 0; k < 4; ++k) gr.q[k] += (dq[k] - qn[k] * qd) / ql;
#pragma unroll
  for (int k = 0; k < 3; ++k) gr.ls[k] += dsig[k] * sig[k] * lsg[k];
}

// The step's Adam constants (adam.wgsl's uniforms), read once.
struct AdamK {
  float b1, omb1, b2, omb2, eps, bc1_rcp, bc2_sqrt_rcp;
};
SKY_DEV AdamK adam_consts(const StepParams& sp) {
  return AdamK{sp.beta1, 1.0f - sp.beta1, sp.beta2, 1.0f - sp.beta2, sp.adam_eps, sp.bc1_rcp,
               sp.bc2_sqrt_rcp};
}

// One Adam update of a parameter p and its moments m1, m2 (values, updated in
// place), in the reference's operation order.
SKY_DEV void adam_vals(float& p, float& m1, float& m2, float g, float lr, const AdamK& k) {
  const float a = k.b1 * m1;
  const float bb = k.omb1 * g;
  const float nm1 = a + bb;
  const float c = k.b2 * m2;
  const float d = (k.omb2 * g) * g;
  const float nm2 = c + d;
  const float denom = sqrtf(nm2) * k.bc2_sqrt_rcp + k.eps;
  const float step = lr * k.bc1_rcp;
  p = p - step * (nm1 / denom);
  m1 = nm1;
  m2 = nm2;
}

// N values passed by value (an array captured by reference would be placed
// in local memory).
template <int N>
struct Vals {
  float v[N];
};

// Adam over N consecutive planes of Gaussian g: every load first, then the
// updates, then the stores (a load after a store to another plane would wait
// for it: the arrays may alias as far as the compiler knows).
template <int N>
SKY_DEV void adam_planes(const DevBuffers& b, uint32_t stride, int plane0, uint32_t g, Vals<N> grad,
                         Vals<N> lr, const AdamK& k) {
  float P[N], M1[N], M2[N];
#pragma unroll
  for (int j = 0; j < N; ++j) {
    const size_t idx = (size_t)(plane0 + j) * stride + g;
    P[j] = b.params[idx];
    M1[j] = b.m1[idx];
    M2[j] = b.m2[idx];
  }
#pragma unroll
  for (int j = 0; j < N; ++j) adam_vals(P[j], M1[j], M2[j], grad.v[j], lr.v[j], k);
#pragma unroll
  for (int j = 0; j < N; ++j) {
    const size_t idx = (size_t)(plane0 + j) * stride + g;
    b.params[idx] = P[j];
    b.m1[idx] = M1[j];
    b.m2[idx] = M2[j];
  }
}

constexpr int kGeomThreads = 128;

// Exact mode: per (view, Gaussian) item, the sum of its intersections'
// partials in emission order (pairs added as ((s + a) + c), an odd last one
// alone), written as 3 float4.  A streaming pass with one thread per item,
// so the geometry kernel reads one fixed-size record per view instead of a
// variable-length chain of dependent loads.  Only partials the backward
// flagged in b.reached are read; the others are zero (intersections beyond
// every pixel's last contributor, about half of them, and all-zero sums).
__global__ void __launch_bounds__(256) k_item_sums(DevBuffers b) {
  const StepParams& sp = *b.sp;
  if (capacity_failed(b.status)) return;
  const size_t items = (size_t)sp.num_views * sp.n;
  for (size_t item = (size_t)blockIdx.x * blockDim.x + threadIdx.x; item < items;
       item += (size_t)gridDim.x * blockDim.x) {
    const uint32_t cnt = b.counts[item];
    if (cnt == 0) continue;  // never read
    float in9[9];
#pragma unroll
    for (int k = 0; k < 9; ++k) in9[k] = 0.0f;
    const uint32_t e1 = b.perm ? b.item_end[item] : b.cumsum[item], e0 = e1 - cnt;
    uint32_t e = e0;
    const float4 z = make_float4(0.f, 0.f, 0.f, 0.f);
    for (; e + 1 < e1; e += 2) {  // two partials in flight
      const bool fa = b.reached[e] != 0u, fc = b.reached[e + 1] != 0u;
      const float4 a0 = fa ? b.partials[(size_t)e * 3 + 0] : z;
      const float4 a1 = fa ? b.partials[(size_t)e * 3 + 1] : z;
      const float4 a2 = fa ? b.partials[(size_t)e * 3 + 2] : z;
      const float4 c0 = fc ? b.partials[(size_t)e * 3 + 3] : z;
      const float4 c1 = fc ? b.partials[(size_t)e * 3 + 4] : z;
      const float4 c2 = fc ? b.partials[(size_t)e * 3 + 5] : z;
      in9[0] = (in9[0] + a0.x) + c0.x; in9[1] = (in9[1] + a0.y) + c0.y;
      in9[2] = (in9[2] + a0.z) + c0.z; in9[3] = (in9[3] + a0.w) + c0.w;
      in9[4] = (in9[4] + a1.x) + c1.x; in9[5] = (in9[5] + a1.y) + c1.y;
      in9[6] = (in9[6] + a1.z) + c1.z; in9[7] = (in9[7] + a1.w) + c1.w;
      in9[8] = (in9[8] + a2.x) + c2.x;
    }
    if (e < e1 && b.reached[e] != 0u) {
      const float4 a0 = b.partials[(size_t)e * 3 + 0];
      const float4 a1 = b.partials[(size_t)e * 3 + 1];
      const float4 a2 = b.partials[(size_t)e * 3 + 2];
      in9[0] = in9[0] + a0.x; in9[1] = in9[1] + a0.y; in9[2] = in9[2] + a0.z;
      in9[3] = in9[3] + a0.w; in9[4] = in9[4] + a1.x; in9[5] = in9[5] + a1.y;
      in9[6] = in9[6] + a1.z; in9[7] = in9[7] + a1.w; in9[8] = in9[8] + a2.x;
    }
    float4* o = b.item_sums + item * 3;
    o[0] = make_float4(in9[0], in9[1], in9[2], in9[3]);
    o[1] = make_float4(in9[4], in9[5], in9[6], in9[7]);
    o[2] = make_float4(in9[8], 0.0f, 0.0f, 0.0f);
  }
}

// Dynamic shared memory of k_geom_adam: SH values and SH-gradient
// accumulators (48 x threads f32 each), two buffers of the threads' item
// sums (3 float4 per thread) and two of their (depth, radius) pairs.
constexpr size_t kGeomSmem =
    (size_t)96 * kGeomThreads * 4 + (size_t)2 * 3 * kGeomThreads * 16 + (size_t)2 * kGeomThreads * 8;

// SH values and SH-gradient accumulators live in shared memory (one column
// per thread, conflict-free), as do the item sums of the next view, copied
// asynchronously while the current view's adjoint runs, and the step's
// cameras; three blocks per multiprocessor resident (168 registers, 60 KB of
// dynamic and 12 KB of static shared memory each).
static_assert(sizeof(ViewInfo) % 4 == 0, "cameras are copied as 32-bit words");
__global__ void __launch_bounds__(kGeomThreads, 3) k_geom_adam(DevBuffers b) {
  extern __shared__ float4 s_dyn[];
  float* const s_base = reinterpret_cast<float*>(s_dyn);
  float (*s_sh)[kGeomThreads] = reinterpret_cast<float (*)[kGeomThreads]>(s_base);
  float (*s_gsh)[kGeomThreads] = reinterpret_cast<float (*)[kGeomThreads]>(s_base + 48 * kGeomThreads);
  float4 (*s_is)[3][kGeomThreads] =
      reinterpret_cast<float4 (*)[3][kGeomThreads]>(s_base + 96 * kGeomThreads);
  float2 (*s_aux)[kGeomThreads] =
      reinterpret_cast<float2 (*)[kGeomThreads]>(s_base + 96 * kGeomThreads + 2 * 3 * kGeomThreads * 4);
  const StepParams& sp = *b.sp;
  // the step's cameras, read by every thread in every view iteration
  __shared__ ViewInfo s_views[kMaxViews];
  {
    const uint32_t words = sp.num_views * (uint32_t)(sizeof(ViewInfo) / 4);
    const uint32_t* src = reinterpret_cast<const uint32_t*>(sp.views);
    uint32_t* dst = reinterpret_cast<uint32_t*>(s_views);
    for (uint32_t i = threadIdx.x; i < words; i += blockDim.x) dst[i] = src[i];
  }
  __syncthreads();
  if (capacity_failed(b.status)) return;
  const int t = threadIdx.x;
  const uint32_t g = blockIdx.x * blockDim.x + t;
  if (g >= sp.n) return;
  const uint32_t stride = sp.plane_stride;
  const bool r16 = sp.round_f16 != 0;
  const int deg = (int)sp.sh_deg;
  const int ncoef = (deg + 1) * (deg + 1);
  const bool ref = sp.bwd_mode != 0;
  const bool need_sh_grads = sp.sh_update || sp.write_grads;
  // the SH coefficients go to this thread's column of s_sh by asynchronous
  // copies, all in flight at once, then rounded in place
#pragma unroll
  for (int k = 0; k < 48; ++k) {
    if (!ref && k < 3 * ncoef) cp_async4(&s_sh[k][t], &b.params[(size_t)(11 + k) * stride + g]);
    else s_sh[k][t] = 0.0f;
    s_gsh[k][t] = 0.0f;
  }
  cp_async_commit();
  float prm[11];
#pragma unroll
  for (int k = 0; k < 11; ++k) prm[k] = load_plane_rw(b.params, stride, k, g, r16);
  cp_async_wait0();
  if (r16) {
#pragma unroll
    for (int k = 0; k < 48; ++k) s_sh[k][t] = round_f16(s_sh[k][t]);
  }
  Grad11 gr;
#pragma unroll
  for (int k = 0; k < 3; ++k) { gr.pos[k] = 0.f; gr.ls[k] = 0.f; }
#pragma unroll
  for (int k = 0; k < 4; ++k) gr.q[k] = 0.f;
  gr.logit = 0.f;
  auto get = [&](int plane) { return plane < 11 ? prm[plane] : s_sh[plane - 11][t]; };
  GaussCov3 gc;
  gauss_cov3(get, gc);
  float g3[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};  // dL/dC3 summed over the views
  // Densification statistics of training steps, per view in view order:
  // importance-accum.wgsl:19-40 (decayed tile count, visibility, screen
  // radius) and densify-accum.wgsl:19-46 (|dL/dmean2d|, |dL/dconic|, count).
  const bool stats = sp.apply_adam != 0 && b.importance != nullptr;
  float4 imp = make_float4(0.f, 0.f, 0.f, 0.f), acc = make_float4(0.f, 0.f, 0.f, 0.f);
  if (stats) {
    imp = reinterpret_cast<const float4*>(b.importance)[g];
    acc = reinterpret_cast<const float4*>(b.densify_accum)[g];
  }
  // The next view's tile count is loaded one iteration ahead and its item
  // sums are copied into shared memory, so their latency hides behind the
  // current view's adjoint.  Each thread copies and reads only its own column
  // (no block barrier); a copy of an item with no tiles is never read.
  auto stage = [&](uint32_t v, int buf) {
    const size_t it = (size_t)v * sp.n + g;
    if (!ref) {
      const float4* src = b.item_sums + it * 3;
      cp_async16(&s_is[buf][0][t], src + 0);
      cp_async16(&s_is[buf][1][t], src + 1);
      cp_async16(&s_is[buf][2][t], src + 2);
    }
    if (stats) cp_async8(&s_aux[buf][t], b.aux + it);
  };
  stage(0, 0);
  cp_async_commit();
  // with culled lists the statistics count the rectangle's tiles instead,
  // loaded one view ahead as well
  const bool rect_tiles = stats && sp.tile_cull;
  uint32_t cnt_next = b.counts[g];
  uint32_t area_next = rect_tiles ? rect_area(b.rects[g]) : 0u;
  for (uint32_t v = 0; v < sp.num_views; ++v) {
    const size_t item = (size_t)v * sp.n + g;
    const int buf = (int)(v & 1u);
    if (v + 1 < sp.num_views) stage(v + 1, buf ^ 1);
    cp_async_commit();
    cp_async_wait1();  // every group but the newest is complete: view v's copy
    const uint32_t cnt = cnt_next, area = area_next;
    if (v + 1 < sp.num_views) {
      cnt_next = b.counts[item + sp.n];
      if (rect_tiles) area_next = rect_area(b.rects[item + sp.n]);
    }
    float4 a0 = make_float4(0.f, 0.f, 0.f, 0.f), a1 = a0, a2 = a0;
    if (cnt > 0u && !ref) {
      a0 = s_is[buf][0][t];
      a1 = s_is[buf][1][t];
      a2 = s_is[buf][2][t];
    }
    if (stats) {
      imp.x = imp.x * sp.importance_decay;
      imp.y = imp.y * sp.importance_decay;
      imp.z = imp.z * sp.importance_decay;
      // the statistic counts the tiles of the item's rectangle, also when
      // the intersection lists hold only the tiles its ellipse reaches
      const uint32_t tiles = rect_tiles ? area : cnt;
      if (tiles > 0u) {
        imp.x = imp.x + (float)tiles;
        imp.y = imp.y + 1.0f;
        imp.z = fmax_(imp.z, s_aux[buf][t].y);
      }
    }
    if (cnt == 0) continue;
    float in9[9];
#pragma unroll
    for (int k = 0; k < 9; ++k) in9[k] = 0.0f;
    bool any = false;
    if (!ref) {
      in9[0] = a0.x; in9[1] = a0.y; in9[2] = a0.z; in9[3] = a0.w;
      in9[4] = a1.x; in9[5] = a1.y; in9[6] = a1.z; in9[7] = a1.w; in9[8] = a2.x;
#pragma unroll
      for (int k = 0; k < 9; ++k) any = any || in9[k] != 0.0f;
    } else {
      const long long* sref = b.gsum54 + item * 54;
      const float sc = 1.0f / 65536.0f;
      in9[3] = (float)sref[0] * sc;
      in9[4] = (float)sref[1] * sc; in9[5] = (float)sref[2] * sc; in9[6] = (float)sref[3] * sc;
      in9[7] = (float)sref[4] * sc; in9[8] = (float)sref[5] * sc;
#pragma unroll
      for (int k = 0; k < 9; ++k) any = any || in9[k] != 0.0f;
      for (int k = 0; k < 48; ++k) {
        const long long q = sref[6 + k];
        any = any || q != 0;
        if (need_sh_grads) s_gsh[k][t] += (float)q * sc;
      }
    }
    if (stats) {
      const float n2d = sqrtf(in9[7] * in9[7] + in9[8] * in9[8]);
      float nc = in9[4] * in9[4] + in9[5] * in9[5];
      nc = sqrtf(nc + in9[6] * in9[6]);
      if (n2d > 1e-10f || nc > 1e-10f) {
        acc.x = acc.x + n2d;
        acc.y = 0.0f;
        acc.z = acc.z + nc;
        acc.w = acc.w + 1.0f;
      }
    }
    if (!any) continue;
    // an item with tiles passed the preprocess's culling with these same
    // parameters, so only the camera-space mean, the view direction and the
    // colour are formed again
    const ViewInfo& vi = s_views[v];
    float pc[4];
    view_position(get, vi, pc);
    ProjOut o;
    view_color(get, pc, deg, !ref, o);
    geom_view(pc, o, vi, sp, gc.C3, in9, !ref, &s_sh[0][t], kGeomThreads, deg, gr, g3);
    if (need_sh_grads && !ref) {
      float Y[16];
      sh_basis(o.dir[0], o.dir[1], o.dir[2], deg, Y);
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        const float dr = o.raw[c] > 0.0f ? in9[c] : 0.0f;
#pragma unroll
        for (int k = 0; k < 16; ++k)
          if (k < ncoef) s_gsh[3 * k + c][t] += Y[k] * dr;
      }
    }
  }
  if (stats) {
    reinterpret_cast<float4*>(b.importance)[g] = imp;
    reinterpret_cast<float4*>(b.densify_accum)[g] = acc;
  }
  geom_cov_final(prm, g3, gr);
  float g11[11] = {gr.pos[0], gr.pos[1], gr.pos[2], gr.ls[0], gr.ls[1], gr.ls[2],
                   gr.q[0],   gr.q[1],   gr.q[2],   gr.q[3],  gr.logit};
  if (sp.write_grads) {
#pragma unroll
    for (int k = 0; k < 11; ++k) b.grads[(size_t)k * stride + g] = g11[k];
    for (int k = 0; k < 48; ++k) b.grads[(size_t)(11 + k) * stride + g] = s_gsh[k][t];
  }
  if (sp.apply_adam) {
    const AdamK ak = adam_consts(sp);
    const float lr_pos = sp.lr_pos, lr_scale = sp.lr_scale, lr_rot = sp.lr_rot, lr_op = sp.lr_opacity;
    const float lr_sh = sp.lr_sh;
    adam_planes<11>(b, stride, 0, g,
                    Vals<11>{{g11[0], g11[1], g11[2], g11[3], g11[4], g11[5], g11[6], g11[7], g11[8],
                              g11[9], g11[10]}},
                    Vals<11>{{lr_pos, lr_pos, lr_pos, lr_scale, lr_scale, lr_scale, lr_rot, lr_rot,
                              lr_rot, lr_rot, lr_op}}, ak);
    if (sp.sh_update) {
#pragma unroll
      for (int k0 = 0; k0 < 48; k0 += 12) {
        Vals<12> gv, lv;
#pragma unroll
        for (int j = 0; j < 12; ++j) { gv.v[j] = s_gsh[k0 + j][t]; lv.v[j] = lr_sh; }
        adam_planes<12>(b, stride, 11 + k0, g, gv, lv, ak);
      }
    }
  }
}

}  // namespace

// ---------------------------------------------------------------------------
// Launchers
// ---------------------------------------------------------------------------
void launch_preprocess(const DevBuffers& b, uint32_t n, uint32_t views, cudaStream_t s) {
  // the step's cameras in dynamic shared memory (3 KB for 16 views: 8 blocks
  // of 27 KB stay resident per multiprocessor)
  k_preprocess<<<(n + kPrepThreads - 1) / kPrepThreads, kPrepThreads, views * sizeof(ViewInfo), s>>>(b);
}

void launch_scan(const DevBuffers& b, uint32_t n_items, cudaStream_t s) {
  const uint32_t nb = (n_items + kScanTile - 1) / kScanTile;
  if (nb == 0) return;
  k_scan_reduce<<<nb, kScanThreads, 0, s>>>(b, n_items);
  k_scan_blocks<<<1, 1024, 0, s>>>(b, nb);
  k_scan_final<<<nb, kScanThreads, 0, s>>>(b, n_items);
}

uint32_t scan_block_count(uint32_t n_items) { return (n_items + kScanTile - 1) / kScanTile; }

void launch_group_bounds(const DevBuffers& b, cudaStream_t s) { k_group_bounds<<<1, 64, 0, s>>>(b); }

void launch_emit(const DevBuffers& b, uint32_t n, uint32_t views, cudaStream_t s) {
  dim3 grid((n + 255) / 256, views);
  k_emit<<<grid, 256, 0, s>>>(b);
}

void launch_ranges(const DevBuffers& b, uint32_t icap, cudaStream_t s) {
  if (icap) {
    const uint32_t blocks = min((icap / 4 + 255) / 256 + 1, (uint32_t)sm_count() * 8);
    k_ranges<<<blocks, 256, 0, s>>>(b);
  }
  k_ranges_empty<<<1, 256, 0, s>>>(b);
}

// Zeroes the partials the last backward did not write (unflagged), for a
// read-back of the buffer.
__global__ void __launch_bounds__(256) k_partials_fill(DevBuffers b, uint32_t total) {
  for (uint32_t e = blockIdx.x * blockDim.x + threadIdx.x; e < total; e += gridDim.x * blockDim.x)
    if (b.reached[e] == 0u) {
      float4* dst = b.partials + (size_t)e * kPartialF4;
      dst[0] = dst[1] = dst[2] = make_float4(0.f, 0.f, 0.f, 0.f);
    }
}

void launch_partials_fill(const DevBuffers& b, uint32_t total, cudaStream_t s) {
  if (!total) return;
  const uint32_t blocks = min((total + 255) / 256, (uint32_t)sm_count() * 16);
  k_partials_fill<<<blocks, 256, 0, s>>>(b, total);
}

void launch_flatten_fill(const DevBuffers& b, uint32_t total, cudaStream_t s) {
  if (!total) return;
  const uint32_t blocks = min((total + 255) / 256, (uint32_t)sm_count() * 16);
  k_flatten_fill<<<blocks, 256, 0, s>>>(b, total);
}

template <int TS>
void launch_forward_ts(const DevBuffers& b, uint32_t max_tiles, uint32_t fb, bool count,
                       cudaStream_t s) {
  if (TS == 16 && count && (fb == 0 || fb == (uint32_t)kFwdBatch)) {
    k_forward<TS, kFwdBatch, true><<<max_tiles, TS * TS, 0, s>>>(b);
    return;
  }
  switch (fb) {
    case 64: k_forward<TS, 64><<<max_tiles, TS * TS, 0, s>>>(b); break;
    case 128: k_forward<TS, 128><<<max_tiles, TS * TS, 0, s>>>(b); break;
    default: k_forward<TS, kFwdBatch><<<max_tiles, TS * TS, 0, s>>>(b); break;
  }
}

void launch_forward(const DevBuffers& b, uint32_t max_tiles, uint32_t ts, uint32_t fb, bool ssim,
                    uint32_t views, uint32_t max_view_pixels, bool count, cudaStream_t s) {
  if (max_tiles == 0) return;
  switch (ts) {
    case 8: launch_forward_ts<8>(b, max_tiles, fb, false, s); break;
    case 32: launch_forward_ts<32>(b, max_tiles, fb, false, s); break;
    default: launch_forward_ts<16>(b, max_tiles, fb, count, s); break;
  }
  if (ssim) {
    dim3 grid((max_view_pixels + 255) / 256, views);
    k_ssim<<<grid, 256, 0, s>>>(b);
  }
}

void launch_loss_final(const DevBuffers& b, cudaStream_t s) { k_loss_final<<<1, 1024, 0, s>>>(b); }

void launch_backward(const DevBuffers& b, uint32_t max_tiles, uint32_t ts, uint32_t bb, bool ref,
                     bool count, cudaStream_t s) {
  if (max_tiles == 0) return;
  if (!ref) {
    switch (ts) {
      case 8: k_backward_exact<8><<<max_tiles, 64, 0, s>>>(b); break;
      case 32: k_backward_exact<32><<<max_tiles, 1024, 0, s>>>(b); break;
      default:
        if (count && (bb == 0 || bb == kBwdBatch16)) {
          k_backward_exact2<kBwdBatch16, true><<<max_tiles, 128, 0, s>>>(b);
          break;
        }
        switch (bb) {
          case 32: k_backward_exact2<32><<<max_tiles, 128, 0, s>>>(b); break;
          case 128: k_backward_exact2<128><<<max_tiles, 128, 0, s>>>(b); break;
          default: k_backward_exact2<kBwdBatch16><<<max_tiles, 128, 0, s>>>(b); break;
        }
        break;
    }
  } else {
    switch (ts) {
      case 8: k_backward_ref<8><<<max_tiles, 64, 0, s>>>(b); break;
      case 32: k_backward_ref<32><<<max_tiles, 1024, 0, s>>>(b); break;
      default: k_backward_ref<16><<<max_tiles, 256, 0, s>>>(b); break;
    }
  }
}

void launch_geom_adam(const DevBuffers& b, uint32_t n, cudaStream_t s) {
  if (n == 0) return;
  // per device: the opt-in above 48 KB of shared memory (idempotent, so two
  // threads that both see it unset both set it)
  static std::atomic<bool> smem_set[64];
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) dev = 0;
  if (!smem_set[dev].load(std::memory_order_acquire)) {
    cudaFuncSetAttribute(k_geom_adam, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kGeomSmem);
    smem_set[dev].store(true, std::memory_order_release);
  }
  k_geom_adam<<<(n + kGeomThreads - 1) / kGeomThreads, kGeomThreads, kGeomSmem, s>>>(b);
}

void launch_item_sums(const DevBuffers& b, uint64_t items, cudaStream_t s) {
  if (items == 0) return;
  const uint64_t blocks = std::min<uint64_t>((items + 255) / 256, (uint64_t)sm_count() * 16);
  k_item_sums<<<(uint32_t)blocks, 256, 0, s>>>(b);
}

}  // namespace sky
