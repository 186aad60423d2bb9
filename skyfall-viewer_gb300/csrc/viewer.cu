// Headless viewer render: the reference's frame() path -- preprocess
// (preprocess.wgsl:116-215), a global depth sort (radix_sort.wgsl), one
// screen-space quad per splat (gaussian.wgsl:15-52) blended back to front
// with src-alpha / one-minus-src-alpha (gaussian-renderer.ts:863-868) into a
// cleared target -- as CUDA kernels writing an f32 RGBA device buffer.
//
// The quads are binned into 16x16 pixel tiles in depth order, and every
// pixel blends, in that order, each splat whose quad covers its centre: the
// same sequence of blend operations the rasterizer performs per pixel, so
// the result matches a per-quad CPU restatement bit for bit.  Coverage is
// tested at pixel centres in f32 with the top-left rule (left and top quad
// edges inside); a hardware rasterizer snaps quad corners to its sub-pixel
// grid, so pixels within that snap of a quad edge can differ from it.
#include "sky_math.cuh"
#include "viewer.cuh"

namespace sky {
namespace {

SKY_DEV float load_param(const float* P, uint32_t stride, int plane, uint32_t g, bool r16) {
  const float v = P[(size_t)plane * stride + g];
  return r16 ? round_f16(v) : v;
}

// float_to_ordered_uint (preprocess.wgsl:101-105) of -z_camera: ascending key
// = far to near.
SKY_DEV uint32_t ordered_key(float x) {
  const uint32_t bits = __float_as_uint(x);
  const uint32_t mask = (bits & 0x80000000u) ? 0xFFFFFFFFu : 0x80000000u;
  return bits ^ mask;
}

__global__ void __launch_bounds__(256)
k_viewer_project(ViewerParams vp, const float* __restrict__ P, float4* __restrict__ splats,
                 uint32_t* __restrict__ keys, uint32_t* __restrict__ counts,
                 uint2* __restrict__ rects, unsigned long long* __restrict__ total) {
  const uint32_t g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= vp.n) return;
  const bool r16 = vp.round_f16 != 0;
  auto get = [&](int plane) { return load_param(P, vp.plane_stride, plane, g, r16); };
  keys[g] = 0xFFFFFFFFu;
  counts[g] = 0u;
  rects[g] = make_uint2(0u, 0u);
  const float px = get(0), py = get(1), pz = get(2);
  float pc[4];
#pragma unroll
  for (int r = 0; r < 4; ++r) pc[r] = mat4_row(vp.view, r, px, py, pz, 1.0f);
  float clip[4];
#pragma unroll
  for (int r = 0; r < 4; ++r) clip[r] = mat4_row(vp.proj, r, pc[0], pc[1], pc[2], pc[3]);
  const float w = clip[3];
  const float ndc_x = clip[0] / w, ndc_y = clip[1] / w;
  if (fabsf(ndc_x) > 1.2f || fabsf(ndc_y) > 1.2f || pc[2] < 0.0f) return;
  const float opacity = 1.0f / (1.0f + sky_expf(-get(10)));
  float sig[3];
#pragma unroll
  for (int k = 0; k < 3; ++k)
    sig[k] = vp.gaussian_scaling * sky_expf(clampf_(get(3 + k), -10.0f, 10.0f));
  const float q0 = get(6), q1 = get(7), q2 = get(8), q3 = get(9);
  float qq = q0 * q0 + q1 * q1;
  qq = qq + q2 * q2;
  qq = qq + q3 * q3;
  const float ql = sqrtf(qq);
  const float rx = q0 / ql, ry = q1 / ql, rz = q2 / ql, rw = q3 / ql;
  float R[3][3];  // WGSL column-major R[col][row] (quat_to_mat3, :100-107)
  R[0][0] = 1.0f - 2.0f * (ry * ry + rz * rz);
  R[0][1] = 2.0f * (rx * ry - rw * rz);
  R[0][2] = 2.0f * (rx * rz + rw * ry);
  R[1][0] = 2.0f * (rx * ry + rw * rz);
  R[1][1] = 1.0f - 2.0f * (rx * rx + rz * rz);
  R[1][2] = 2.0f * (ry * rz - rw * rx);
  R[2][0] = 2.0f * (rx * rz - rw * ry);
  R[2][1] = 2.0f * (ry * rz + rw * rx);
  R[2][2] = 1.0f - 2.0f * (rx * rx + ry * ry);
  // C3D = transpose(S R) S R with S = diag(scaling * sigma)
  float A[3][3];
#pragma unroll
  for (int j = 0; j < 3; ++j)
#pragma unroll
    for (int r = 0; r < 3; ++r) A[j][r] = (sig[j] * R[r][j]) * sig[j];
  float C3[3][3];
#pragma unroll
  for (int j = 0; j < 3; ++j)
#pragma unroll
    for (int r = 0; r < 3; ++r) {
      float acc = A[0][r] * R[j][0];
      acc = acc + A[1][r] * R[j][1];
      acc = acc + A[2][r] * R[j][2];
      C3[j][r] = acc;
    }
  // C2D = T C3D T^T with T = J Rwc (J as the WGSL constructor lays it out)
  const float tx = pc[0], ty = pc[1], tz = pc[2];
  const float fx = vp.focal[0], fy = vp.focal[1];
  const float tz2 = tz * tz;
  const float J00 = fx / tz, J11 = fy / tz;
  const float J02 = -(fx * tx) / tz2, J12 = -(fy * ty) / tz2;
  float T[3][3];
#pragma unroll
  for (int j = 0; j < 3; ++j) {
    const float v0 = vp.view[j * 4 + 0], v1 = vp.view[j * 4 + 1];
    T[j][0] = J00 * v0;
    T[j][1] = J11 * v1;
    T[j][2] = J02 * v0 + J12 * v1;
  }
  float B0[3], B1[3];
#pragma unroll
  for (int j = 0; j < 3; ++j) {
    float a0 = T[0][0] * C3[j][0];
    a0 = a0 + T[1][0] * C3[j][1];
    a0 = a0 + T[2][0] * C3[j][2];
    B0[j] = a0;
    float a1 = T[0][1] * C3[j][0];
    a1 = a1 + T[1][1] * C3[j][1];
    a1 = a1 + T[2][1] * C3[j][2];
    B1[j] = a1;
  }
  float c00 = B0[0] * T[0][0];
  c00 = c00 + B0[1] * T[1][0];
  c00 = c00 + B0[2] * T[2][0];
  float c11 = B1[0] * T[0][1];
  c11 = c11 + B1[1] * T[1][1];
  c11 = c11 + B1[2] * T[2][1];
  float c01 = B1[0] * T[0][0];
  c01 = c01 + B1[1] * T[1][0];
  c01 = c01 + B1[2] * T[2][0];
  c00 = c00 + 0.3f;
  c11 = c11 + 0.3f;
  const float det = c00 * c11 - c01 * c01;
  if (det <= 0.0f) return;
  const float det_inv = 1.0f / det;
  const float ca = c11 * det_inv, cb = (-c01) * det_inv, cc = c00 * det_inv;
  const float v0 = -pc[0], v1 = -pc[1], v2 = -pc[2];
  float vv = v0 * v0 + v1 * v1;
  vv = vv + v2 * v2;
  const float vl = sqrtf(vv);
  const float d0 = v0 / vl, d1 = v1 / vl, d2 = v2 / vl;
  float col[3];
  const int deg = (int)min(vp.sh_deg, 3u);
  auto sh = [&](int k, int c) { return get(11 + 3 * k + c); };
  sh_color_raw(sh, d0, d1, d2, deg, col);
#pragma unroll
  for (int c = 0; c < 3; ++c) col[c] = fmax_(0.0f, col[c]);
  const float mid = 0.5f * (c00 + c11);
  const float disc = sqrtf(fmax_(mid * mid - det, 0.0f));
  const float l1 = mid + disc, l2 = mid - disc;
  const float radius = ceilf(3.0f * sqrtf(fmax_(l1, l2)));
  const float cx = (ndc_x * 0.5f + 0.5f) * vp.viewport[0];
  const float cy = (ndc_y * -0.5f + 0.5f) * vp.viewport[1];
  splats[(size_t)g * 3 + 0] = make_float4(cx, cy, ca, cb);
  splats[(size_t)g * 3 + 1] = make_float4(cc, opacity, col[0], col[1]);
  splats[(size_t)g * 3 + 2] = make_float4(col[2], radius, 0.0f, 0.0f);
  keys[g] = ordered_key(-pc[2]);
  // tiles holding a pixel centre the quad may cover (one pixel of margin
  // each side; the raster kernel tests coverage exactly)
  const float X0 = cx - radius, X1 = cx + radius, Y0 = cy - radius, Y1 = cy + radius;
  if (!(X1 > 0.0f) || !(Y1 > 0.0f) || !(X0 < (float)vp.width) || !(Y0 < (float)vp.height)) return;
  // clamped in f32 before the conversions (the bounds may be huge or infinite)
  const int xlo = (int)fmax_(floorf(X0 - 0.5f) - 1.0f, 0.0f);
  const int ylo = (int)fmax_(floorf(Y0 - 0.5f) - 1.0f, 0.0f);
  const int xhi = (int)fmin_(ceilf(X1 - 0.5f) + 1.0f, (float)vp.width - 1.0f);
  const int yhi = (int)fmin_(ceilf(Y1 - 0.5f) + 1.0f, (float)vp.height - 1.0f);
  if (xhi < xlo || yhi < ylo) return;
  const uint32_t tx0 = (uint32_t)xlo / kViewTile, tx1 = (uint32_t)xhi / kViewTile + 1;
  const uint32_t ty0 = (uint32_t)ylo / kViewTile, ty1 = (uint32_t)yhi / kViewTile + 1;
  const uint32_t cnt = (tx1 - tx0) * (ty1 - ty0);
  counts[g] = cnt;
  rects[g] = make_uint2(tx0 | (ty0 << 16), tx1 | (ty1 << 16));
  atomicAdd(total, (unsigned long long)cnt);
}

__global__ void k_viewer_gather_counts(const uint32_t* __restrict__ order,
                                       const uint32_t* __restrict__ counts, uint32_t n,
                                       uint32_t* __restrict__ out) {
  const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n) out[k] = counts[order[k]];
}

__global__ void __launch_bounds__(256)
k_viewer_emit(ViewerParams vp, const uint32_t* __restrict__ order, const uint32_t* __restrict__ cum,
              const uint32_t* __restrict__ counts_sorted, const uint2* __restrict__ rects,
              uint32_t n, uint32_t* __restrict__ tile_keys, uint32_t* __restrict__ gidx) {
  const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  const uint32_t c = counts_sorted[k];
  if (c == 0) return;
  const uint32_t g = order[k];
  const uint2 rc = rects[g];
  const uint32_t x0 = rc.x & 0xFFFFu, y0 = rc.x >> 16, x1 = rc.y & 0xFFFFu, y1 = rc.y >> 16;
  uint32_t o = cum[k] - c;
  for (uint32_t ty = y0; ty < y1; ++ty)
    for (uint32_t tx = x0; tx < x1; ++tx) {
      tile_keys[o] = ty * vp.tiles_x + tx;
      gidx[o] = g;
      ++o;
    }
}

__global__ void k_viewer_ranges(const uint32_t* __restrict__ keys, uint32_t total, uint32_t tiles,
                                uint32_t* __restrict__ offsets) {
  const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t > tiles) return;
  uint32_t lo = 0, hi = total;  // first index with key >= t
  while (lo < hi) {
    const uint32_t mid = lo + ((hi - lo) >> 1);
    if (keys[mid] < t) lo = mid + 1;
    else hi = mid;
  }
  offsets[t] = t == tiles ? total : lo;
}

constexpr int kViewBatch = 256;

__global__ void __launch_bounds__(kViewTile* kViewTile)
k_viewer_raster(ViewerParams vp, const float4* __restrict__ splats,
                const uint32_t* __restrict__ offsets, const uint32_t* __restrict__ gidx,
                float4* __restrict__ rgba) {
  __shared__ float4 s_sp[kViewBatch * 3];
  const uint32_t tile = blockIdx.x;
  const uint32_t tx = tile % vp.tiles_x, ty = tile / vp.tiles_x;
  const uint32_t tid = threadIdx.x;
  const uint32_t x = tx * kViewTile + tid % kViewTile, y = ty * kViewTile + tid / kViewTile;
  const bool inside = x < vp.width && y < vp.height;
  const float pxf = (float)x + 0.5f, pyf = (float)y + 0.5f;
  const uint32_t start = offsets[tile], end = offsets[tile + 1];
  float C0 = 0.0f, C1 = 0.0f, C2 = 0.0f, A = 0.0f;  // cleared to transparent black
  for (uint32_t bs = start; bs < end; bs += kViewBatch) {
    const uint32_t cnt = min((uint32_t)kViewBatch, end - bs);
    __syncthreads();
    for (uint32_t k = tid; k < cnt; k += kViewTile * kViewTile) {
      const size_t g = gidx[bs + k];
      s_sp[k * 3 + 0] = splats[g * 3 + 0];
      s_sp[k * 3 + 1] = splats[g * 3 + 1];
      s_sp[k * 3 + 2] = splats[g * 3 + 2];
    }
    __syncthreads();
    if (!inside) continue;
    for (uint32_t k = 0; k < cnt; ++k) {
      const float4 q0 = s_sp[k * 3 + 0];
      const float4 q2 = s_sp[k * 3 + 2];
      const float r = q2.y;
      if (!(pxf >= q0.x - r && pxf < q0.x + r && pyf >= q0.y - r && pyf < q0.y + r)) continue;
      const float4 q1 = s_sp[k * 3 + 1];
      const float dx = pxf - q0.x, dy = pyf - q0.y;
      float s = 0.5f * ((q0.z * dx) * dx + (q1.x * dy) * dy);
      s = s + (q0.w * dx) * dy;
      if (s < 0.0f) continue;  // discard
      const float a = clampf_(q1.y * sky_expf(-s), 0.0f, 1.0f);
      const float om = 1.0f - a;
      C0 = q1.z * a + C0 * om;
      C1 = q1.w * a + C1 * om;
      C2 = q2.x * a + C2 * om;
      A = a + A * om;
    }
  }
  if (inside) rgba[(size_t)y * vp.width + x] = make_float4(C0, C1, C2, A);
}

uint32_t blocks(uint32_t n, uint32_t t) { return (n + t - 1) / t; }

}  // namespace

void launch_viewer_project(const ViewerParams& vp, const float* params, float4* splats,
                           uint32_t* keys, uint32_t* counts, uint2* rects,
                           unsigned long long* total, cudaStream_t s) {
  if (vp.n)
    k_viewer_project<<<blocks(vp.n, 256), 256, 0, s>>>(vp, params, splats, keys, counts, rects, total);
}

void launch_viewer_gather_counts(const uint32_t* order, const uint32_t* counts, uint32_t n,
                                 uint32_t* counts_sorted, cudaStream_t s) {
  if (n) k_viewer_gather_counts<<<blocks(n, 256), 256, 0, s>>>(order, counts, n, counts_sorted);
}

void launch_viewer_emit(const ViewerParams& vp, const uint32_t* order, const uint32_t* cum,
                        const uint32_t* counts_sorted, const uint2* rects, uint32_t n,
                        uint32_t* tile_keys, uint32_t* gidx, cudaStream_t s) {
  if (n)
    k_viewer_emit<<<blocks(n, 256), 256, 0, s>>>(vp, order, cum, counts_sorted, rects, n, tile_keys,
                                                 gidx);
}

void launch_viewer_ranges(const uint32_t* tile_keys, uint32_t total, uint32_t tiles,
                          uint32_t* offsets, cudaStream_t s) {
  k_viewer_ranges<<<blocks(tiles + 1, 256), 256, 0, s>>>(tile_keys, total, tiles, offsets);
}

void launch_viewer_raster(const ViewerParams& vp, const float4* splats, const uint32_t* offsets,
                          const uint32_t* gidx, float4* rgba, cudaStream_t s) {
  const uint32_t tiles = vp.tiles_x * vp.tiles_y;
  if (tiles)
    k_viewer_raster<<<tiles, kViewTile * kViewTile, 0, s>>>(vp, splats, offsets, gidx, rgba);
}

}  // namespace sky
