// TEST INFRASTRUCTURE ONLY -- the parity oracle.  Nothing in the product
// (the skyfall library, its Python host mirror) links, imports or calls this
// file; only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg
// load it, and there only as the checker or as the timed CPU baseline.
//
// A CPU restatement, in C++, of the Gaussian-splat training hot path of
// krispy-kenay/Skyfall-Viewer (TypeScript + WGSL).  Each function cites the
// reference file:line it follows.  Semantics that WGSL leaves to the
// implementation are pinned here and mirrored by the CUDA kernels:
//   * every f32 operation is a separate IEEE operation in source order
//     (compiled with -ffp-contract=off; matrix/vector products sum their
//     terms in ascending index order);
//   * exp() is sky_expf below (Cody-Waite reduction + degree-7 Taylor
//     polynomial, within 2 ulp of exp), so alpha thresholds decide the
//     same way on the CPU and the GPU;
//   * normalize(v) = v / sqrt(dot(v, v));
//   * f32 -> u32/i32 conversions truncate toward zero and saturate (WGSL),
//     NaN -> 0;
//   * pack2x16float rounds to nearest even.
// Parity status: the reference ships no tests, fixtures or golden vectors,
// and its WGSL cannot run on this hardware (no WebGPU runtime), so this
// oracle is "parity unpinned" against the reference's own outputs; it is
// pinned instead by analytic known-answer tests (tests/test_oracle.py) and
// FP64 finite differences of its loss.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <thread>
#include <vector>

namespace {

inline uint32_t f2u(float f) { uint32_t u; std::memcpy(&u, &f, 4); return u; }
inline float u2f(uint32_t u) { float f; std::memcpy(&f, &u, 4); return f; }

// ---------------------------------------------------------------------------
// Scalar primitives
// ---------------------------------------------------------------------------

// exp(x): Cody-Waite range reduction x = k ln2 + r, |r| <= ln2/2, then a
// degree-7 Taylor polynomial of e^r by Horner with fused multiply-adds, then
// scaling by 2^k through the exponent bits.  Defined on [-87, 88]; returns 0
// below and +inf above.
float sky_expf(float x) {
  if (x != x) return x;
  if (x > 88.0f) return INFINITY;
  if (x < -87.0f) return 0.0f;
  const float kLog2e = 1.44269502f;       // float(log2(e))
  const float kLn2Hi = 0.693147182f;      // float(ln 2)
  const float kLn2Lo = -1.90465421e-09f;  // ln 2 - kLn2Hi
  const float kRound = 12582912.0f;       // 1.5 * 2^23
  float t = x * kLog2e;
  float u = t + kRound;
  float k = u - kRound;
  float r = std::fmaf(-k, kLn2Hi, x);
  r = std::fmaf(-k, kLn2Lo, r);
  float p = 1.98412701e-04f;                // 1/5040
  p = std::fmaf(p, r, 1.38888892e-03f);     // 1/720
  p = std::fmaf(p, r, 8.33333377e-03f);     // 1/120
  p = std::fmaf(p, r, 4.16666679e-02f);     // 1/24
  p = std::fmaf(p, r, 1.66666672e-01f);     // 1/6
  p = std::fmaf(p, r, 0.5f);
  p = std::fmaf(p, r, 1.0f);
  p = std::fmaf(p, r, 1.0f);
  uint32_t kbits = f2u(u) - f2u(kRound);  // k as two's complement
  return u2f(f2u(p) + (kbits << 23));
}

// log(x): x = m 2^e, m in [sqrt(1/2), sqrt(2)); log m = 2 atanh(s) with
// s = (m - 1) / (m + 1), odd series to s^11 by Horner in s^2 with fused
// multiply-adds; log x = e ln2 (split hi/lo) + log m.  Within 2 ulp.
float sky_logf(float x) {
  if (x != x || x < 0.0f) return NAN;
  if (x == 0.0f) return -INFINITY;
  if (x == INFINITY) return x;
  uint32_t b = f2u(x);
  int e = 0;
  if (b < 0x00800000u) {
    x = x * 8388608.0f;
    b = f2u(x);
    e = -23;
  }
  e += (int)(b >> 23) - 127;
  float m = u2f((b & 0x007FFFFFu) | 0x3F800000u);
  if (m > 1.41421354f) {
    m = m * 0.5f;
    e += 1;
  }
  const float s = (m - 1.0f) / (m + 1.0f);
  const float z = s * s;
  float p = 0.181818187f;
  p = std::fmaf(p, z, 0.222222224f);
  p = std::fmaf(p, z, 0.285714298f);
  p = std::fmaf(p, z, 0.400000006f);
  p = std::fmaf(p, z, 0.666666687f);
  const float lm = std::fmaf(s * z, p, 2.0f * s);
  const float fe = (float)e;
  return std::fmaf(fe, 0.693147182f, std::fmaf(fe, -1.90465421e-09f, lm));
}

// f32 -> f16 -> f32 with round-to-nearest-even (pack2x16float/unpack2x16float).
float round_f16(float f) {
  uint32_t x = f2u(f);
  uint32_t sign = x & 0x80000000u;
  uint32_t ax = x & 0x7FFFFFFFu;
  if (ax >= 0x7F800000u) return f;                        // inf, nan
  if (ax >= 0x477FF000u) return u2f(sign | 0x7F800000u);  // >= 65520 -> inf
  if (ax < 0x38800000u) {                                 // f16 subnormal range
    float q = std::nearbyint(std::fabs(f) * 16777216.0f);  // units of 2^-24
    float v = q * 5.9604644775390625e-08f;
    return sign ? -v : v;
  }
  uint32_t lsb = (ax >> 13) & 1u;
  ax = (ax + 0x0FFFu + lsb) & ~0x1FFFu;
  return u2f(sign | ax);
}

uint32_t wgsl_u32(float f) {
  if (!(f > 0.0f)) return 0u;
  if (f >= 4294967296.0f) return 0xFFFFFFFFu;
  return (uint32_t)f;
}
uint32_t wgsl_u32(double f) {
  if (!(f > 0.0)) return 0u;
  if (f >= 4294967296.0) return 0xFFFFFFFFu;
  return (uint32_t)f;
}
int32_t wgsl_i32(float f) {
  if (f != f) return 0;
  if (f >= 2147483648.0f) return INT32_MAX;
  if (f <= -2147483648.0f) return INT32_MIN;
  return (int32_t)f;
}

inline float ex(float x) { return sky_expf(x); }
inline double ex(double x) { return std::exp(x); }
inline float sq(float x) { return std::sqrt(x); }
inline double sq(double x) { return std::sqrt(x); }

// SH constants (common.wgsl:1-18), as f32.
const float SH_C0 = 0.28209479177387814f;
const float SH_C1 = 0.4886025119029199f;
const float SH_C2[5] = {1.0925484305920792f, -1.0925484305920792f, 0.31539156525252005f,
                        -1.0925484305920792f, 0.5462742152960396f};
const float SH_C3[7] = {-0.5900435899266435f, 2.890611442640554f, -0.4570457994644658f,
                        0.3731763325901154f, -0.4570457994644658f, 1.445305721320277f,
                        -0.5900435899266435f};

const float MIN_ALPHA = 1.0f / 255.0f;   // training-forward-tiles.wgsl:38-41
const float MAX_ALPHA = 0.999f;
const float T_THRESH = 1e-4f;

// ---------------------------------------------------------------------------
// Shared settings (mirrors the fields of SkyConfig the oracle needs)
// ---------------------------------------------------------------------------
struct Cam {          // SkyCamera
  float view[16];
  float proj[16];
  float focal[2];
  uint32_t width, height;
};

struct Settings {
  uint32_t tile_size;
  float near_plane, far_plane, radius_clip, eps2d;
  float bg[3];
  float w_l2, w_l1, w_ssim;
  uint32_t round_f16;
  uint32_t nthreads;
};

template <typename F>
struct Rec {
  F mean[2], conic[3], opacity, color[3], depth, radius;
  F raw[3];       // colour before the clamp (for the adjoint)
  F dir[3];       // normalize(-p_cam): SH evaluation direction
  uint32_t count, rect[4];
};

template <typename Fn>
void parallel_for(uint32_t n, uint32_t nthreads, Fn fn) {
  if (nthreads <= 1 || n < 64) {
    for (uint32_t i = 0; i < n; ++i) fn(i);
    return;
  }
  std::atomic<uint32_t> next(0);
  std::vector<std::thread> th;
  const uint32_t chunk = std::max<uint32_t>(1, n / (nthreads * 16));
  for (uint32_t t = 0; t < nthreads; ++t) {
    th.emplace_back([&]() {
      for (;;) {
        uint32_t b = next.fetch_add(chunk);
        if (b >= n) break;
        uint32_t e = std::min(n, b + chunk);
        for (uint32_t i = b; i < e; ++i) fn(i);
      }
    });
  }
  for (auto& t : th) t.join();
}

// ---------------------------------------------------------------------------
// Projection: training-tiles.wgsl:40-180 (project_gaussians_for_tiling) with
// the SH colour of training-forward-tiles.wgsl:65-105 / preprocess.wgsl:69-99
// and the sigmoid of training-forward-tiles.wgsl:188.
// ---------------------------------------------------------------------------
template <typename F>
void sh_color(const F* sh /*48, index 3k+c*/, F dx, F dy, F dz, int deg, F out_raw[3]) {
  const F C0 = (F)SH_C0, C1 = (F)SH_C1;
  for (int ch = 0; ch < 3; ++ch) out_raw[ch] = C0 * sh[ch];
  if (deg > 0) {
    F x = dx, y = dy, z = dz;
    F a1 = (-C1) * y, a2 = C1 * z, a3 = C1 * x;
    for (int ch = 0; ch < 3; ++ch) {
      F t = a1 * sh[3 + ch] + a2 * sh[6 + ch];
      t = t - a3 * sh[9 + ch];
      out_raw[ch] = out_raw[ch] + t;
    }
    if (deg > 1) {
      F xx = x * x, yy = y * y, zz = z * z;
      F xy = x * y, yz = y * z, xz = x * z;
      F b4 = (F)SH_C2[0] * xy;
      F b5 = (F)SH_C2[1] * yz;
      F b6 = (F)SH_C2[2] * (((F)2.0 * zz - xx) - yy);
      F b7 = (F)SH_C2[3] * xz;
      F b8 = (F)SH_C2[4] * (xx - yy);
      for (int ch = 0; ch < 3; ++ch) {
        F t = b4 * sh[12 + ch] + b5 * sh[15 + ch];
        t = t + b6 * sh[18 + ch];
        t = t + b7 * sh[21 + ch];
        t = t + b8 * sh[24 + ch];
        out_raw[ch] = out_raw[ch] + t;
      }
      if (deg > 2) {
        F c9 = ((F)SH_C3[0] * y) * ((F)3.0 * xx - yy);
        F c10 = ((F)SH_C3[1] * xy) * z;
        F c11 = ((F)SH_C3[2] * y) * (((F)4.0 * zz - xx) - yy);
        F c12 = ((F)SH_C3[3] * z) * (((F)2.0 * zz - (F)3.0 * xx) - (F)3.0 * yy);
        F c13 = ((F)SH_C3[4] * x) * (((F)4.0 * zz - xx) - yy);
        F c14 = ((F)SH_C3[5] * z) * (xx - yy);
        F c15 = ((F)SH_C3[6] * x) * (xx - (F)3.0 * yy);
        for (int ch = 0; ch < 3; ++ch) {
          F t = c9 * sh[27 + ch] + c10 * sh[30 + ch];
          t = t + c11 * sh[33 + ch];
          t = t + c12 * sh[36 + ch];
          t = t + c13 * sh[39 + ch];
          t = t + c14 * sh[42 + ch];
          t = t + c15 * sh[45 + ch];
          out_raw[ch] = out_raw[ch] + t;
        }
      }
    }
  }
  for (int ch = 0; ch < 3; ++ch) out_raw[ch] = out_raw[ch] + (F)0.5;
}

// WGSL M * v for a column-major 4x4 matrix: columns combined in index order.
template <typename F>
void mat4_vec(const float* m, const F v[4], F out[4]) {
  for (int r = 0; r < 4; ++r) {
    F acc = (F)m[0 * 4 + r] * v[0];
    acc = acc + (F)m[1 * 4 + r] * v[1];
    acc = acc + (F)m[2 * 4 + r] * v[2];
    acc = acc + (F)m[3 * 4 + r] * v[3];
    out[r] = acc;
  }
}

template <typename F>
F load_param(const float* P, uint64_t stride, uint32_t plane, uint32_t i, bool r16) {
  float v = P[(uint64_t)plane * stride + i];
  return (F)(r16 ? round_f16(v) : v);
}

template <typename F>
F load_param_d(const F* P, uint64_t stride, uint32_t plane, uint32_t i) {
  return P[(uint64_t)plane * stride + i];
}

// Camera-space position, as p_cam = view * (p, 1).
template <typename F>
void cam_space(const Cam& cam, const F p[3], F pc[4]) {
  F pw[4] = {p[0], p[1], p[2], (F)1.0};
  mat4_vec<F>(cam.view, pw, pc);
}

template <typename F, typename Src>
void project_one(Src&& get, const Cam& cam, const Settings& s, int sh_deg, Rec<F>& o) {
  o.count = 0;
  o.radius = 0;
  o.depth = 0;
  o.rect[0] = o.rect[1] = o.rect[2] = o.rect[3] = 0;
  o.mean[0] = o.mean[1] = 0;
  o.dir[0] = o.dir[1] = o.dir[2] = 0;
  o.conic[0] = o.conic[1] = o.conic[2] = 0;
  o.opacity = 0;
  o.color[0] = o.color[1] = o.color[2] = 0;
  o.raw[0] = o.raw[1] = o.raw[2] = 0;

  F p[3] = {get(0), get(1), get(2)};
  F pc[4];
  cam_space<F>(cam, p, pc);
  F clip[4];
  mat4_vec<F>(cam.proj, pc, clip);
  F w = clip[3];
  F ndc_x = clip[0] / w, ndc_y = clip[1] / w;
  // training-tiles.wgsl:67-80
  if (std::fabs(ndc_x) > (F)1.2f || std::fabs(ndc_y) > (F)1.2f || pc[2] <= (F)0.0) return;
  F depth = pc[2];
  if (depth < (F)s.near_plane || depth > (F)s.far_plane) return;

  // :82-98 scale and rotation
  F ls[3];
  for (int k = 0; k < 3; ++k) ls[k] = std::min(std::max(get(3 + k), (F)-10.0), (F)10.0);
  F sig[3] = {ex(ls[0]), ex(ls[1]), ex(ls[2])};
  F q[4] = {get(6), get(7), get(8), get(9)};
  F qq = q[0] * q[0] + q[1] * q[1];
  qq = qq + q[2] * q[2];
  qq = qq + q[3] * q[3];
  F qlen = sq(qq);
  for (int k = 0; k < 4; ++k) q[k] = q[k] / qlen;
  F rx = q[0], ry = q[1], rz = q[2], rw = q[3];
  // quat_to_mat3_tiling (:30-37), WGSL column-major: R[col][row]
  F R[3][3];
  R[0][0] = (F)1.0 - (F)2.0 * (ry * ry + rz * rz);
  R[0][1] = (F)2.0 * (rx * ry - rw * rz);
  R[0][2] = (F)2.0 * (rx * rz + rw * ry);
  R[1][0] = (F)2.0 * (rx * ry + rw * rz);
  R[1][1] = (F)1.0 - (F)2.0 * (rx * rx + rz * rz);
  R[1][2] = (F)2.0 * (ry * rz - rw * rx);
  R[2][0] = (F)2.0 * (rx * rz - rw * ry);
  R[2][1] = (F)2.0 * (ry * rz + rw * rx);
  R[2][2] = (F)1.0 - (F)2.0 * (rx * rx + ry * ry);
  // C3D = transpose(S * R) * S * R (:101); SR[j][r] = sig[r] * R[j][r];
  // A = transpose(SR) * S, A[j][r] = SR[r][j] * sig[j]; C3D = A * R.
  F A[3][3];
  for (int j = 0; j < 3; ++j)
    for (int r = 0; r < 3; ++r) A[j][r] = (sig[j] * R[r][j]) * sig[j];
  F C3[3][3];
  for (int j = 0; j < 3; ++j)
    for (int r = 0; r < 3; ++r) {
      F acc = A[0][r] * R[j][0];
      acc = acc + A[1][r] * R[j][1];
      acc = acc + A[2][r] * R[j][2];
      C3[j][r] = acc;
    }
  // J (:106-110), Rwc (:112), T = J * Rwc (:113)
  F tx = pc[0], ty = pc[1], tz = pc[2];
  F fx = (F)cam.focal[0], fy = (F)cam.focal[1];
  F tz2 = tz * tz;
  F J00 = fx / tz, J11 = fy / tz;
  F J02 = -(fx * tx) / tz2, J12 = -(fy * ty) / tz2;  // J[0][2], J[1][2]
  F T[3][3];  // T[j][r]
  for (int j = 0; j < 3; ++j) {
    F v0 = (F)cam.view[j * 4 + 0], v1 = (F)cam.view[j * 4 + 1];
    T[j][0] = J00 * v0;
    T[j][1] = J11 * v1;
    T[j][2] = J02 * v0 + J12 * v1;
  }
  // C2D = T * C3D * transpose(T) (:115); B = T * C3D, B[j][r] = sum_k T[k][r] C3[j][k]
  F B0[3], B1[3];  // B[j][0], B[j][1]
  for (int j = 0; j < 3; ++j) {
    F a0 = T[0][0] * C3[j][0];
    a0 = a0 + T[1][0] * C3[j][1];
    a0 = a0 + T[2][0] * C3[j][2];
    B0[j] = a0;
    F a1 = T[0][1] * C3[j][0];
    a1 = a1 + T[1][1] * C3[j][1];
    a1 = a1 + T[2][1] * C3[j][2];
    B1[j] = a1;
  }
  // C2D[j][r] = sum_k B[k][r] * T[k][j]
  F c00 = B0[0] * T[0][0];
  c00 = c00 + B0[1] * T[1][0];
  c00 = c00 + B0[2] * T[2][0];
  F c11 = B1[0] * T[0][1];
  c11 = c11 + B1[1] * T[1][1];
  c11 = c11 + B1[2] * T[2][1];
  F c01 = B1[0] * T[0][0];  // C2D[0][1] = column 0, row 1
  c01 = c01 + B1[1] * T[1][0];
  c01 = c01 + B1[2] * T[2][0];
  c00 = c00 + (F)s.eps2d;
  c11 = c11 + (F)s.eps2d;
  F det = c00 * c11 - c01 * c01;
  if (det <= (F)0.0) return;
  F mid = (F)0.5 * (c00 + c11);
  F disc = sq(std::max(mid * mid - det, (F)0.0));
  F l1 = mid + disc, l2 = mid - disc;
  F radius = std::ceil((F)3.0 * sq(std::max(l1, l2)));
  if (radius > (F)s.radius_clip || radius < (F)1.0) return;
  F det_inv = (F)1.0 / det;
  o.conic[0] = c11 * det_inv;
  o.conic[1] = (-c01) * det_inv;
  o.conic[2] = c00 * det_inv;
  F W = (F)(float)cam.width, H = (F)(float)cam.height;
  o.mean[0] = ((F)0.5 * (ndc_x + (F)1.0)) * W;
  o.mean[1] = ((F)0.5 * (ndc_y + (F)1.0)) * H;
  o.radius = radius;
  o.depth = depth;
  // :161-179 tile rectangle
  F ts = (F)(float)s.tile_size;
  uint32_t TW = (cam.width + s.tile_size - 1) / s.tile_size;
  uint32_t TH = (cam.height + s.tile_size - 1) / s.tile_size;
  F tile_x = o.mean[0] / ts, tile_y = o.mean[1] / ts;
  F trx = radius / ts;
  uint32_t x0 = std::min(wgsl_u32(std::floor(tile_x - trx)), TW);
  uint32_t y0 = std::min(wgsl_u32(std::floor(tile_y - trx)), TH);
  uint32_t x1 = std::min(wgsl_u32(std::ceil(tile_x + trx)), TW);
  uint32_t y1 = std::min(wgsl_u32(std::ceil(tile_y + trx)), TH);
  int32_t nx = (int32_t)x1 - (int32_t)x0, ny = (int32_t)y1 - (int32_t)y0;
  o.count = (nx <= 0 || ny <= 0) ? 0u : (uint32_t)(nx * ny);
  o.rect[0] = x0; o.rect[1] = y0; o.rect[2] = x1; o.rect[3] = y1;
  // opacity (training-forward-tiles.wgsl:188) and colour (:185-190)
  F logit = get(10);
  o.opacity = (F)1.0 / ((F)1.0 + ex(-logit));
  F v[3] = {-pc[0], -pc[1], -pc[2]};
  F vv = v[0] * v[0] + v[1] * v[1];
  vv = vv + v[2] * v[2];
  F vl = sq(vv);
  F d[3] = {v[0] / vl, v[1] / vl, v[2] / vl};
  o.dir[0] = d[0]; o.dir[1] = d[1]; o.dir[2] = d[2];
  F sh[48];
  for (int k = 0; k < 48; ++k) sh[k] = get(11 + k);
  sh_color<F>(sh, d[0], d[1], d[2], sh_deg, o.raw);
  for (int c = 0; c < 3; ++c) o.color[c] = std::max((F)0.0, o.raw[c]);
}

uint32_t tiles_w(const Cam& c, const Settings& s) { return (c.width + s.tile_size - 1) / s.tile_size; }
uint32_t tiles_h(const Cam& c, const Settings& s) { return (c.height + s.tile_size - 1) / s.tile_size; }

// Key of one intersection: (tile << 16) | u32(clamp(depth, 0, 65535)) & 0xFFFF.
// encode_isect_key (training-tiles.wgsl:193-199) with camera 0 and a tile
// field wide enough for the view (identical to the 12-bit field when the
// view has at most 4096 tiles).
uint32_t isect_key(uint32_t tile, float depth) {
  float dc = std::min(std::max(depth, 0.0f), 65535.0f);
  return (tile << 16) | (wgsl_u32(dc) & 0xFFFFu);
}

// ---------------------------------------------------------------------------
// Forward: training-forward-tiles.wgsl:107-215 for one pixel.
// ---------------------------------------------------------------------------
template <typename F>
struct PixOut {
  F rgb[3];
  F alpha;
  F tprod;   // transmittance as the running product of (1 - alpha)
  uint32_t last;
};

template <typename F>
void forward_pixel(const Rec<F>* rec, const uint32_t* flat, uint32_t start, uint32_t end,
                   F px, F py, const Settings& s, PixOut<F>& o, uint64_t* sig) {
  F col[3] = {0, 0, 0};
  F alpha = 0;
  F tp = 1;
  uint32_t last = start;
  for (uint32_t i = start; i < end; ++i) {
    last = i;
    const Rec<F>& g = rec[flat[i]];
    F dx = px - g.mean[0], dy = py - g.mean[1];
    F s1 = (g.conic[0] * dx) * dx;
    F s2 = (g.conic[2] * dy) * dy;
    F so2 = (F)0.5 * (s1 + s2);
    so2 = so2 + (g.conic[1] * dx) * dy;
    if (so2 < (F)0.0) continue;
    F G = ex(-so2);
    F al = g.opacity * G;
    F a = std::min(al, (F)MAX_ALPHA);
    if (a < (F)MIN_ALPHA) continue;
    if (sig) *sig = (*sig * 1099511628211ull) ^ (uint64_t)(i + 1);
    F om = (F)1.0 - alpha;
    F ca = a * om;
    for (int c = 0; c < 3; ++c) col[c] = col[c] + g.color[c] * ca;
    alpha = alpha + ca;
    tp = tp * ((F)1.0 - a);
    if ((F)1.0 - alpha < (F)T_THRESH) break;
  }
  F T = (F)1.0 - alpha;
  for (int c = 0; c < 3; ++c) o.rgb[c] = col[c] + T * (F)s.bg[c];
  o.alpha = alpha;
  o.tprod = tp;
  o.last = last;
}

// ---------------------------------------------------------------------------
// Loss: training-loss.wgsl:86-126 (+ the SSIM pseudo-gradient :33-84).
// ---------------------------------------------------------------------------
float sign_f(float x) { return x > 0.0f ? 1.0f : (x < 0.0f ? -1.0f : 0.0f); }

}  // namespace

// ===========================================================================
// C interface (ctypes)
// ===========================================================================
extern "C" {

struct OrcCam { float view[16]; float proj[16]; float focal[2]; uint32_t width, height; };
struct OrcSettings {
  uint32_t tile_size;
  float near_plane, far_plane, radius_clip, eps2d;
  float bg[3];
  float w_l2, w_l1, w_ssim;
  uint32_t round_f16;
  uint32_t nthreads;
};

static Cam to_cam(const OrcCam* c) {
  Cam r;
  std::memcpy(&r, c, sizeof(Cam));
  return r;
}
static Settings to_set(const OrcSettings* s) {
  Settings r;
  std::memcpy(&r, s, sizeof(Settings));
  if (r.nthreads == 0) r.nthreads = 1;
  return r;
}

void orc_expf(const float* x, float* y, uint64_t n) {
  for (uint64_t i = 0; i < n; ++i) y[i] = sky_expf(x[i]);
}
void orc_round_f16(const float* x, float* y, uint64_t n) {
  for (uint64_t i = 0; i < n; ++i) y[i] = round_f16(x[i]);
}
void orc_logf(const float* x, float* y, uint64_t n) {
  for (uint64_t i = 0; i < n; ++i) y[i] = sky_logf(x[i]);
}

// knn_init (knn-init.wgsl:40-90) by brute force, as the reference runs it:
// positions read through f16, the three smallest distances to the other
// points (insert_sorted, strict <, starting at 1e10), their mean, sigma =
// min(clamp(max(mean / 3, bias), lo, hi), 0.1) with lo / hi / bias =
// extent x (0.0007, 0.007, 0.0015) in f32, log sigma stored through f16.
// Outputs per point: density (mean distance) and the f16 log sigma.
void orc_knn_init(const float* params, uint64_t stride, uint32_t n, float extent, float* density,
                  float* log_sigma, uint32_t nthreads) {
  std::vector<float> pos((size_t)n * 3);
  for (uint32_t i = 0; i < n; ++i)
    for (int k = 0; k < 3; ++k) pos[(size_t)i * 3 + k] = round_f16(params[(uint64_t)k * stride + i]);
  const float lo_s = extent * 0.0007f, hi_s = extent * 0.007f, bias = extent * 0.0015f;
  parallel_for(n, nthreads, [&](uint32_t i) {
    float d[3] = {1e10f, 1e10f, 1e10f};
    const float* p = &pos[(size_t)i * 3];
    for (uint32_t j = 0; j < n; ++j) {
      if (j == i) continue;
      const float* q = &pos[(size_t)j * 3];
      const float dx = p[0] - q[0], dy = p[1] - q[1], dz = p[2] - q[2];
      float s = dx * dx + dy * dy;
      s = s + dz * dz;
      const float dist = std::sqrt(s);
      if (dist < d[0]) {
        d[2] = d[1];
        d[1] = d[0];
        d[0] = dist;
      } else if (dist < d[1]) {
        d[2] = d[1];
        d[1] = dist;
      } else if (dist < d[2]) {
        d[2] = dist;
      }
    }
    const float mean = ((d[0] + d[1]) + d[2]) / 3.0f;
    float sig = std::max(mean / 3.0f, bias);
    sig = std::min(std::max(sig, lo_s), hi_s);
    sig = std::min(sig, 0.1f);
    if (density) density[i] = mean;
    log_sigma[i] = round_f16(sky_logf(std::max(sig, 1e-6f)));
  });
}

// Projection of n Gaussians for one camera.  rec12: 12 f32 per Gaussian
// (mean x, y, conic a, b, c, opacity, colour r, g, b, depth, radius, 0);
// rect: 4 u32 per Gaussian (x0, y0, x1, y1); counts: tiles per Gaussian.
int orc_project(const float* params, uint64_t stride, uint32_t n, const OrcCam* cam_in,
                const OrcSettings* s_in, int sh_deg, float* rec12, uint32_t* counts,
                uint32_t* rects, float* raw3, float* dirs3) {
  Cam cam = to_cam(cam_in);
  Settings s = to_set(s_in);
  bool r16 = s.round_f16 != 0;
  parallel_for(n, s.nthreads, [&](uint32_t i) {
    Rec<float> o;
    auto get = [&](uint32_t plane) { return load_param<float>(params, stride, plane, i, r16); };
    project_one<float>(get, cam, s, sh_deg, o);
    float* r = rec12 + (uint64_t)i * 12;
    r[0] = o.mean[0]; r[1] = o.mean[1];
    r[2] = o.conic[0]; r[3] = o.conic[1]; r[4] = o.conic[2];
    r[5] = o.opacity;
    r[6] = o.color[0]; r[7] = o.color[1]; r[8] = o.color[2];
    r[9] = o.depth; r[10] = o.radius; r[11] = 0.0f;
    counts[i] = o.count;
    for (int k = 0; k < 4; ++k) rects[(uint64_t)i * 4 + k] = o.rect[k];
    if (raw3)
      for (int k = 0; k < 3; ++k) raw3[(uint64_t)i * 3 + k] = o.raw[k];
    if (dirs3)
      for (int k = 0; k < 3; ++k) dirs3[(uint64_t)i * 3 + k] = o.dir[k];
  });
  return 0;
}

// Host cumsum (gaussian-renderer.ts:1814-1828), emission (training-tiles.wgsl:
// 202-247), stable sort (radix_sort.wgsl, an LSD radix sort, is stable) and
// tile offsets with the backward min-fill (training-tiles.wgsl:250-271,
// gaussian-renderer.ts:1966-2020).  Arrays of size n_isect must be allocated
// by the caller (n_isect = sum of counts).
int orc_tiles(const float* rec12, const uint32_t* counts, const uint32_t* rects, uint32_t n,
              const OrcCam* cam_in, const OrcSettings* s_in, uint32_t* cumsum,
              uint32_t* keys_emit, uint32_t* gidx_emit, uint32_t* keys_sorted,
              uint32_t* gidx_sorted, uint32_t* offsets) {
  Cam cam = to_cam(cam_in);
  Settings s = to_set(s_in);
  uint32_t TW = tiles_w(cam, s), TH = tiles_h(cam, s), T = TW * TH;
  uint64_t run = 0;
  for (uint32_t i = 0; i < n; ++i) {
    run += counts[i];
    cumsum[i] = (uint32_t)run;
  }
  uint64_t I = run;
  for (uint32_t i = 0; i < n; ++i) {
    if (counts[i] == 0) continue;
    uint64_t cur = i == 0 ? 0 : cumsum[i - 1];
    const uint32_t* rc = rects + (uint64_t)i * 4;
    float depth = rec12[(uint64_t)i * 12 + 9];
    for (uint32_t ty = rc[1]; ty < rc[3]; ++ty)
      for (uint32_t tx = rc[0]; tx < rc[2]; ++tx) {
        keys_emit[cur] = isect_key(ty * TW + tx, depth);
        gidx_emit[cur] = i;
        ++cur;
      }
  }
  std::vector<uint32_t> perm(I);
  for (uint64_t k = 0; k < I; ++k) perm[k] = (uint32_t)k;
  std::stable_sort(perm.begin(), perm.end(),
                   [&](uint32_t a, uint32_t b) { return keys_emit[a] < keys_emit[b]; });
  for (uint64_t k = 0; k < I; ++k) {
    keys_sorted[k] = keys_emit[perm[k]];
    gidx_sorted[k] = gidx_emit[perm[k]];
  }
  for (uint32_t t = 0; t <= T; ++t) offsets[t] = (uint32_t)I;
  for (uint64_t k = 0; k < I; ++k) {
    uint32_t tile = keys_sorted[k] >> 16;
    if (tile < T) offsets[tile] = std::min(offsets[tile], (uint32_t)k);
  }
  for (int t = (int)T - 1; t >= 0; --t) offsets[t] = std::min(offsets[t], offsets[t + 1]);
  return 0;
}

static std::vector<Rec<float>> recs_from12(const float* rec12, uint32_t n) {
  std::vector<Rec<float>> r(n);
  for (uint32_t i = 0; i < n; ++i) {
    const float* q = rec12 + (uint64_t)i * 12;
    Rec<float>& o = r[i];
    o.mean[0] = q[0]; o.mean[1] = q[1];
    o.conic[0] = q[2]; o.conic[1] = q[3]; o.conic[2] = q[4];
    o.opacity = q[5];
    o.color[0] = q[6]; o.color[1] = q[7]; o.color[2] = q[8];
    o.depth = q[9]; o.radius = q[10];
  }
  return r;
}

// Forward raster of one view.  rgba: 4 f32 per pixel (alpha channel 1.0 as
// the reference's rgba32float texture); last: 0xFFFFFFFF on empty tiles (the
// reference leaves those unwritten); tprod: final transmittance as the
// product of (1 - alpha) over the composited splats (exact-mode backward).
int orc_forward(const float* rec12, uint32_t n, const OrcCam* cam_in, const OrcSettings* s_in,
                const uint32_t* gidx_sorted, const uint32_t* offsets, float* rgba, float* alpha,
                uint32_t* last, float* tprod) {
  Cam cam = to_cam(cam_in);
  Settings s = to_set(s_in);
  auto rec = recs_from12(rec12, n);
  uint32_t TW = tiles_w(cam, s);
  parallel_for(cam.height, s.nthreads, [&](uint32_t y) {
    for (uint32_t x = 0; x < cam.width; ++x) {
      uint32_t tile = (y / s.tile_size) * TW + (x / s.tile_size);
      uint32_t start = offsets[tile], end = offsets[tile + 1];
      uint64_t p = (uint64_t)y * cam.width + x;
      if (start >= end) {
        for (int c = 0; c < 3; ++c) rgba[p * 4 + c] = s.bg[c];
        rgba[p * 4 + 3] = 1.0f;
        alpha[p] = 0.0f;
        last[p] = 0xFFFFFFFFu;
        if (tprod) tprod[p] = 1.0f;
        continue;
      }
      PixOut<float> o;
      forward_pixel<float>(rec.data(), gidx_sorted, start, end, (float)x + 0.5f,
                           (float)y + 0.5f, s, o, nullptr);
      for (int c = 0; c < 3; ++c) rgba[p * 4 + c] = o.rgb[c];
      rgba[p * 4 + 3] = 1.0f;
      alpha[p] = o.alpha;
      last[p] = o.last;
      if (tprod) tprod[p] = o.tprod;
    }
  });
  return 0;
}

// Loss of one view.  target: 3 f32 per pixel.  residual: 4 f32 per pixel
// (dL/dC r, g, b, 0).  loss: sum of 0.5 w_l2 r^2 + w_l1 |r| (f64).
int orc_loss(const float* rgba, const float* target, const OrcCam* cam_in,
             const OrcSettings* s_in, float* residual, double* loss) {
  Cam cam = to_cam(cam_in);
  Settings s = to_set(s_in);
  const int W = (int)cam.width, H = (int)cam.height;
  double total = 0.0;
  auto pred = [&](int x, int y, int c) {
    x = std::min(std::max(x, 0), W - 1);
    y = std::min(std::max(y, 0), H - 1);
    return rgba[((uint64_t)y * W + x) * 4 + c];
  };
  auto targ = [&](int x, int y, int c) {
    x = std::min(std::max(x, 0), W - 1);
    y = std::min(std::max(y, 0), H - 1);
    return target[((uint64_t)y * W + x) * 3 + c];
  };
  for (int y = 0; y < H; ++y)
    for (int x = 0; x < W; ++x) {
      uint64_t p = (uint64_t)y * W + x;
      float g[3];
      for (int c = 0; c < 3; ++c) {
        float diff = rgba[p * 4 + c] - target[p * 3 + c];
        g[c] = s.w_l2 * diff + s.w_l1 * sign_f(diff);
        total += 0.5 * (double)s.w_l2 * (double)diff * (double)diff +
                 (double)s.w_l1 * std::fabs((double)diff);
      }
      if (s.w_ssim > 0.0f) {
        // computeSSIMGrad (training-loss.wgsl:33-84)
        // WGSL const-expressions 0.01 * 0.01 and 0.03 * 0.03 are evaluated
        // exactly and rounded to f32 once.
        const float C1 = 0.0001f, C2 = 0.0009f, nwin = 25.0f;
        for (int c = 0; c < 3; ++c) {
          float mx = 0.0f, my = 0.0f;
          for (int dy = -2; dy <= 2; ++dy)
            for (int dx = -2; dx <= 2; ++dx) {
              mx = mx + pred(x + dx, y + dy, c);
              my = my + targ(x + dx, y + dy, c);
            }
          mx = mx / nwin;
          my = my / nwin;
          float sx = 0.0f, sy = 0.0f, sxy = 0.0f;
          for (int dy = -2; dy <= 2; ++dy)
            for (int dx = -2; dx <= 2; ++dx) {
              float a = pred(x + dx, y + dy, c) - mx;
              float b = targ(x + dx, y + dy, c) - my;
              sx = sx + a * a;
              sy = sy + b * b;
              sxy = sxy + a * b;
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
          float gs = dssim * (pred(x, y, c) - targ(x, y, c));
          g[c] = g[c] + s.w_ssim * gs;
        }
      }
      for (int c = 0; c < 3; ++c) residual[p * 4 + c] = g[c];
      residual[p * 4 + 3] = 0.0f;
    }
  *loss = total;
  return 0;
}

// ---------------------------------------------------------------------------
// Backward of one view.
//  mode 0 (exact): per pair the quantities of backward-tiles-local.wgsl:
//    296-362 without the alpha > 0.98 skip, with a zero alpha-gradient when
//    the alpha clamp at 0.999 is active, traversing each pixel's list back
//    to front from the product transmittance tprod (not 1 - alpha, which
//    loses relative precision as alpha -> 1).  Outputs per Gaussian the sums (f64) and absolute sums of
//    9 values: dL/dcolour r,g,b, dL/dlogit, dL/dconic a,b,c, dL/dmean x,y.
//  mode 1 (reference): backward-tiles-local.wgsl:185-382 literally --
//    batches of 64 ascending, each batch back to front, alpha > 0.98
//    skipped, every value truncated to i32 fixed point (x65536) and summed
//    per (tile, intersection) in 54 slots (TILE_GRAD layout :43-47);
//    tile_grads: 54 i32 per sorted intersection; gsum: 54 i64 per Gaussian,
//    the exact sums of backward-reduce.wgsl:35-71's inputs.
// ---------------------------------------------------------------------------
static void sh_basis(float x, float y, float z, int deg, float Y[16]) {
  for (int k = 0; k < 16; ++k) Y[k] = 0.0f;
  Y[0] = SH_C0;
  if (deg > 0) { Y[1] = -SH_C1 * y; Y[2] = SH_C1 * z; Y[3] = -SH_C1 * x; }
  if (deg > 1) {
    float xx = x * x, yy = y * y, zz = z * z, xy = x * y, yz = y * z, xz = x * z;
    Y[4] = SH_C2[0] * xy;
    Y[5] = SH_C2[1] * yz;
    Y[6] = SH_C2[2] * ((2.0f * zz - xx) - yy);
    Y[7] = SH_C2[3] * xz;
    Y[8] = SH_C2[4] * (xx - yy);
    if (deg > 2) {
      Y[9] = (SH_C3[0] * y) * (3.0f * xx - yy);
      Y[10] = (SH_C3[1] * xy) * z;
      Y[11] = (SH_C3[2] * y) * ((4.0f * zz - xx) - yy);
      Y[12] = (SH_C3[3] * z) * ((2.0f * zz - 3.0f * xx) - 3.0f * yy);
      Y[13] = (SH_C3[4] * x) * ((4.0f * zz - xx) - yy);
      Y[14] = (SH_C3[5] * z) * (xx - yy);
      Y[15] = (SH_C3[6] * x) * (xx - 3.0f * yy);
    }
  }
}

int orc_backward(const float* rec12, uint32_t n, const OrcCam* cam_in, const OrcSettings* s_in,
                 int mode, int sh_deg, const float* dirs3, const uint32_t* gidx_sorted,
                 const uint32_t* offsets, const float* alpha_img, const uint32_t* last_img,
                 const float* tprod_img, const float* residual, double* gsum9, double* gabs9, int32_t* tile_grads,
                 int64_t* gsum54) {
  Cam cam = to_cam(cam_in);
  Settings s = to_set(s_in);
  auto rec = recs_from12(rec12, n);
  const uint32_t TW = tiles_w(cam, s), TH = tiles_h(cam, s), T = TW * TH;
  const uint32_t ts = s.tile_size;
  const uint32_t I = offsets[T];
  if (mode == 0) {
    std::fill(gsum9, gsum9 + (uint64_t)n * 9, 0.0);
    std::fill(gabs9, gabs9 + (uint64_t)n * 9, 0.0);
  } else {
    std::fill(tile_grads, tile_grads + (uint64_t)I * 54, 0);
  }
  // Per-intersection accumulators (each intersection belongs to one tile),
  // so tiles can run in parallel without sharing.
  std::vector<double> isum, iabs;
  if (mode == 0) {
    isum.assign((uint64_t)I * 9, 0.0);
    iabs.assign((uint64_t)I * 9, 0.0);
  }
  parallel_for(T, s.nthreads, [&](uint32_t tile) {
    uint32_t start = offsets[tile], end = offsets[tile + 1];
    if (start >= end) return;
    uint32_t tx = tile % TW, ty = tile / TW;
    for (uint32_t ly = 0; ly < ts; ++ly)
      for (uint32_t lx = 0; lx < ts; ++lx) {
        uint32_t x = tx * ts + lx, y = ty * ts + ly;
        if (x >= cam.width || y >= cam.height) continue;
        uint64_t p = (uint64_t)y * cam.width + x;
        uint32_t binf = last_img[p];
        if (binf < start) continue;
        float res[3] = {residual[p * 4 + 0], residual[p * 4 + 1], residual[p * 4 + 2]};
        float Tc = mode == 0 ? tprod_img[p] : 1.0f - alpha_img[p];
        float acc[3] = {s.bg[0], s.bg[1], s.bg[2]};
        float px = (float)x + 0.5f, py = (float)y + 0.5f;
        auto visit = [&](uint32_t i) {
          uint32_t gi = gidx_sorted[i];
          const Rec<float>& g = rec[gi];
          float dx = px - g.mean[0], dy = py - g.mean[1];
          float s1 = (g.conic[0] * dx) * dx;
          float s2 = (g.conic[2] * dy) * dy;
          float so2 = 0.5f * (s1 + s2);
          so2 = so2 + (g.conic[1] * dx) * dy;
          if (so2 < 0.0f) return;
          float G = sky_expf(-so2);
          float al = g.opacity * G;
          float a = std::min(al, MAX_ALPHA);
          if (a < MIN_ALPHA) return;
          if (mode == 1 && a > 0.98f) return;
          float om = std::max(1.0f - a, 0.0001f);
          float Tb = Tc / om;
          float contrib = a * Tb;
          float fg = res[0] * g.color[0] + res[1] * g.color[1];
          fg = fg + res[2] * g.color[2];
          float bgt = res[0] * acc[0] + res[1] * acc[1];
          bgt = bgt + res[2] * acc[2];
          float dLda = (fg - bgt) * Tb;
          float dlogit = (dLda * a) * (1.0f - g.opacity);
          float dLdG = dLda * g.opacity;
          if (mode == 0 && al > MAX_ALPHA) { dlogit = 0.0f; dLdG = 0.0f; }
          float dLds = dLdG * (-G);
          float ca = ((dLds * 0.5f) * dx) * dx;
          float cb = (dLds * dx) * dy;
          float cc = ((dLds * 0.5f) * dy) * dy;
          float ddx = dLds * ((g.conic[0] * dx) + (g.conic[1] * dy));
          float ddy = dLds * ((g.conic[1] * dx) + (g.conic[2] * dy));
          if (mode == 0) {
            float v[9] = {res[0] * contrib, res[1] * contrib, res[2] * contrib, dlogit,
                          ca, cb, cc, -ddx, -ddy};
            for (int k = 0; k < 9; ++k) {
              isum[(uint64_t)i * 9 + k] += (double)v[k];
              iabs[(uint64_t)i * 9 + k] += std::fabs((double)v[k]);
            }
          } else {
            int32_t* tg = tile_grads + (uint64_t)i * 54;
            auto add = [&](int slot, float v) {
              tg[slot] = (int32_t)((uint32_t)tg[slot] + (uint32_t)wgsl_i32(v * 65536.0f));
            };
            float rs[3] = {res[0] * contrib, res[1] * contrib, res[2] * contrib};
            const float* d = dirs3 + (uint64_t)gi * 3;
            float xd = d[0], yd = d[1], zd = d[2];
            // wg_accumulate_sh_grads (backward-tiles-local.wgsl:104-183)
            auto put = [&](int k, float coef) {
              for (int c = 0; c < 3; ++c) add(6 + 3 * k + c, coef * rs[c]);
            };
            put(0, SH_C0);
            if (sh_deg > 0) {
              put(1, -SH_C1 * yd);
              put(2, SH_C1 * zd);
              put(3, -SH_C1 * xd);
              if (sh_deg > 1) {
                float xx = xd * xd, yy = yd * yd, zz = zd * zd;
                float xy = xd * yd, yz = yd * zd, xz = xd * zd;
                put(4, SH_C2[0] * xy);
                put(5, SH_C2[1] * yz);
                put(6, SH_C2[2] * ((2.0f * zz - xx) - yy));
                put(7, SH_C2[3] * xz);
                put(8, SH_C2[4] * (xx - yy));
                if (sh_deg > 2) {
                  put(9, (SH_C3[0] * yd) * (3.0f * xx - yy));
                  put(10, (SH_C3[1] * xy) * zd);
                  put(11, (SH_C3[2] * yd) * ((4.0f * zz - xx) - yy));
                  put(12, (SH_C3[3] * zd) * ((2.0f * zz - 3.0f * xx) - 3.0f * yy));
                  put(13, (SH_C3[4] * xd) * ((4.0f * zz - xx) - yy));
                  put(14, (SH_C3[5] * zd) * (xx - yy));
                  put(15, (SH_C3[6] * xd) * (xx - 3.0f * yy));
                }
              }
            }
            add(0, dlogit);
            add(1, ca);
            add(2, cb);
            add(3, cc);
            add(4, -ddx);
            add(5, -ddy);
          }
          for (int c = 0; c < 3; ++c) acc[c] = a * g.color[c] + (1.0f - a) * acc[c];
          Tc = Tb;
        };
        if (mode == 0) {
          uint32_t hi = std::min(binf, end - 1);
          for (int64_t i = (int64_t)hi; i >= (int64_t)start; --i) visit((uint32_t)i);
        } else {
          uint32_t nb = (end - start + 63) / 64;
          for (uint32_t b = 0; b < nb; ++b) {
            uint32_t bs = start + b * 64;
            uint32_t be = std::min(bs + 64, end);
            uint32_t pe = std::min(be, binf + 1);
            for (int64_t i = (int64_t)pe - 1; i >= (int64_t)bs; --i) visit((uint32_t)i);
          }
        }
      }
  });
  if (mode == 0) {
    for (uint32_t i = 0; i < I; ++i) {
      uint32_t gi = gidx_sorted[i];
      for (int k = 0; k < 9; ++k) {
        gsum9[(uint64_t)gi * 9 + k] += isum[(uint64_t)i * 9 + k];
        gabs9[(uint64_t)gi * 9 + k] += iabs[(uint64_t)i * 9 + k];
      }
    }
  } else {
    std::fill(gsum54, gsum54 + (uint64_t)n * 54, (int64_t)0);
    for (uint32_t i = 0; i < I; ++i) {
      uint32_t gi = gidx_sorted[i];
      for (int k = 0; k < 54; ++k) gsum54[(uint64_t)gi * 54 + k] += tile_grads[(uint64_t)i * 54 + k];
    }
  }
  return 0;
}

// ---------------------------------------------------------------------------
// Exact adjoint of the projection for one view: from the per-Gaussian sums
// of (dL/dcolour, dL/dlogit, dL/dconic, dL/dmean) to the 59 parameter
// planes, accumulated (+=) into grads.  Differentiates the forward as
// implemented (training-tiles.wgsl:40-180, incl. its perspective-free 2D
// covariance) with straight-through f16 rounding.  sh_deg: active degree;
// with_sh == 0 skips the SH planes (steps that do not update them).
// ---------------------------------------------------------------------------
int orc_geom(const float* params, uint64_t stride, uint32_t n, const OrcCam* cam_in,
             const OrcSettings* s_in, int sh_deg, int with_sh, const float* g9, float* grads,
             uint64_t gstride) {
  Cam cam = to_cam(cam_in);
  Settings s = to_set(s_in);
  bool r16 = s.round_f16 != 0;
  parallel_for(n, s.nthreads, [&](uint32_t i) {
    const float* gi = g9 + (uint64_t)i * 9;
    bool any = false;
    for (int k = 0; k < 9; ++k) any = any || gi[k] != 0.0f;
    if (!any) return;
    auto get = [&](uint32_t plane) { return load_param<float>(params, stride, plane, i, r16); };
    Rec<float> o;
    project_one<float>(get, cam, s, sh_deg, o);
    if (o.radius == 0.0f) return;
    double P[3] = {get(0), get(1), get(2)};
    double V[4][4];
    for (int j = 0; j < 4; ++j)
      for (int r = 0; r < 4; ++r) V[j][r] = cam.view[j * 4 + r];  // V[col][row]
    double pc[3];
    for (int r = 0; r < 3; ++r) pc[r] = V[0][r] * P[0] + V[1][r] * P[1] + V[2][r] * P[2] + V[3][r];
    double dpc[3] = {0, 0, 0};
    // mean: ndc = clip.xy / clip.w, clip = proj * (pc, 1)
    double Pm[4][4];
    for (int j = 0; j < 4; ++j)
      for (int r = 0; r < 4; ++r) Pm[j][r] = cam.proj[j * 4 + r];
    double clip[4];
    for (int r = 0; r < 4; ++r) clip[r] = Pm[0][r] * pc[0] + Pm[1][r] * pc[1] + Pm[2][r] * pc[2] + Pm[3][r];
    double ndx = clip[0] / clip[3], ndy = clip[1] / clip[3];
    double hW = 0.5 * cam.width, hH = 0.5 * cam.height;
    for (int j = 0; j < 3; ++j) {
      dpc[j] += gi[7] * hW * (Pm[j][0] - ndx * Pm[j][3]) / clip[3];
      dpc[j] += gi[8] * hH * (Pm[j][1] - ndy * Pm[j][3]) / clip[3];
    }
    // covariance
    double ls[3], sig[3], lsg[3];
    for (int k = 0; k < 3; ++k) {
      double raw = get(3 + k);
      ls[k] = std::min(std::max(raw, -10.0), 10.0);
      sig[k] = std::exp(ls[k]);
      lsg[k] = (raw > -10.0 && raw < 10.0) ? 1.0 : 0.0;
    }
    double qr[4] = {get(6), get(7), get(8), get(9)};
    double ql = std::sqrt(qr[0] * qr[0] + qr[1] * qr[1] + qr[2] * qr[2] + qr[3] * qr[3]);
    double q[4] = {qr[0] / ql, qr[1] / ql, qr[2] / ql, qr[3] / ql};
    double x = q[0], y = q[1], z = q[2], w = q[3];
    double R[3][3] = {{1 - 2 * (y * y + z * z), 2 * (x * y - w * z), 2 * (x * z + w * y)},
                      {2 * (x * y + w * z), 1 - 2 * (x * x + z * z), 2 * (y * z - w * x)},
                      {2 * (x * z - w * y), 2 * (y * z + w * x), 1 - 2 * (x * x + y * y)}};
    double M[3][3];  // R S
    for (int a = 0; a < 3; ++a)
      for (int b = 0; b < 3; ++b) M[a][b] = R[a][b] * sig[b];
    double C3[3][3];
    for (int a = 0; a < 3; ++a)
      for (int b = 0; b < 3; ++b) {
        double t = 0;
        for (int k = 0; k < 3; ++k) t += M[a][k] * M[b][k];
        C3[a][b] = t;
      }
    double V3[3][3];  // math matrix rows
    for (int r = 0; r < 3; ++r)
      for (int j = 0; j < 3; ++j) V3[r][j] = V[j][r];
    double Wm[3][3];  // V3 C3 V3^T
    double tmp[3][3];
    for (int a = 0; a < 3; ++a)
      for (int b = 0; b < 3; ++b) {
        double t = 0;
        for (int k = 0; k < 3; ++k) t += V3[a][k] * C3[k][b];
        tmp[a][b] = t;
      }
    for (int a = 0; a < 3; ++a)
      for (int b = 0; b < 3; ++b) {
        double t = 0;
        for (int k = 0; k < 3; ++k) t += tmp[a][k] * V3[b][k];
        Wm[a][b] = t;
      }
    double tz = pc[2], fx = cam.focal[0], fy = cam.focal[1];
    double kx = fx / tz, ky = fy / tz;
    double C00 = kx * kx * Wm[0][0], C01 = kx * ky * Wm[0][1], C11 = ky * ky * Wm[1][1];
    double e00 = C00 + s.eps2d, e11 = C11 + s.eps2d;
    double det = e00 * e11 - C01 * C01;
    double Qa = e11 / det, Qb = -C01 / det, Qc = e00 / det;
    double GQ[2][2] = {{gi[4], 0.5 * gi[5]}, {0.5 * gi[5], gi[6]}};
    double Q[2][2] = {{Qa, Qb}, {Qb, Qc}};
    double T1[2][2], dC[2][2];
    for (int a = 0; a < 2; ++a)
      for (int b = 0; b < 2; ++b) T1[a][b] = GQ[a][0] * Q[0][b] + GQ[a][1] * Q[1][b];
    for (int a = 0; a < 2; ++a)
      for (int b = 0; b < 2; ++b) dC[a][b] = -(Q[a][0] * T1[0][b] + Q[a][1] * T1[1][b]);
    double dC00 = dC[0][0], dC11 = dC[1][1], dC01 = dC[0][1] + dC[1][0];
    double dW00 = dC00 * kx * kx, dW01 = dC01 * kx * ky, dW11 = dC11 * ky * ky;
    dpc[2] += -2.0 / tz * (dC00 * C00 + dC01 * C01 + dC11 * C11);
    double GW[3][3] = {{dW00, 0.5 * dW01, 0}, {0.5 * dW01, dW11, 0}, {0, 0, 0}};
    double G3[3][3];  // V3^T GW V3
    for (int a = 0; a < 3; ++a)
      for (int b = 0; b < 3; ++b) {
        double t = 0;
        for (int k = 0; k < 3; ++k) t += GW[a][k] * V3[k][b];
        tmp[a][b] = t;
      }
    for (int a = 0; a < 3; ++a)
      for (int b = 0; b < 3; ++b) {
        double t = 0;
        for (int k = 0; k < 3; ++k) t += V3[k][a] * tmp[k][b];
        G3[a][b] = t;
      }
    double dM[3][3];
    for (int a = 0; a < 3; ++a)
      for (int b = 0; b < 3; ++b) {
        double t = 0;
        for (int k = 0; k < 3; ++k) t += G3[a][k] * M[k][b];
        dM[a][b] = 2.0 * t;
      }
    double dR[3][3], dsig[3] = {0, 0, 0};
    for (int a = 0; a < 3; ++a)
      for (int b = 0; b < 3; ++b) {
        dR[a][b] = dM[a][b] * sig[b];
        dsig[b] += dM[a][b] * R[a][b];
      }
    double dq[4];
    dq[0] = 2 * y * (dR[0][1] + dR[1][0]) + 2 * z * (dR[0][2] + dR[2][0]) +
            2 * w * (dR[2][1] - dR[1][2]) - 4 * x * (dR[1][1] + dR[2][2]);
    dq[1] = -4 * y * (dR[0][0] + dR[2][2]) + 2 * x * (dR[0][1] + dR[1][0]) +
            2 * w * (dR[0][2] - dR[2][0]) + 2 * z * (dR[1][2] + dR[2][1]);
    dq[2] = -4 * z * (dR[0][0] + dR[1][1]) + 2 * w * (dR[1][0] - dR[0][1]) +
            2 * x * (dR[0][2] + dR[2][0]) + 2 * y * (dR[1][2] + dR[2][1]);
    dq[3] = -2 * z * dR[0][1] + 2 * y * dR[0][2] + 2 * z * dR[1][0] - 2 * x * dR[1][2] -
            2 * y * dR[2][0] + 2 * x * dR[2][1];
    double qd = q[0] * dq[0] + q[1] * dq[1] + q[2] * dq[2] + q[3] * dq[3];
    double dqr[4];
    for (int k = 0; k < 4; ++k) dqr[k] = (dq[k] - q[k] * qd) / ql;
    // colour -> SH and view direction
    double dirv[3] = {-pc[0], -pc[1], -pc[2]};
    double dl = std::sqrt(dirv[0] * dirv[0] + dirv[1] * dirv[1] + dirv[2] * dirv[2]);
    double d[3] = {dirv[0] / dl, dirv[1] / dl, dirv[2] / dl};
    double draw[3];
    for (int c = 0; c < 3; ++c) draw[c] = o.raw[c] > 0.0f ? (double)gi[c] : 0.0;
    float Yf[16];
    sh_basis((float)d[0], (float)d[1], (float)d[2], sh_deg, Yf);
    const int ncoef = (sh_deg + 1) * (sh_deg + 1);
    if (with_sh)
      for (int k = 0; k < ncoef; ++k)
        for (int c = 0; c < 3; ++c)
          grads[(uint64_t)(11 + 3 * k + c) * gstride + i] += (float)((double)Yf[k] * draw[c]);
    // d colour / d dir
    double X = d[0], Yv = d[1], Z = d[2];
    double dY[16][3] = {};
    double c1 = SH_C1;
    if (sh_deg > 0) {
      dY[1][1] = -c1; dY[2][2] = c1; dY[3][0] = -c1;
    }
    if (sh_deg > 1) {
      double a0 = SH_C2[0], a1 = SH_C2[1], a2 = SH_C2[2], a3 = SH_C2[3], a4 = SH_C2[4];
      dY[4][0] = a0 * Yv; dY[4][1] = a0 * X;
      dY[5][1] = a1 * Z; dY[5][2] = a1 * Yv;
      dY[6][0] = -2 * a2 * X; dY[6][1] = -2 * a2 * Yv; dY[6][2] = 4 * a2 * Z;
      dY[7][0] = a3 * Z; dY[7][2] = a3 * X;
      dY[8][0] = 2 * a4 * X; dY[8][1] = -2 * a4 * Yv;
    }
    if (sh_deg > 2) {
      double b0 = SH_C3[0], b1 = SH_C3[1], b2 = SH_C3[2], b3 = SH_C3[3], b4 = SH_C3[4],
             b5 = SH_C3[5], b6 = SH_C3[6];
      double xx = X * X, yy = Yv * Yv, zz = Z * Z;
      dY[9][0] = b0 * 6 * X * Yv; dY[9][1] = b0 * (3 * xx - 3 * yy);
      dY[10][0] = b1 * Yv * Z; dY[10][1] = b1 * X * Z; dY[10][2] = b1 * X * Yv;
      dY[11][0] = b2 * (-2 * X * Yv); dY[11][1] = b2 * (4 * zz - xx - 3 * yy); dY[11][2] = b2 * 8 * Yv * Z;
      dY[12][0] = b3 * (-6 * X * Z); dY[12][1] = b3 * (-6 * Yv * Z); dY[12][2] = b3 * (6 * zz - 3 * xx - 3 * yy);
      dY[13][0] = b4 * (4 * zz - 3 * xx - yy); dY[13][1] = b4 * (-2 * X * Yv); dY[13][2] = b4 * 8 * X * Z;
      dY[14][0] = b5 * 2 * X * Z; dY[14][1] = b5 * (-2 * Yv * Z); dY[14][2] = b5 * (xx - yy);
      dY[15][0] = b6 * (3 * xx - 3 * yy); dY[15][1] = b6 * (-6 * X * Yv);
    }
    double ddir[3] = {0, 0, 0};
    for (int k = 1; k < ncoef; ++k)
      for (int c = 0; c < 3; ++c) {
        double shv = get(11 + 3 * k + c);
        for (int j = 0; j < 3; ++j) ddir[j] += draw[c] * shv * dY[k][j];
      }
    double dd = d[0] * ddir[0] + d[1] * ddir[1] + d[2] * ddir[2];
    for (int j = 0; j < 3; ++j) dpc[j] += -(ddir[j] - d[j] * dd) / dl;
    // world position
    for (int j = 0; j < 3; ++j) {
      double t = 0;
      for (int r = 0; r < 3; ++r) t += V3[r][j] * dpc[r];
      grads[(uint64_t)(0 + j) * gstride + i] += (float)t;
    }
    for (int k = 0; k < 3; ++k)
      grads[(uint64_t)(3 + k) * gstride + i] += (float)(dsig[k] * sig[k] * lsg[k]);
    for (int k = 0; k < 4; ++k) grads[(uint64_t)(6 + k) * gstride + i] += (float)dqr[k];
    grads[(uint64_t)10 * gstride + i] += gi[3];
  });
  return 0;
}

// Adam (adam.wgsl:18-38): per element, f32, source order.
void orc_adam(float* p, float* m1, float* m2, const float* g, uint64_t count, float lr,
              float beta1, float beta2, float eps, float bc1_rcp, float bc2_sqrt_rcp) {
  for (uint64_t i = 0; i < count; ++i) {
    float gi = g[i];
    float a = beta1 * m1[i];
    float b = (1.0f - beta1) * gi;
    float nm1 = a + b;
    float c = beta2 * m2[i];
    float d = ((1.0f - beta2) * gi) * gi;
    float nm2 = c + d;
    float denom = std::sqrt(nm2) * bc2_sqrt_rcp + eps;
    float step = lr * bc1_rcp;
    p[i] = p[i] - step * (nm1 / denom);
    m1[i] = nm1;
    m2[i] = nm2;
  }
}

// ---------------------------------------------------------------------------
// FP64 forward + loss of one view for finite differences.  Decisions (cull,
// tile rectangle, depth key order, alpha thresholds, early termination) are
// hashed into *sig so a caller can reject perturbations that change them.
// ---------------------------------------------------------------------------
double orc_loss_f64(const double* params, uint64_t stride, uint32_t n, const OrcCam* cam_in,
                    const OrcSettings* s_in, int sh_deg, const float* target, uint64_t* sig) {
  Cam cam = to_cam(cam_in);
  Settings s = to_set(s_in);
  std::vector<Rec<double>> rec(n);
  for (uint32_t i = 0; i < n; ++i) {
    auto get = [&](uint32_t plane) { return load_param_d<double>(params, stride, plane, i); };
    project_one<double>(get, cam, s, sh_deg, rec[i]);
  }
  uint64_t h = 1469598103934665603ull;
  const uint32_t TW = tiles_w(cam, s), TH = tiles_h(cam, s), T = TW * TH;
  std::vector<uint32_t> counts(n), cum(n);
  uint64_t run = 0;
  for (uint32_t i = 0; i < n; ++i) {
    counts[i] = rec[i].count;
    run += counts[i];
    cum[i] = (uint32_t)run;
    h = (h * 1099511628211ull) ^ counts[i];
    for (int k = 0; k < 4; ++k) h = (h * 1099511628211ull) ^ rec[i].rect[k];
  }
  uint64_t I = run;
  std::vector<uint32_t> keys(I), gid(I);
  for (uint32_t i = 0; i < n; ++i) {
    if (!counts[i]) continue;
    uint64_t cur = i == 0 ? 0 : cum[i - 1];
    double dc = std::min(std::max(rec[i].depth, 0.0), 65535.0);
    uint32_t dq = wgsl_u32(dc) & 0xFFFFu;
    for (uint32_t ty = rec[i].rect[1]; ty < rec[i].rect[3]; ++ty)
      for (uint32_t tx = rec[i].rect[0]; tx < rec[i].rect[2]; ++tx) {
        keys[cur] = ((ty * TW + tx) << 16) | dq;
        gid[cur] = i;
        ++cur;
      }
  }
  std::vector<uint32_t> perm(I);
  for (uint64_t k = 0; k < I; ++k) perm[k] = (uint32_t)k;
  std::stable_sort(perm.begin(), perm.end(), [&](uint32_t a, uint32_t b) { return keys[a] < keys[b]; });
  std::vector<uint32_t> flat(I);
  std::vector<uint32_t> off(T + 1, (uint32_t)I);
  for (uint64_t k = 0; k < I; ++k) {
    flat[k] = gid[perm[k]];
    uint32_t t = keys[perm[k]] >> 16;
    off[t] = std::min(off[t], (uint32_t)k);
    h = (h * 1099511628211ull) ^ flat[k];
  }
  for (int t = (int)T - 1; t >= 0; --t) off[t] = std::min(off[t], off[t + 1]);
  double loss = 0.0;
  for (uint32_t y = 0; y < cam.height; ++y)
    for (uint32_t x = 0; x < cam.width; ++x) {
      uint32_t tile = (y / s.tile_size) * TW + (x / s.tile_size);
      uint64_t p = (uint64_t)y * cam.width + x;
      double rgb[3] = {s.bg[0], s.bg[1], s.bg[2]};
      if (off[tile] < off[tile + 1]) {
        PixOut<double> o;
        uint64_t ps = 0;
        forward_pixel<double>(rec.data(), flat.data(), off[tile], off[tile + 1], x + 0.5,
                              y + 0.5, s, o, &ps);
        h = (h * 1099511628211ull) ^ ps;
        for (int c = 0; c < 3; ++c) rgb[c] = o.rgb[c];
      }
      for (int c = 0; c < 3; ++c) {
        double r = rgb[c] - (double)target[p * 3 + c];
        loss += 0.5 * s.w_l2 * r * r + s.w_l1 * std::fabs(r);
        if (s.w_l1 != 0.0f) h = (h * 1099511628211ull) ^ (r > 0.0 ? 1u : (r < 0.0 ? 2u : 3u));
      }
    }
  if (sig) *sig = h;
  return loss;
}

// ---------------------------------------------------------------------------
// Viewer frame (gaussian-renderer.ts:4111-4123): preprocess.wgsl:116-215 per
// Gaussian, a stable ascending sort of float_to_ordered_uint(-z_camera)
// (:94-98; the reference's atomic compaction order is replaced by index
// order), then one quad per splat drawn in that order (gaussian.wgsl:15-67)
// and blended with src-alpha / one-minus-src-alpha for colour and one /
// one-minus-src-alpha for alpha (gaussian-renderer.ts:863-868) into an f32
// target cleared to zero.  A pixel is covered when its centre lies in
// [cx - r, cx + r) x [cy - r, cy + r) (top-left rule).
// splats12: per Gaussian {cx, cy, a, b, c, opacity, r, g, b, radius, 0, 0};
// keys: sort key per Gaussian (0xFFFFFFFF when culled).
// ---------------------------------------------------------------------------
int orc_view_render(const float* params, uint64_t stride, uint32_t n, const OrcCam* cam_in,
                    float scaling, uint32_t sh_deg, uint32_t round16, float* rgba,
                    float* splats12, uint32_t* keys_out) {
  Cam cam = to_cam(cam_in);
  const int deg = (int)std::min(sh_deg, 3u);
  std::vector<float> sp((size_t)n * 12, 0.0f);
  std::vector<uint32_t> key(n, 0xFFFFFFFFu);
  for (uint32_t g = 0; g < n; ++g) {
    auto get = [&](int plane) { return load_param<float>(params, stride, plane, g, round16 != 0); };
    float p[3] = {get(0), get(1), get(2)};
    float pc[4], clip[4];
    cam_space<float>(cam, p, pc);
    mat4_vec<float>(cam.proj, pc, clip);
    const float w = clip[3];
    const float ndc_x = clip[0] / w, ndc_y = clip[1] / w;
    if (std::fabs(ndc_x) > 1.2f || std::fabs(ndc_y) > 1.2f || pc[2] < 0.0f) continue;  // :143
    const float opacity = 1.0f / (1.0f + sky_expf(-get(10)));                          // :146
    float sig[3];
    for (int k = 0; k < 3; ++k)                                                       // :149-156
      sig[k] = scaling * sky_expf(std::min(std::max(get(3 + k), -10.0f), 10.0f));
    float q[4] = {get(6), get(7), get(8), get(9)};                                    // :159
    float qq = q[0] * q[0] + q[1] * q[1];
    qq = qq + q[2] * q[2];
    qq = qq + q[3] * q[3];
    const float ql = std::sqrt(qq);
    const float rx = q[0] / ql, ry = q[1] / ql, rz = q[2] / ql, rw = q[3] / ql;
    float R[3][3];  // quat_to_mat3 (:100-107), R[col][row]
    R[0][0] = 1.0f - 2.0f * (ry * ry + rz * rz);
    R[0][1] = 2.0f * (rx * ry - rw * rz);
    R[0][2] = 2.0f * (rx * rz + rw * ry);
    R[1][0] = 2.0f * (rx * ry + rw * rz);
    R[1][1] = 1.0f - 2.0f * (rx * rx + rz * rz);
    R[1][2] = 2.0f * (ry * rz - rw * rx);
    R[2][0] = 2.0f * (rx * rz - rw * ry);
    R[2][1] = 2.0f * (ry * rz + rw * rx);
    R[2][2] = 1.0f - 2.0f * (rx * rx + ry * ry);
    float A[3][3], C3[3][3];  // C3D = transpose(S R) S R (:163)
    for (int j = 0; j < 3; ++j)
      for (int r = 0; r < 3; ++r) A[j][r] = (sig[j] * R[r][j]) * sig[j];
    for (int j = 0; j < 3; ++j)
      for (int r = 0; r < 3; ++r) {
        float acc = A[0][r] * R[j][0];
        acc = acc + A[1][r] * R[j][1];
        acc = acc + A[2][r] * R[j][2];
        C3[j][r] = acc;
      }
    const float tx = pc[0], ty = pc[1], tz = pc[2];                                   // :165-176
    const float fx = cam.focal[0], fy = cam.focal[1];
    const float tz2 = tz * tz;
    const float J00 = fx / tz, J11 = fy / tz;
    const float J02 = -(fx * tx) / tz2, J12 = -(fy * ty) / tz2;
    float T[3][3];
    for (int j = 0; j < 3; ++j) {
      const float v0 = cam.view[j * 4 + 0], v1 = cam.view[j * 4 + 1];
      T[j][0] = J00 * v0;
      T[j][1] = J11 * v1;
      T[j][2] = J02 * v0 + J12 * v1;
    }
    float B0[3], B1[3];
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
    c00 = c00 + 0.3f;                                                                  // :179-180
    c11 = c11 + 0.3f;
    const float det = c00 * c11 - c01 * c01;
    if (det <= 0.0f) continue;
    const float det_inv = 1.0f / det;                                                  // :185-188
    const float ca = c11 * det_inv, cb = (-c01) * det_inv, cc = c00 * det_inv;
    float v[3] = {-pc[0], -pc[1], -pc[2]};                                             // :190
    float vv = v[0] * v[0] + v[1] * v[1];
    vv = vv + v[2] * v[2];
    const float vl = std::sqrt(vv);
    float sh[48], raw[3];
    for (int k = 0; k < 48; ++k) sh[k] = get(11 + k);
    sh_color<float>(sh, v[0] / vl, v[1] / vl, v[2] / vl, deg, raw);
    const float mid = 0.5f * (c00 + c11);                                              // :194-198
    const float disc = std::sqrt(std::max(mid * mid - det, 0.0f));
    const float l1 = mid + disc, l2 = mid - disc;
    const float radius = std::ceil(3.0f * std::sqrt(std::max(l1, l2)));
    // gaussian.wgsl:27: center_px = (ndc * (0.5, -0.5) + 0.5) * viewport
    const float cx = (ndc_x * 0.5f + 0.5f) * (float)cam.width;
    const float cy = (ndc_y * -0.5f + 0.5f) * (float)cam.height;
    float* o = &sp[(size_t)g * 12];
    o[0] = cx; o[1] = cy; o[2] = ca; o[3] = cb; o[4] = cc; o[5] = opacity;
    for (int c = 0; c < 3; ++c) o[6 + c] = std::max(0.0f, raw[c]);
    o[9] = radius;
    const uint32_t bits = f2u(-pc[2]);
    key[g] = bits ^ ((bits & 0x80000000u) ? 0xFFFFFFFFu : 0x80000000u);
  }
  std::vector<uint32_t> order;
  for (uint32_t g = 0; g < n; ++g)
    if (key[g] != 0xFFFFFFFFu) order.push_back(g);
  std::stable_sort(order.begin(), order.end(),
                   [&](uint32_t a, uint32_t b) { return key[a] < key[b]; });
  const uint32_t W = cam.width, H = cam.height;
  std::fill(rgba, rgba + (size_t)W * H * 4, 0.0f);
  for (uint32_t g : order) {
    const float* s = &sp[(size_t)g * 12];
    const float cx = s[0], cy = s[1], r = s[9];
    const float X0 = cx - r, X1 = cx + r, Y0 = cy - r, Y1 = cy + r;
    if (!(X1 > 0.0f) || !(Y1 > 0.0f) || !(X0 < (float)W) || !(Y0 < (float)H)) continue;
    const int xlo = (int)std::max(std::floor(X0 - 0.5f) - 1.0f, 0.0f);
    const int ylo = (int)std::max(std::floor(Y0 - 0.5f) - 1.0f, 0.0f);
    const int xhi = (int)std::min(std::ceil(X1 - 0.5f) + 1.0f, (float)W - 1.0f);
    const int yhi = (int)std::min(std::ceil(Y1 - 0.5f) + 1.0f, (float)H - 1.0f);
    for (int y = ylo; y <= yhi; ++y)
      for (int x = xlo; x <= xhi; ++x) {
        const float px = (float)x + 0.5f, py = (float)y + 0.5f;
        if (!(px >= cx - r && px < cx + r && py >= cy - r && py < cy + r)) continue;
        const float dx = px - cx, dy = py - cy;                                       // fs_main
        float so2 = 0.5f * ((s[2] * dx) * dx + (s[4] * dy) * dy);
        so2 = so2 + (s[3] * dx) * dy;
        if (so2 < 0.0f) continue;
        const float a = std::min(std::max(s[5] * sky_expf(-so2), 0.0f), 1.0f);
        const float om = 1.0f - a;
        float* d = &rgba[((size_t)y * W + x) * 4];
        d[0] = s[6] * a + d[0] * om;
        d[1] = s[7] * a + d[1] * om;
        d[2] = s[8] * a + d[2] * om;
        d[3] = a + d[3] * om;
      }
  }
  if (splats12) std::memcpy(splats12, sp.data(), sp.size() * sizeof(float));
  if (keys_out) std::memcpy(keys_out, key.data(), key.size() * sizeof(uint32_t));
  return 0;
}

}  // extern "C"
