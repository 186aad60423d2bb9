// Device arithmetic shared by the skyfall kernels.
//
// Every function here evaluates the reference's WGSL formulas as separate
// IEEE-754 f32 operations in source order (the library is compiled with
// -fmad=false, and the few deliberate fused multiply-adds are written as
// __fmaf_rn).  Matrix-vector and matrix-matrix products sum their terms in
// ascending index order, min/max follow C++ std::min/std::max, exp() is
// sky_expf (below) and f16 storage rounds to nearest even.  With those rules
// fixed, the per-pixel compositing decisions (alpha < 1/255, early
// termination) are reproducible by a CPU implementation bit for bit.
#pragma once

#include <cuda_fp16.h>
#include <stdint.h>

#define SKY_DEV __device__ __forceinline__

namespace sky {

// SH constants, src/shaders/common.wgsl:1-18 (f32).
constexpr float SH_C0 = 0.28209479177387814f;
constexpr float SH_C1 = 0.4886025119029199f;
constexpr float SH_C2_0 = 1.0925484305920792f;
constexpr float SH_C2_1 = -1.0925484305920792f;
constexpr float SH_C2_2 = 0.31539156525252005f;
constexpr float SH_C2_3 = -1.0925484305920792f;
constexpr float SH_C2_4 = 0.5462742152960396f;
constexpr float SH_C3_0 = -0.5900435899266435f;
constexpr float SH_C3_1 = 2.890611442640554f;
constexpr float SH_C3_2 = -0.4570457994644658f;
constexpr float SH_C3_3 = 0.3731763325901154f;
constexpr float SH_C3_4 = -0.4570457994644658f;
constexpr float SH_C3_5 = 1.445305721320277f;
constexpr float SH_C3_6 = -0.5900435899266435f;

// Compositing constants, src/shaders/training-forward-tiles.wgsl:38-41.
constexpr float MIN_ALPHA = 1.0f / 255.0f;
constexpr float MAX_ALPHA = 0.999f;
constexpr float T_THRESH = 1e-4f;

SKY_DEV float fmin_(float a, float b) { return (b < a) ? b : a; }
SKY_DEV float fmax_(float a, float b) { return (a < b) ? b : a; }
SKY_DEV float clampf_(float x, float lo, float hi) { return fmin_(fmax_(x, lo), hi); }

// exp(x): Cody-Waite reduction x = k ln2 + r with |r| <= ln2/2, degree-7
// Taylor polynomial of e^r (Horner, fused multiply-adds), scaled by 2^k
// through the exponent field.  Within 1 ulp of exp on [-87, 88]; 0 below,
// +inf above.  Written out here so that the CPU oracle can evaluate the same
// function bit for bit.
SKY_DEV float sky_expf_inrange(float x);

SKY_DEV float sky_expf(float x) {
  if (x != x) return x;
  if (x > 88.0f) return __int_as_float(0x7F800000);
  if (x < -87.0f) return 0.0f;
  return sky_expf_inrange(x);
}

// sky_expf without its range checks, for arguments known to lie in
// [-87, 88] (the rasterizers' -s with 0 <= s <= ln(255) + 1e-3): the same
// operations, so the same result.
SKY_DEV float sky_expf_inrange(float x) {
  const float kLog2e = 1.44269502f;
  const float kLn2Hi = 0.693147182f;
  const float kLn2Lo = -1.90465421e-09f;
  const float kRound = 12582912.0f;  // 1.5 * 2^23
  float t = __fmul_rn(x, kLog2e);
  float u = __fadd_rn(t, kRound);
  float k = __fsub_rn(u, kRound);
  float r = __fmaf_rn(-k, kLn2Hi, x);
  r = __fmaf_rn(-k, kLn2Lo, r);
  float p = 1.98412701e-04f;
  p = __fmaf_rn(p, r, 1.38888892e-03f);
  p = __fmaf_rn(p, r, 8.33333377e-03f);
  p = __fmaf_rn(p, r, 4.16666679e-02f);
  p = __fmaf_rn(p, r, 1.66666672e-01f);
  p = __fmaf_rn(p, r, 0.5f);
  p = __fmaf_rn(p, r, 1.0f);
  p = __fmaf_rn(p, r, 1.0f);
  uint32_t kbits = __float_as_uint(u) - __float_as_uint(kRound);
  return __uint_as_float(__float_as_uint(p) + (kbits << 23));
}

// log(x): x = m 2^e with m in [sqrt(1/2), sqrt(2)); log m = 2 atanh(s),
// s = (m - 1) / (m + 1), |s| <= 0.172, by its odd series to s^11 (Horner in
// s^2, fused multiply-adds); log x = e ln2 + log m with ln2 split in two.
// Within 2 ulp of log for positive normal and subnormal x; -inf at 0, NaN
// below, +inf at +inf.  Written out so that the CPU oracle evaluates the
// same function bit for bit.
SKY_DEV float sky_logf(float x) {
  if (x != x || x < 0.0f) return __int_as_float(0x7FC00000);
  if (x == 0.0f) return __int_as_float(0xFF800000);
  if (x == __int_as_float(0x7F800000)) return x;
  uint32_t b = __float_as_uint(x);
  int e = 0;
  if (b < 0x00800000u) {  // subnormal: scale by 2^23
    x = __fmul_rn(x, 8388608.0f);
    b = __float_as_uint(x);
    e = -23;
  }
  e += (int)(b >> 23) - 127;
  float m = __uint_as_float((b & 0x007FFFFFu) | 0x3F800000u);
  if (m > 1.41421354f) {
    m = __fmul_rn(m, 0.5f);
    e += 1;
  }
  const float s = __fdiv_rn(__fsub_rn(m, 1.0f), __fadd_rn(m, 1.0f));
  const float z = __fmul_rn(s, s);
  float p = 0.181818187f;               // 2/11
  p = __fmaf_rn(p, z, 0.222222224f);    // 2/9
  p = __fmaf_rn(p, z, 0.285714298f);    // 2/7
  p = __fmaf_rn(p, z, 0.400000006f);    // 2/5
  p = __fmaf_rn(p, z, 0.666666687f);    // 2/3
  const float lm = __fmaf_rn(__fmul_rn(s, z), p, __fmul_rn(2.0f, s));
  const float fe = (float)e;
  return __fmaf_rn(fe, 0.693147182f, __fmaf_rn(fe, -1.90465421e-09f, lm));
}

SKY_DEV float round_f16(float x) { return __half2float(__float2half_rn(x)); }

// WGSL f32 -> u32: truncation toward zero, saturating; NaN -> 0.
SKY_DEV uint32_t wgsl_u32(float f) {
  if (!(f > 0.0f)) return 0u;
  if (f >= 4294967296.0f) return 0xFFFFFFFFu;
  return (uint32_t)f;
}
// WGSL f32 -> i32: truncation toward zero, saturating; NaN -> 0.
SKY_DEV int32_t wgsl_i32(float f) {
  if (f != f) return 0;
  if (f >= 2147483648.0f) return 2147483647;
  if (f <= -2147483648.0f) return (int32_t)0x80000000u;
  return (int32_t)f;
}

// WGSL mat4x4 * vec4 row r for a column-major matrix m: columns combined in
// index order.
SKY_DEV float mat4_row(const float* m, int r, float x, float y, float z, float w) {
  float acc = m[0 * 4 + r] * x;
  acc = acc + m[1 * 4 + r] * y;
  acc = acc + m[2 * 4 + r] * z;
  acc = acc + m[3 * 4 + r] * w;
  return acc;
}

// SH colour before the clamp, computeColorFromSH_tf
// (src/shaders/training-forward-tiles.wgsl:65-105).  sh(k, c) returns
// coefficient k, channel c.
template <typename ShFn>
SKY_DEV void sh_color_raw(ShFn sh, float x, float y, float z, int deg, float out[3]) {
#pragma unroll
  for (int c = 0; c < 3; ++c) out[c] = SH_C0 * sh(0, c);
  if (deg > 0) {
    float a1 = (-SH_C1) * y, a2 = SH_C1 * z, a3 = SH_C1 * x;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      float t = a1 * sh(1, c) + a2 * sh(2, c);
      t = t - a3 * sh(3, c);
      out[c] = out[c] + t;
    }
    if (deg > 1) {
      float xx = x * x, yy = y * y, zz = z * z;
      float xy = x * y, yz = y * z, xz = x * z;
      float b4 = SH_C2_0 * xy;
      float b5 = SH_C2_1 * yz;
      float b6 = SH_C2_2 * ((2.0f * zz - xx) - yy);
      float b7 = SH_C2_3 * xz;
      float b8 = SH_C2_4 * (xx - yy);
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        float t = b4 * sh(4, c) + b5 * sh(5, c);
        t = t + b6 * sh(6, c);
        t = t + b7 * sh(7, c);
        t = t + b8 * sh(8, c);
        out[c] = out[c] + t;
      }
      if (deg > 2) {
        float c9 = (SH_C3_0 * y) * (3.0f * xx - yy);
        float c10 = (SH_C3_1 * xy) * z;
        float c11 = (SH_C3_2 * y) * ((4.0f * zz - xx) - yy);
        float c12 = (SH_C3_3 * z) * ((2.0f * zz - 3.0f * xx) - 3.0f * yy);
        float c13 = (SH_C3_4 * x) * ((4.0f * zz - xx) - yy);
        float c14 = (SH_C3_5 * z) * (xx - yy);
        float c15 = (SH_C3_6 * x) * (xx - 3.0f * yy);
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          float t = c9 * sh(9, c) + c10 * sh(10, c);
          t = t + c11 * sh(11, c);
          t = t + c12 * sh(12, c);
          t = t + c13 * sh(13, c);
          t = t + c14 * sh(14, c);
          t = t + c15 * sh(15, c);
          out[c] = out[c] + t;
        }
      }
    }
  }
#pragma unroll
  for (int c = 0; c < 3; ++c) out[c] = out[c] + 0.5f;
}

// SH basis values Y_k(dir) in the order and form the reference's
// wg_accumulate_sh_grads uses (backward-tiles-local.wgsl:104-183).
SKY_DEV void sh_basis(float x, float y, float z, int deg, float Y[16]) {
#pragma unroll
  for (int k = 0; k < 16; ++k) Y[k] = 0.0f;
  Y[0] = SH_C0;
  if (deg > 0) {
    Y[1] = (-SH_C1) * y;
    Y[2] = SH_C1 * z;
    Y[3] = (-SH_C1) * x;
  }
  if (deg > 1) {
    float xx = x * x, yy = y * y, zz = z * z, xy = x * y, yz = y * z, xz = x * z;
    Y[4] = SH_C2_0 * xy;
    Y[5] = SH_C2_1 * yz;
    Y[6] = SH_C2_2 * ((2.0f * zz - xx) - yy);
    Y[7] = SH_C2_3 * xz;
    Y[8] = SH_C2_4 * (xx - yy);
    if (deg > 2) {
      Y[9] = (SH_C3_0 * y) * (3.0f * xx - yy);
      Y[10] = (SH_C3_1 * xy) * z;
      Y[11] = (SH_C3_2 * y) * ((4.0f * zz - xx) - yy);
      Y[12] = (SH_C3_3 * z) * ((2.0f * zz - 3.0f * xx) - 3.0f * yy);
      Y[13] = (SH_C3_4 * x) * ((4.0f * zz - xx) - yy);
      Y[14] = (SH_C3_5 * z) * (xx - yy);
      Y[15] = (SH_C3_6 * x) * (xx - 3.0f * yy);
    }
  }
}

}  // namespace sky
