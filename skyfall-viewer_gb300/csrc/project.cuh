// Projection of one Gaussian into one view, shared by the preprocess kernel
// and the geometry adjoint.  Follows project_gaussians_for_tiling
// (src/shaders/training-tiles.wgsl:40-180) operation for operation in the
// order fixed by sky_math.cuh, plus the per-Gaussian opacity and SH colour
// the reference evaluates per pixel (training-forward-tiles.wgsl:184-190).
#pragma once

#include "sky_math.cuh"
#include "sky_types.cuh"

namespace sky {

struct ProjOut {
  float mx, my;          // pixel-space mean
  float ca, cb, cc;      // conic
  float opacity;         // sigmoid(logit)
  float col[3];          // clamped colour
  float raw[3];          // colour before the clamp
  float dir[3];          // normalize(-p_cam)
  float depth, radius;
  float cov00, cov11;    // diagonal of the 2D covariance (with eps2d)
  float pc[4];           // camera-space position
  uint32_t count, x0, y0, x1, y1;
};

// The view-independent part of the projection: the 3D covariance
// R S S^T R^T (scales exp(clamp(log sigma, -10, 10)), R from the normalised
// quaternion) and the sigmoid opacity, computed once per Gaussian.
struct GaussCov3 {
  float C3[3][3];
  float opacity;
};

// Quaternion (planes 6..9) normalised and turned into the rotation matrix,
// R[a][c] = row a, column c of the rotation (quat_to_mat3_tiling,
// training-tiles.wgsl:30-37, of the quaternion read at :97-98).
template <typename Get>
SKY_DEV void gauss_rotation(Get get, float R[3][3], float qn[4], float& ql) {
  float q0 = get(6), q1 = get(7), q2 = get(8), q3 = get(9);
  float qq = q0 * q0 + q1 * q1;
  qq = qq + q2 * q2;
  qq = qq + q3 * q3;
  ql = sqrtf(qq);
  const float rx = q0 / ql, ry = q1 / ql, rz = q2 / ql, rw = q3 / ql;
  qn[0] = rx; qn[1] = ry; qn[2] = rz; qn[3] = rw;
  R[0][0] = 1.0f - 2.0f * (ry * ry + rz * rz);
  R[0][1] = 2.0f * (rx * ry - rw * rz);
  R[0][2] = 2.0f * (rx * rz + rw * ry);
  R[1][0] = 2.0f * (rx * ry + rw * rz);
  R[1][1] = 1.0f - 2.0f * (rx * rx + rz * rz);
  R[1][2] = 2.0f * (ry * rz - rw * rx);
  R[2][0] = 2.0f * (rx * rz - rw * ry);
  R[2][1] = 2.0f * (ry * rz + rw * rx);
  R[2][2] = 1.0f - 2.0f * (rx * rx + ry * ry);
}

template <typename Get>
SKY_DEV void gauss_cov3(Get get, GaussCov3& gc) {
  float sig[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) sig[k] = sky_expf(clampf_(get(3 + k), -10.0f, 10.0f));
  float R[3][3], qn[4], ql;
  gauss_rotation(get, R, qn, ql);
  float A[3][3];
#pragma unroll
  for (int j = 0; j < 3; ++j)
#pragma unroll
    for (int r = 0; r < 3; ++r) A[j][r] = (sig[j] * R[r][j]) * sig[j];
#pragma unroll
  for (int j = 0; j < 3; ++j)
#pragma unroll
    for (int r = 0; r < 3; ++r) {
      float acc = A[0][r] * R[j][0];
      acc = acc + A[1][r] * R[j][1];
      acc = acc + A[2][r] * R[j][2];
      gc.C3[j][r] = acc;
    }
  gc.opacity = 1.0f / (1.0f + sky_expf(-get(10)));
}

// Camera-space position pc = view * (p, 1) of the Gaussian's mean (planes 0..2).
template <typename Get>
SKY_DEV void view_position(Get get, const ViewInfo& vi, float pc[4]) {
  const float px = get(0), py = get(1), pz = get(2);
#pragma unroll
  for (int r = 0; r < 4; ++r) pc[r] = mat4_row(vi.view, r, px, py, pz, 1.0f);
}

// View direction normalize(-pc) and, when want_color, the SH colour before
// and after the clamp at zero.
template <typename Get>
SKY_DEV void view_color(Get get, const float pc[4], int deg, bool want_color, ProjOut& o) {
  const float v0 = -pc[0], v1 = -pc[1], v2 = -pc[2];
  float vv = v0 * v0 + v1 * v1;
  vv = vv + v2 * v2;
  const float vl = sqrtf(vv);
  o.dir[0] = v0 / vl;
  o.dir[1] = v1 / vl;
  o.dir[2] = v2 / vl;
  if (want_color) {
    auto sh = [&](int k, int c) { return get(11 + 3 * k + c); };
    sh_color_raw(sh, o.dir[0], o.dir[1], o.dir[2], deg, o.raw);
#pragma unroll
    for (int c = 0; c < 3; ++c) o.col[c] = fmax_(0.0f, o.raw[c]);
  }
}

// get(plane) returns parameter plane `plane` of the Gaussian (already f16
// rounded when the reference storage format is emulated); gc holds its
// gauss_cov3.  Returns false if the Gaussian is culled (then count ==
// radius == depth == 0).
template <typename Get>
SKY_DEV bool project_gaussian(Get get, const GaussCov3& gc, const ViewInfo& vi,
                              const StepParams& sp, int deg, bool want_color, ProjOut& o) {
  o.count = 0; o.x0 = o.y0 = o.x1 = o.y1 = 0;
  o.radius = 0.0f; o.depth = 0.0f;
  o.mx = o.my = 0.0f; o.ca = o.cb = o.cc = 0.0f; o.opacity = 0.0f;
  o.col[0] = o.col[1] = o.col[2] = 0.0f;
  o.raw[0] = o.raw[1] = o.raw[2] = 0.0f;
  o.dir[0] = o.dir[1] = o.dir[2] = 0.0f;
  float pc[4];
  view_position(get, vi, pc);
#pragma unroll
  for (int r = 0; r < 4; ++r) o.pc[r] = pc[r];
  float clip[4];
#pragma unroll
  for (int r = 0; r < 4; ++r) clip[r] = mat4_row(vi.proj, r, pc[0], pc[1], pc[2], pc[3]);
  const float w = clip[3];
  const float ndc_x = clip[0] / w, ndc_y = clip[1] / w;
  if (fabsf(ndc_x) > 1.2f || fabsf(ndc_y) > 1.2f || pc[2] <= 0.0f) return false;
  const float depth = pc[2];
  if (depth < sp.near_plane || depth > sp.far_plane) return false;
  const auto& C3 = gc.C3;
  const float tx = pc[0], ty = pc[1], tz = pc[2];
  const float fx = vi.focal[0], fy = vi.focal[1];
  const float tz2 = tz * tz;
  const float J00 = fx / tz, J11 = fy / tz;
  const float J02 = -(fx * tx) / tz2, J12 = -(fy * ty) / tz2;
  float T[3][3];
#pragma unroll
  for (int j = 0; j < 3; ++j) {
    float v0 = vi.view[j * 4 + 0], v1 = vi.view[j * 4 + 1];
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
  c00 = c00 + sp.eps2d;
  c11 = c11 + sp.eps2d;
  const float det = c00 * c11 - c01 * c01;
  if (det <= 0.0f) return false;
  const float mid = 0.5f * (c00 + c11);
  const float disc = sqrtf(fmax_(mid * mid - det, 0.0f));
  const float l1 = mid + disc, l2 = mid - disc;
  const float radius = ceilf(3.0f * sqrtf(fmax_(l1, l2)));
  if (radius > sp.radius_clip || radius < 1.0f) return false;
  const float det_inv = 1.0f / det;
  o.cov00 = c00;
  o.cov11 = c11;
  o.ca = c11 * det_inv;
  o.cb = (-c01) * det_inv;
  o.cc = c00 * det_inv;
  o.mx = (0.5f * (ndc_x + 1.0f)) * (float)vi.width;
  o.my = (0.5f * (ndc_y + 1.0f)) * (float)vi.height;
  o.radius = radius;
  o.depth = depth;
  // ts is 8, 16 or 32: multiplying by its exact reciprocal is the IEEE
  // quotient bit for bit, without three division sequences
  const float rts = 1.0f / (float)sp.tile_size;
  const float tile_x = o.mx * rts, tile_y = o.my * rts;
  const float trx = radius * rts;
  o.x0 = min(wgsl_u32(floorf(tile_x - trx)), vi.tiles_x);
  o.y0 = min(wgsl_u32(floorf(tile_y - trx)), vi.tiles_y);
  o.x1 = min(wgsl_u32(ceilf(tile_x + trx)), vi.tiles_x);
  o.y1 = min(wgsl_u32(ceilf(tile_y + trx)), vi.tiles_y);
  const int nx = (int)o.x1 - (int)o.x0, ny = (int)o.y1 - (int)o.y0;
  o.count = (nx <= 0 || ny <= 0) ? 0u : (uint32_t)(nx * ny);
  o.opacity = gc.opacity;
  view_color(get, pc, deg, want_color, o);
  return true;
}

}  // namespace sky
