// PLY import with the reference's semantics and a 3DGS-layout export (host
// code).
//
// Import follows load() (src/utils/load.ts:14-172) with decodeHeader /
// readRawVertex (src/utils/plyreader.ts:1-77):
//   * vertex properties in header order; `float` is a little-endian f32,
//     `uchar` is read as value / 255;
//   * 3DGS files (f_dc_0, opacity, rot_0, scale_0 present): SH coefficient k
//     of channel c is f_dc_c for k = 0 and f_rest_{c * K + k - 1} otherwise
//     (K = f_rest count / 3); degree sqrt(K + 1) - 1;
//   * xyz + rgb files: DC = (red / 255 - 0.5) / SH_C0 where `red` already
//     went through the uchar / 255 of readRawVertex (the reference divides
//     twice); other coefficients 0;
//   * files without those: opacity -2.197, rotation halves (0, 0, 0, 1),
//     log sigma ln(0.01);
//   * every value is stored through f16 (Float16Array: the double is rounded
//     to f32, then to f16 with ties to even), as the reference's packed
//     buffers hold it; the rotation halves rot_0..3 are read by the shaders
//     as the quaternion (rot_1, rot_2, rot_3, rot_0) = (x, y, z, w).
// Where the reference would silently misread a file (a vertex property type
// other than float or uchar, a non-binary-little-endian body, a truncated
// body) the importer reports an error instead.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <map>
#include <sstream>

#include "plyio.cuh"

namespace sky {
namespace {

constexpr double kShC0 = 0.28209479177387814;

float f16_round(float f) {
  uint32_t x;
  std::memcpy(&x, &f, 4);
  const uint32_t sign = x & 0x80000000u;
  uint32_t ax = x & 0x7FFFFFFFu;
  float r;
  if (ax >= 0x7F800000u) return f;
  if (ax >= 0x477FF000u) {
    const uint32_t inf = sign | 0x7F800000u;
    std::memcpy(&r, &inf, 4);
    return r;
  }
  if (ax < 0x38800000u) {  // f16 subnormals: multiples of 2^-24
    const float q = std::nearbyint(std::fabs(f) * 16777216.0f);
    const float v = q * 5.9604644775390625e-08f;
    return sign ? -v : v;
  }
  const uint32_t lsb = (ax >> 13) & 1u;
  ax = (ax + 0x0FFFu + lsb) & ~0x1FFFu;
  const uint32_t b = sign | ax;
  std::memcpy(&r, &b, 4);
  return r;
}

float store16(double v) { return f16_round((float)v); }

}  // namespace

int ply_read(const char* path, PlyScene& out, std::string& err) {
  std::ifstream f(path, std::ios::binary);
  if (!f) {
    err = std::string("cannot open ") + path;
    return -1;
  }
  std::string data((std::istreambuf_iterator<char>(f)), std::istreambuf_iterator<char>());
  const size_t eh = data.find("end_header");
  if (eh == std::string::npos) {
    err = "no end_header in PLY header";
    return -1;
  }
  std::istringstream hs(data.substr(0, eh));
  std::string line, element;
  uint64_t count = 0;
  bool le = false;
  std::vector<std::pair<std::string, std::string>> props;  // vertex (type, name)
  while (std::getline(hs, line)) {
    std::istringstream ls(line);
    std::string w0;
    ls >> w0;
    if (w0 == "format") {
      std::string fmt;
      ls >> fmt;
      le = fmt == "binary_little_endian";
    } else if (w0 == "element") {
      ls >> element;
      if (element == "vertex") ls >> count;
    } else if (w0 == "property" && element == "vertex") {
      std::string type, name;
      ls >> type >> name;
      if (type != "float" && type != "uchar") {
        err = "vertex property '" + name + "' has type '" + type + "' (float and uchar are read)";
        return -1;
      }
      props.emplace_back(type, name);
    }
  }
  if (!le) {
    err = "PLY body is not binary_little_endian";
    return -1;
  }
  if (count == 0 || count >= (1ull << 31)) {
    err = "vertex count out of range";
    return -1;
  }
  size_t stride = 0;
  std::map<std::string, size_t> off;  // byte offset of each property
  std::map<std::string, bool> is_u8;
  for (auto& p : props) {
    off[p.second] = stride;
    is_u8[p.second] = p.first == "uchar";
    stride += p.first == "uchar" ? 1 : 4;
  }
  const size_t body = eh + std::strlen("end_header") + 1;
  if (data.size() < body || (data.size() - body) / stride < count) {
    err = "PLY body shorter than its vertex count";
    return -1;
  }
  auto has = [&](const char* k) { return off.count(k) != 0; };
  const bool gauss = has("f_dc_0") && has("opacity") && has("rot_0") && has("scale_0");
  const bool rgb = has("red") && has("green") && has("blue") && !gauss;
  uint32_t nrest = 0;
  for (auto& p : props)
    if (p.second.rfind("f_rest_", 0) == 0) ++nrest;
  int deg = 0;
  uint32_t per = 0;
  if (gauss) {
    per = nrest / 3;
    const double d = std::sqrt((double)per + 1.0) - 1.0;
    deg = (int)d;
    if ((double)deg != d || deg > 3 || per * 3 != nrest) {
      err = "unsupported SH layout: " + std::to_string(nrest) + " f_rest properties";
      return -1;
    }
  }
  const uint32_t ncoef = (uint32_t)((deg + 1) * (deg + 1));
  const uint32_t n = (uint32_t)count;
  out.n = n;
  out.sh_deg = (uint32_t)deg;
  out.gaussian_format = gauss;
  out.planes.assign((size_t)59 * n, 0.0f);
  auto P = [&](int plane, uint32_t i) -> float& { return out.planes[(size_t)plane * n + i]; };
  const char* base = data.data() + body;
  auto get = [&](const std::string& k, uint32_t i, double dflt) -> double {
    auto it = off.find(k);
    if (it == off.end()) return dflt;
    const char* q = base + (size_t)i * stride + it->second;
    if (is_u8[k]) return (double)(uint8_t)q[0] / 255.0;
    float v;
    std::memcpy(&v, q, 4);  // both hosts here are little endian
    return (double)v;
  };
  double mn[3] = {INFINITY, INFINITY, INFINITY}, mx[3] = {-INFINITY, -INFINITY, -INFINITY};
  const char* axes[3] = {"x", "y", "z"};
  for (uint32_t i = 0; i < n; ++i) {
    for (int k = 0; k < 3; ++k) {
      const double v = get(axes[k], i, NAN);  // undefined -> NaN half in the reference
      P(k, i) = store16(v);
      mn[k] = std::fmin(mn[k], v);
      mx[k] = std::fmax(mx[k], v);
    }
    if (gauss) {
      for (uint32_t k = 0; k < ncoef; ++k)
        for (int c = 0; c < 3; ++c) {
          const std::string name = k == 0 ? "f_dc_" + std::to_string(c)
                                          : "f_rest_" + std::to_string(c * per + k - 1);
          P(11 + 3 * k + c, i) = store16(get(name, i, NAN));
        }
      P(10, i) = store16(get("opacity", i, NAN));
      // halves rot_0..3 -> quaternion (rot_1, rot_2, rot_3, rot_0)
      P(9, i) = store16(get("rot_0", i, NAN));
      P(6, i) = store16(get("rot_1", i, NAN));
      P(7, i) = store16(get("rot_2", i, NAN));
      P(8, i) = store16(get("rot_3", i, NAN));
      for (int k = 0; k < 3; ++k) P(3 + k, i) = store16(get("scale_" + std::to_string(k), i, NAN));
    } else {
      if (rgb) {
        const char* ch[3] = {"red", "green", "blue"};
        for (int c = 0; c < 3; ++c) {
          const double r = get(ch[c], i, 255.0) / 255.0;
          P(11 + c, i) = store16((r - 0.5) / kShC0);
        }
      }
      P(10, i) = store16(-2.197);
      // default halves (0, 0, 0, 1) = (rot_0, rot_1, rot_2, rot_3)
      P(9, i) = 0.0f;
      P(6, i) = 0.0f;
      P(7, i) = 0.0f;
      P(8, i) = 1.0f;
      for (int k = 0; k < 3; ++k) P(3 + k, i) = store16(std::log(0.01));
    }
  }
  out.extent = std::fmax(std::fmax(mx[0] - mn[0], mx[1] - mn[1]), mx[2] - mn[2]);
  return 0;
}

int ply_write(const char* path, const float* planes, uint64_t stride, uint32_t n, uint32_t sh_deg,
              std::string& err) {
  if (sh_deg > 3) sh_deg = 3;
  const uint32_t ncoef = (sh_deg + 1) * (sh_deg + 1), per = ncoef - 1;
  FILE* f = std::fopen(path, "wb");
  if (!f) {
    err = std::string("cannot create ") + path;
    return -1;
  }
  std::string h = "ply\nformat binary_little_endian 1.0\nelement vertex " + std::to_string(n) + "\n";
  const char* head[] = {"x", "y", "z", "nx", "ny", "nz", "f_dc_0", "f_dc_1", "f_dc_2"};
  for (const char* p : head) h += std::string("property float ") + p + "\n";
  for (uint32_t k = 0; k < 3 * per; ++k) h += "property float f_rest_" + std::to_string(k) + "\n";
  const char* tail[] = {"opacity", "scale_0", "scale_1", "scale_2", "rot_0", "rot_1", "rot_2", "rot_3"};
  for (const char* p : tail) h += std::string("property float ") + p + "\n";
  h += "end_header\n";
  bool ok = std::fwrite(h.data(), 1, h.size(), f) == h.size();
  const uint32_t nf = 9 + 3 * per + 8;
  std::vector<float> row(nf);
  auto P = [&](int plane, uint32_t i) { return planes[(size_t)plane * stride + i]; };
  for (uint32_t i = 0; i < n && ok; ++i) {
    uint32_t o = 0;
    for (int k = 0; k < 3; ++k) row[o++] = P(k, i);
    for (int k = 0; k < 3; ++k) row[o++] = 0.0f;
    for (int c = 0; c < 3; ++c) row[o++] = P(11 + c, i);
    for (int c = 0; c < 3; ++c)
      for (uint32_t k = 1; k < ncoef; ++k) row[o++] = P(11 + 3 * k + c, i);
    row[o++] = P(10, i);
    for (int k = 0; k < 3; ++k) row[o++] = P(3 + k, i);
    row[o++] = P(9, i);  // rot_0 = w
    row[o++] = P(6, i);
    row[o++] = P(7, i);
    row[o++] = P(8, i);
    ok = std::fwrite(row.data(), 4, nf, f) == nf;
  }
  if (std::fclose(f) != 0) ok = false;
  if (!ok) {
    err = std::string("write failed: ") + path;
    return -1;
  }
  return 0;
}

}  // namespace sky
