// PLY scene files (plyio.cu): the reference's importer (src/utils/load.ts,
// src/utils/plyreader.ts) and a 3DGS-layout exporter.
#pragma once

#include <stdint.h>

#include <string>
#include <vector>

namespace sky {

struct PlyScene {
  uint32_t n = 0;
  uint32_t sh_deg = 0;          // degree implied by the f_rest_* count
  bool gaussian_format = false; // f_dc_0, opacity, rot_0 and scale_0 present
  double extent = 0.0;          // max bounding-box extent of x, y, z
  std::vector<float> planes;    // 59 planes of n values (the context layout)
};

// Returns 0, or -1 with a message in err.
int ply_read(const char* path, PlyScene& out, std::string& err);
// 3DGS layout: x y z nx ny nz f_dc_0..2 f_rest_0.. opacity scale_0..2 rot_0..3
// (f32, binary little endian); SH coefficients of degree <= sh_deg.
int ply_write(const char* path, const float* planes, uint64_t stride, uint32_t n, uint32_t sh_deg,
              std::string& err);

}  // namespace sky
