// Launch interface of the k-nearest-neighbour scale initialisation (knn.cu).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace sky {

struct KnnGrid {
  float lo[3];          // grid origin (minimum of the f16 positions)
  float h;              // cell edge
  uint32_t dims[3];     // cells per axis
  uint32_t cells;       // dims product
};

// Bounds of the f16-rounded positions: out[0..2] = min, out[3..5] = max, as
// order-preserving u32 encodings (out initialised by knn_bounds_init).
void launch_knn_bounds(const float* params, uint32_t stride, uint32_t n, uint32_t* out,
                       cudaStream_t s);
uint32_t knn_bounds_init(int k);     // initial word k of `out`
float knn_bounds_decode(uint32_t u);  // word -> float
// Cell key and index per point.
void launch_knn_keys(const float* params, uint32_t stride, uint32_t n, const KnnGrid& g,
                     uint32_t* keys, cudaStream_t s);
// cell_start[c] = first sorted position of cell c, c in [0, cells]
void launch_knn_cell_ranges(const uint32_t* keys_sorted, uint32_t n, uint32_t cells,
                            uint32_t* cell_start, cudaStream_t s);
// Three nearest other points of each point by an exact ring search over the
// grid, then the reference's sigma rule; writes density (may be null) and
// the f16 log sigma into the three scale planes of params (every other
// plane is rounded through f16, as the reference's re-sync does).
void launch_knn_query(float* params, uint32_t stride, uint32_t n, const KnnGrid& g,
                      const uint32_t* order, const uint32_t* cell_start, float extent,
                      float* density, float* log_sigma, cudaStream_t s);
void launch_knn_write(float* params, uint32_t stride, uint32_t n, const float* log_sigma,
                      cudaStream_t s);

}  // namespace sky
