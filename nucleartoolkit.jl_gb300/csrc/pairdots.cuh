// Matrix of dot products between two sets of device vectors (obtr.cu).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace smgpu {

// Number of chunks per dot product for vectors of length len.
int pair_dot_chunks(int64_t len);
// out[a*ny + b] = Σ_i x[a][i]·y[b][i] (nx*ny <= 65535); partial holds
// nx*ny*pair_dot_chunks(len) doubles.  Deterministic: fixed chunking and a
// fixed reduction order.
void launch_pair_dots(const double* x, int nx, const double* y, int ny, int64_t len, double* partial, double* out,
                      cudaStream_t st);

}  // namespace smgpu
