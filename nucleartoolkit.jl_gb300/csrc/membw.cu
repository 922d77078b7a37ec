// Read bandwidth of an L2-resident buffer (smgpu_l2_read_bandwidth).
//
// The H·v kernels work on a set of tables and vectors that fits in the GPU's
// L2 cache (48Cr: 11 MB of tables, 8-24 MB of vectors), so their bound is the
// rate at which the SMs can pull data out of L2, not HBM.  This probe gives
// that ceiling on the GPU at hand: every CTA streams the same buffer (sized
// well below the L2) with 16-byte loads that are cached in L2 only, after one
// untimed sweep has brought it into L2.  CUDA events time `reps` launches of
// 16 sweeps each.
#include <cstdint>

#include <cuda_runtime.h>

#include "../../include/smgpu.h"

namespace {

constexpr int kNT = 512;

// `passes` sweeps over the buffer; in each, every float of it is summed (per
// thread), four independent 16-byte loads in flight per thread.  The loads
// are cached in L2 only, so repeated sweeps are served by L2, not by L1.
// The sums are stored only under a condition that never holds for the
// zero-filled buffer, which keeps the loads live.
__global__ void __launch_bounds__(kNT) k_l2_read(const float4* __restrict__ p, int64_t n4, int passes,
                                                 float* __restrict__ out) {
  float4 a0 = make_float4(0.f, 0.f, 0.f, 0.f), a1 = a0, a2 = a0, a3 = a0;
  const int64_t step = (int64_t)gridDim.x * kNT;
  for (int pass = 0; pass < passes; ++pass) {
    int64_t i = blockIdx.x * (int64_t)kNT + threadIdx.x;
    for (; i + 3 * step < n4; i += 4 * step) {
      const float4 x0 = __ldcg(p + i), x1 = __ldcg(p + i + step), x2 = __ldcg(p + i + 2 * step),
                   x3 = __ldcg(p + i + 3 * step);
      a0.x += x0.x; a0.y += x0.y; a0.z += x0.z; a0.w += x0.w;
      a1.x += x1.x; a1.y += x1.y; a1.z += x1.z; a1.w += x1.w;
      a2.x += x2.x; a2.y += x2.y; a2.z += x2.z; a2.w += x2.w;
      a3.x += x3.x; a3.y += x3.y; a3.z += x3.z; a3.w += x3.w;
    }
    for (; i < n4; i += step) {
      const float4 x = __ldcg(p + i);
      a0.x += x.x; a0.y += x.y; a0.z += x.z; a0.w += x.w;
    }
  }
  const float s = a0.x + a0.y + a0.z + a0.w + a1.x + a1.y + a1.z + a1.w + a2.x + a2.y + a2.z + a2.w + a3.x + a3.y +
                  a3.z + a3.w;
  if (s == 1.0f) out[blockIdx.x] = s;
}

}  // namespace

extern "C" int smgpu_l2_read_bandwidth(long long bytes, int reps, double* gbs_out) {
  if (bytes < (1 << 20) || bytes > (1ll << 30) || reps < 1 || !gbs_out) return SMGPU_ERR_ARG;
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
    return SMGPU_ERR_CUDA;
  const int64_t n4 = bytes / 16;
  float4* buf = nullptr;
  float* out = nullptr;
  cudaEvent_t a = nullptr, b = nullptr;
  int rc = SMGPU_OK;
  if (cudaMalloc(&buf, n4 * 16) != cudaSuccess || cudaMalloc(&out, sizeof(float) * 4 * sms) != cudaSuccess) {
    rc = SMGPU_ERR_NOMEM;
  } else if (cudaMemset(buf, 0, n4 * 16) != cudaSuccess || cudaEventCreate(&a) != cudaSuccess ||
             cudaEventCreate(&b) != cudaSuccess) {
    rc = SMGPU_ERR_CUDA;
  } else {
    const int grid = 4 * sms;  // 4 CTAs of 512 threads per SM: every warp slot the SM has
    constexpr int kPasses = 16;  // sweeps per launch: the launch lasts far longer than its start-up
    k_l2_read<<<grid, kNT>>>(buf, n4, 1, out);  // brings the buffer into L2
    cudaEventRecord(a);
    for (int r = 0; r < reps; ++r) k_l2_read<<<grid, kNT>>>(buf, n4, kPasses, out);
    cudaEventRecord(b);
    float ms = 0.f;
    if (cudaEventSynchronize(b) != cudaSuccess || cudaEventElapsedTime(&ms, a, b) != cudaSuccess ||
        cudaGetLastError() != cudaSuccess || !(ms > 0.f))
      rc = SMGPU_ERR_CUDA;
    else
      *gbs_out = (double)n4 * 16.0 * kPasses * reps / (ms * 1e-3) / 1e9;
  }
  if (a) cudaEventDestroy(a);
  if (b) cudaEventDestroy(b);
  if (buf) cudaFree(buf);
  if (out) cudaFree(out);
  return rc;
}
