// Device-side view of one shell-model problem (all pointers are device memory).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace smgpu {

// Coefficient tables exist in FP64 (plain form) and FP32 (mixed form).
template <class TC>
struct CoefTables {
  const TC* pp_val;
  const TC* nn_val;
  const TC* vtab;
};

struct DevTables {
  int nb;
  int64_t len_pad;
  // per block
  const int* np;
  const int* nn;
  const int* stride;
  const int64_t* off_pad;
  const int* pstart;
  const int* nstart;
  const int64_t* tdims;
  // per global proton row: owning block
  const int* prow_block;
  // pp / nn pull CSR
  const int* pp_ptr;
  const int* pp_col;
  const int* nn_ptr;
  const int* nn_col;
  // pn links
  const int4* link_a;      // x = source block, y = nB, z = unused, w = unused
  const int64_t* link_v;   // V table offset
  const int64_t* link_n;   // offset of the link's neutron row pointers
  const int* ppn_ptr;
  const uint32_t* ppn_src;
  const uint32_t* ppn_meta;  // link<<16 | ia<<1 | sign
  const int64_t* npn_ptr;
  const uint32_t* npn_ent;   // n'<<14 | ib<<1 | sign
};

#define SMGPU_CUDA_TRY(expr)                                                      \
  do {                                                                            \
    cudaError_t _e = (expr);                                                      \
    if (_e != cudaSuccess) throw ::smgpu::CudaError{_e, #expr, __FILE__, __LINE__}; \
  } while (0)

struct CudaError {
  cudaError_t err;
  const char* what;
  const char* file;
  int line;
};

// Launch helpers implemented in hv.cu / lanczos.cu
void launch_hv_fp64(const DevTables& t, const double* ep, const double* en, const CoefTables<double>& c,
                    const double* v, double* w, int nrows, const int* done, cudaStream_t st);
void launch_hv_mixed(const DevTables& t, const double* ep, const double* en, const CoefTables<float>& c,
                     const float* v, double* w, int nrows, const int* done, cudaStream_t st);

}  // namespace smgpu
