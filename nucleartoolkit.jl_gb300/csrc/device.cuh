// Device-side view of one shell-model problem (all pointers are device memory)
// and the small structs shared by the kernels.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace smgpu {

// Coefficient tables exist in FP64 (plain form) and FP32 (mixed form).
// vtab holds, per ΔM, the table [2][nA][nB] = (V, −V).
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
  const int64_t* off_pad;  // nb+1
  const int* pstart;       // nb+1
  const int* nstart;       // nb+1
  const int64_t* tdims;    // nb+1
  // pp / nn pull CSR
  const int* pp_ptr;
  const int* pp_col;
  const int* nn_ptr;
  const int* nn_col;
  // pn links (output block b <- source block s)
  const int4* link_a;     // x = source block, y = nB
  const int64_t* link_v;  // offset of the link's signed V table
  const int64_t* link_n;  // offset of the link's neutron row pointers
  const uint32_t* ppn_src;   // proton pull entries: source row
  const uint32_t* ppn_meta;  // link<<16 | ia<<1 | sign
};

// Double-float arithmetic on the FP32 pipe: a value is an unevaluated pair
// hi + lo of FP32 numbers (about 48 significant bits).  GB300 runs FP64 at a
// small fraction of the FP32 rate, so the FP32-mixed solver keeps its
// long vectors of residuals in this form.
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
  s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}
// |a| >= |b| (or a == 0)
__device__ __forceinline__ void fast_two_sum(float a, float b, float& s, float& e) {
  s = __fadd_rn(a, b);
  e = __fsub_rn(b, __fsub_rn(s, a));
}
// (h, l) += x (bh + bl), renormalised; x·bh exact by a fused two-product.
__device__ __forceinline__ void df_fma(float& h, float& l, float x, float bh, float bl) {
  const float p = __fmul_rn(x, bh);
  const float pe = __fmaf_rn(x, bh, -p);
  float s, e;
  two_sum(h, p, s, e);
  const float t = __fadd_rn(__fadd_rn(l, e), __fmaf_rn(x, bl, pe));
  fast_two_sum(s, t, h, l);
}
// (h, l) += (bh + bl), renormalised.
__device__ __forceinline__ void df_add(float& h, float& l, float bh, float bl) {
  float s, e;
  two_sum(h, bh, s, e);
  const float t = __fadd_rn(__fadd_rn(l, bl), e);
  fast_two_sum(s, t, h, l);
}
// x = hi + lo: hi the FP32 rounding of x, lo that of the remainder.
__host__ __device__ __forceinline__ void df_from_double(double x, float& hi, float& lo) {
  hi = (float)x;
  lo = (float)(x - (double)hi);
}

// Row-tile schedule of the H·v kernel.
struct TileTables {
  const int* task_b;       // block of each CTA
  const int* task_p0;      // first row of each CTA
  const int* link_begin;   // nb+1
  const int64_t* rl_base;  // per block: offset into rl
  const int* rl;           // per (row, link slot): first proton entry; slot nl = end
  const int64_t* npn_ptr;  // neutron pull CSR row pointers (per link, nn[b]+1 each)
  const uint32_t* npn_ent; // n'<<14 | (sign*nA*nB + ib)
  // staged pn form (FP32-mixed): per link, the pull entries regrouped by
  // source neutron column ("push" lists).  Entry = slot | ib << 16 | sign << 31,
  // slot = t * nn[b] + n' for the t-th pull entry of output column n'.  The
  // lists of a link are stored as an ELL array [k][position] (coalesced loads
  // across a warp); position order = source columns sorted by list length.
  const int64_t* push_off;   // per link: offset of its ELL array in push_ent
  const int64_t* push_ioff;  // per link: offset of its nn[s] descriptors in push_info
  const int* push_info;      // per position: source column | list length << 16
  const uint32_t* push_ent;
  // nn term of the staged kernel: per block, the nn pull lists as an ELL
  // array [k][n] (padded with zero coefficients on column n)
  const int64_t* nnell_off;  // per block
  const int* nnell_w;        // per block: longest list
  const int* nnell_col;
  const float* nnell_val;
  // two-body pass of the staged form (hv_2b.cu): the pp and nn terms of
  // every element, computed over row and column tiles of each block and left
  // in s2b for the staged kernel's epilogue
  const int4* pp_tasks;  // (block, first row, first of 32 columns, rows)
  const int4* nn_tasks;  // (block, first of 32 rows, first column, columns)
  int n_pp_tasks, n_nn_tasks;
  float* s2b;            // 2 x len_pad: pp sums, then nn sums
  int npmax;             // largest np[b]
  int ymax;     // floats of one row's slot buffer: max over links of (longest pull list) * nn[b]
  int nnmax;    // largest nn[b], rounded up to 4
  int nbmax;    // largest neutron-operator count nB of a link
  int astride;  // row stride (floats) of the per-row coefficient matrices, = 4 mod 8
  int kpad;     // largest proton-entry count of one (row, link), rounded up to 4
};

struct HvConfig {
  int nt;      // threads per CTA
  int rows;    // rows per CTA
  int ntasks;  // CTAs
  int minb;    // minimum resident CTAs per SM requested from the compiler (caps registers)
  int staged;  // 1: the staged pn kernel (hv_staged.cu, FP32-mixed only); 0: the row-tile pull kernel
};

// Scalars and flags of the Lanczos driver (device memory, one per solve).
struct LanczosScalars {
  double nrm_old;
  double nrm;
  double beta;
  double inv_beta;
  double w_norm2;  // ||w - α v_k||² of the current iteration (second-pass test of the double-float solve)
  double pad[3];
};
struct LanczosFlags {
  int done;       // converged (set by the eigenvalue test)
  int elit;       // iteration (1-based) at which it stopped
  int second;     // second CGS pass taken in the last iteration
  int n_second;   // number of second passes taken (diagnostic)
  int bad;        // a device-side guard fired
  int exhausted;  // beta == 0: the Krylov space is exhausted
  int exh_k;      // size of T when that happened
  int fastnorm;   // batched form: this iteration's β was taken in the subtraction pass (no second pass)
};

template <class TV>
struct HvEpilogue {
  const LanczosFlags* fl;  // gate: skip when done/exhausted (null: always run)
  const TV* vprev;         // w -= beta * vprev (null: no correction)
  const double* beta;
  double* alpha_part;      // per-CTA partial sums of v·Hv (null: none)
};

// Coefficients of S interaction samples sharing one basis, interleaved
// sample-innermost: value k of sample s at [k*S + s] (FP32 tables, FP64
// one-body diagonals).
struct MultiCoef {
  const float* pp_val;
  const float* nn_val;
  const float* vtab;
  const double* ep;
  const double* en;
  const float2* ep2;  // the one-body diagonals as double-float pairs, same layout
  const float2* en2;
};

struct MultiEpilogue {
  const int* all_done;      // gate: skip when set (null: always run)
  const float* vprev;       // w_s -= beta_s * vprev_s (null: no correction)
  const double* beta_base;  // beta_s = beta_base[s * beta_stride]
  int beta_stride;
  double* alpha_part;       // [s * ntasks + task] partial sums of v_s·(Hv)_s (null: none)
  int* count;               // incremented once per executed launch (null: none)
  float* wh;                // non-null: w written as the double-float pair (wh, wl) instead of FP64
  float* wl;
  const float2* beta2;      // double-float form: beta_s as (hi, lo) at [s]
};

#ifdef __CUDACC__
// Exact float -> double widening with integer instructions only (sign,
// exponent rebias by 1023-127, mantissa shift).  On this GPU the conversion
// instruction shares the FP64 pipe with DFMA, which the FP64 dot products
// already saturate; this form runs on the integer pipe.  Zeros map to zeros;
// subnormal floats (|x| < 1.2e-38) flush to zero; Krylov vectors hold no
// infinities or NaNs.
__device__ __forceinline__ double widen(float x) {
  const uint32_t u = __float_as_uint(x);
  const uint32_t e = (u >> 23) & 0xffu;
  uint32_t hi = (u & 0x80000000u) | ((e + 896u) << 20) | ((u >> 3) & 0xfffffu);
  uint32_t lo = u << 29;
  if (e == 0u) {
    hi = u & 0x80000000u;
    lo = 0u;
  }
  return __hiloint2double((int)hi, (int)lo);
}
__device__ __forceinline__ double widen(double x) { return x; }

// A launch gate evaluated by thread 0 only and broadcast through shared
// memory.  The Lanczos flags are written by kernels on the other stream
// while a CTA starts; reading them once per CTA sends every thread the same
// way, so no thread leaves before a barrier that the others wait at.  Call
// as cta_gate(threadIdx.x == 0 && <condition>) in one-dimensional CTAs.
__device__ __forceinline__ bool cta_gate(bool thread0_value) {
  __shared__ int s_gate;
  if (threadIdx.x == 0) s_gate = thread0_value ? 1 : 0;
  __syncthreads();
  return s_gate != 0;
}
#endif

#define SMGPU_CUDA_TRY(expr)                                                    \
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

const HvConfig* hv_candidates(int* count);
void launch_hv_fp64(const DevTables& t, const TileTables& tt, const HvConfig& cfg, const double* ep,
                    const double* en, const CoefTables<double>& c, const double* v, double* w,
                    const HvEpilogue<double>& epi, cudaStream_t st);
void launch_hv_mixed(const DevTables& t, const TileTables& tt, const HvConfig& cfg, const double* ep,
                     const double* en, const CoefTables<float>& c, const float* v, double* w,
                     const HvEpilogue<float>& epi, cudaStream_t st);
// FP32-mixed H·v with the Lanczos epilogue in double-float: w = wh + wl;
// ep2/en2 the one-body diagonals as (hi, lo) FP32 pairs.
void launch_hv_mixed_df(const DevTables& t, const TileTables& tt, const HvConfig& cfg, const float2* ep2,
                        const float2* en2, const CoefTables<float>& c, const float* v, float* wh, float* wl,
                        const HvEpilogue<float>& epi, cudaStream_t st);
// Staged-pn FP32-mixed H·v (hv_staged.cu): candidate shapes (staged = 1),
// whether a shape fits the problem, its dynamic shared memory, and the
// one-time set-up of that shared-memory size (call before graph capture).
const HvConfig* hv_staged_candidates(int* count);
bool hv_staged_fits(const HvConfig& cfg, const TileTables& tt, int nnmax_raw);
// ext: the single-problem form, whose pp and nn sums come from the two-body
// pass; otherwise the batched body that computes them itself
size_t hv_staged_smem(const HvConfig& cfg, const TileTables& tt, bool ext = false);
void hv_staged_prepare(const HvConfig& cfg, const TileTables& tt);
void launch_hv_staged_mixed(const DevTables& t, const TileTables& tt, const HvConfig& cfg, const double* ep,
                            const double* en, const CoefTables<float>& c, const float* v, double* w,
                            const HvEpilogue<float>& epi, cudaStream_t st);
void launch_hv_staged_mixed_df(const DevTables& t, const TileTables& tt, const HvConfig& cfg, const float2* ep2,
                               const float2* en2, const CoefTables<float>& c, const float* v, float* wh, float* wl,
                               const HvEpilogue<float>& epi, cudaStream_t st);
// The two-body pass of the staged form (hv_2b.cu): pp and nn sums of every
// element into tt.s2b.  Tile sizes, the shared memory of its two kernels, and
// their one-time set-up (call before graph capture).
constexpr int kPPRows = 128;  // rows of a pp task (its 32 columns are the lanes of a warp), <= 32 per warp
constexpr int kNNCols = 256;  // columns of an nn task (its 32 rows are the lanes of a warp)
size_t hv_2b_nn_smem(const TileTables& tt);
size_t hv_2b_pp_smem(const TileTables& tt);
void hv_2b_prepare(const TileTables& tt);
void launch_hv_2b(const DevTables& t, const TileTables& tt, const CoefTables<float>& c, const float* v,
                  const LanczosFlags* fl, cudaStream_t st);
// Multi-sample H·V (hv_multi.cu).  S in {4, 8, 16}; tt1 = one-row tasks
// (ntasks of them); v/w interleaved; cand = index into hv_multi_candidates().
struct MultiHvConfig {
  int nt;    // threads per CTA
  int minb;  // minimum resident CTAs per SM requested from the compiler
  int km;    // neutron entries cached in registers
};
const MultiHvConfig* hv_multi_candidates(int* count);
bool hv_multi_supported(int S);
void launch_hv_multi(int S, int cand, const DevTables& t, const TileTables& tt1, int ntasks, const MultiCoef& c,
                     const float* v, double* w, const MultiEpilogue& epi, cudaStream_t st);

}  // namespace smgpu
