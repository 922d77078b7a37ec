// FP32-mixed H·v with the pn term in two shared-memory stages.
//
// Same output, tiling and epilogue as the row-tile kernel (hv.cu): a CTA owns
// R consecutive rows (proton Slater determinants p) of one (Mp,Mn) block and
// writes each of their elements once.  What differs is the pn term of a link
// (output block b <- source block s):
//
//   w[p,n] += Σ_{(p',ia,±)∈P(p)} Σ_{(n',ib,±)∈N(n)} ± V[ia][ib] v[s,p',n']
//
// The row-tile kernel evaluates that sum per (row, column) with two gathers
// per update (the coefficient and v), both through L1; on GB300 those
// scattered loads, not HBM, bound it.  Here the sum is re-associated:
//
//   stage 1, one thread per SOURCE column n':  for every neutron operator ib
//            that leaves n' in the block (the "push" list of n'),
//            y = Σ_{(p',ia,±)} (±V[ia][ib]) v[s,p',n'] — the proton entries'
//            coefficients for this row are first gathered into a dense
//            matrix A[ib][j] in shared memory, so the inner loop is one
//            float4 shared load per four FMAs with v[s,p',n'] in registers;
//            y goes to the slot of its output column in shared memory.
//   stage 2, one thread per OUTPUT column n: the sum of its slots (the slots
//            of column n are laid out [t][n], so a warp reads consecutive
//            words), added to the column's Kahan-compensated pn sum.
//
// Every update is still one FP32 multiply-add, in the order of the proton
// entries; the partial sums are FP32 per (row, link, neutron entry), combined
// with Kahan compensation per (row, link) as in the row-tile kernel.  The pp
// and nn terms come from the two-body pass (hv_2b.cu), launched just before
// on the same stream, which leaves them per element in tt.s2b; the one-body
// term and the Lanczos epilogue are those of hv_tile.cuh.  (The batched
// kernel, hv_batch.cu, runs the same row body with the pp and nn terms
// computed in the kernel.)

#include "device.cuh"
#include "hv_staged.cuh"
#include "hv_tile.cuh"

namespace smgpu {

namespace {

template <int NT, int R, int QM, int MINB, bool DF>
__global__ void __launch_bounds__(NT, MINB) hv_staged_kernel(const HvArgs<float, float> a) {
  if (a.fl != nullptr && cta_gate(threadIdx.x == 0 && (a.fl->done || a.fl->exhausted))) return;
  const int task = blockIdx.x;
  const double beta = (a.vprev != nullptr) ? *a.beta : 0.0;
  hv_staged_rows<NT, R, QM, DF, true>(a, a.v, a.w, a.vprev, beta, a.tt.task_b[task], a.tt.task_p0[task],
                                      a.alpha_part != nullptr ? a.alpha_part + task : nullptr);
}

// {threads, rows, -, min CTAs per SM, staged}; a thread owns up to
// qm_for(threads) output columns.
constexpr int qm_for(int nt) { return nt <= 128 ? 5 : 3; }
constexpr HvConfig kStagedCand[] = {{128, 1, 0, 1, 1}, {128, 1, 0, 4, 1}, {128, 1, 0, 5, 1}, {128, 1, 0, 6, 1},
                                    {128, 2, 0, 3, 1},
                                    {192, 1, 0, 2, 1}, {192, 2, 0, 2, 1}, {256, 1, 0, 1, 1}, {256, 1, 0, 2, 1},
                                    {256, 2, 0, 2, 1}};

template <bool DF>
bool dispatch(const HvConfig& cfg, const HvArgs<float, float>& a, size_t smem, cudaStream_t st, bool prepare) {
#define SMGPU_ST_CASE(NT_, R_, MB_)                                                                     \
  if (cfg.nt == NT_ && cfg.rows == R_ && cfg.minb == MB_) {                                             \
    auto k = hv_staged_kernel<NT_, R_, qm_for(NT_), MB_, DF>;                                           \
    if (prepare) {                                                                                      \
      SMGPU_CUDA_TRY(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem)); \
    } else {                                                                                            \
      k<<<cfg.ntasks, NT_, smem, st>>>(a);                                                              \
    }                                                                                                   \
    return true;                                                                                        \
  }
  SMGPU_ST_CASE(128, 1, 1)
  SMGPU_ST_CASE(128, 1, 4)
  SMGPU_ST_CASE(128, 1, 5)
  SMGPU_ST_CASE(128, 1, 6)
  SMGPU_ST_CASE(128, 2, 3)
  SMGPU_ST_CASE(192, 1, 2)
  SMGPU_ST_CASE(192, 2, 2)
  SMGPU_ST_CASE(256, 1, 1)
  SMGPU_ST_CASE(256, 1, 2)
  SMGPU_ST_CASE(256, 2, 2)
#undef SMGPU_ST_CASE
  return false;
}

}  // namespace

const HvConfig* hv_staged_candidates(int* count) {
  *count = (int)(sizeof(kStagedCand) / sizeof(kStagedCand[0]));
  return kStagedCand;
}

size_t hv_staged_smem(const HvConfig& cfg, const TileTables& tt, bool ext) {
  const size_t R = (size_t)cfg.rows;
  return sizeof(float) * R * ((size_t)tt.ymax + (size_t)tt.nbmax * tt.astride + (ext ? 0 : (size_t)tt.nnmax)) +
         sizeof(int) * R * (size_t)tt.kpad;
}

bool hv_staged_fits(const HvConfig& cfg, const TileTables& tt, int nnmax_raw) {
  if (tt.push_ent == nullptr || tt.s2b == nullptr) return false;
  if (nnmax_raw > cfg.nt * qm_for(cfg.nt)) return false;
  return hv_staged_smem(cfg, tt, true) <= 200 * 1024 && hv_2b_nn_smem(tt) <= 200 * 1024 &&
         hv_2b_pp_smem(tt) <= 200 * 1024;
}

void hv_staged_prepare(const HvConfig& cfg, const TileTables& tt) {
  const size_t smem = hv_staged_smem(cfg, tt, true);
  HvArgs<float, float> a{};
  dispatch<false>(cfg, a, smem, nullptr, true);
  dispatch<true>(cfg, a, smem, nullptr, true);
  hv_2b_prepare(tt);
}

void launch_hv_staged_mixed(const DevTables& t, const TileTables& tt, const HvConfig& cfg, const double* ep,
                            const double* en, const CoefTables<float>& c, const float* v, double* w,
                            const HvEpilogue<float>& epi, cudaStream_t st) {
  HvArgs<float, float> a{t, tt, c, ep, en, v, w, epi.fl, epi.vprev, epi.beta, epi.alpha_part,
                         nullptr, nullptr, nullptr, nullptr};
  launch_hv_2b(t, tt, c, v, epi.fl, st);
  if (!dispatch<false>(cfg, a, hv_staged_smem(cfg, tt, true), st, false))
    throw CudaError{cudaErrorInvalidConfiguration, "staged H·v launch shape", __FILE__, __LINE__};
}

void launch_hv_staged_mixed_df(const DevTables& t, const TileTables& tt, const HvConfig& cfg, const float2* ep2,
                               const float2* en2, const CoefTables<float>& c, const float* v, float* wh, float* wl,
                               const HvEpilogue<float>& epi, cudaStream_t st) {
  HvArgs<float, float> a{t, tt, c, nullptr, nullptr, v, nullptr, epi.fl, epi.vprev, epi.beta, epi.alpha_part,
                         wh, wl, ep2, en2};
  launch_hv_2b(t, tt, c, v, epi.fl, st);
  if (!dispatch<true>(cfg, a, hv_staged_smem(cfg, tt, true), st, false))
    throw CudaError{cudaErrorInvalidConfiguration, "staged H·v launch shape", __FILE__, __LINE__};
}

}  // namespace smgpu
