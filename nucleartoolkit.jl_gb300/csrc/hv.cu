// H·v for the M-scheme shell-model Hamiltonian on sm_103a.
//
// Replaces operate_H! (src/ShellModel/lanczos_methods.jl:153-248).  The
// reference walks (block pair, V entry) lists and scatters into twf from one
// thread per block.  Here the output is tiled by rows of a (Mp,Mn) block — a
// row is one proton Slater determinant p with all its neutron partners n —
// and every CTA owns R consecutive rows of one block, pulls every
// contribution to them and writes each output element exactly once:
//
//   w[b,p,n] = (e_p + e_n) v[b,p,n]                         one-body
//            + Σ_{p'} Hpp[p,p'] v[b,p',n]                    pp (coalesced rows)
//            + Σ_{n'} Hnn[n,n'] v[b,p,n']                    nn
//            + Σ_links Σ_{(p',a†c,±)} ± Σ_{(n',b†d,±)} V[ac][bd] v[s,p',n']   pn
//
// The pn term is factorised per link (output block b <- source block s): the
// proton pull entries of each row (source row p', operator index, sign) are
// combined with the neutron pull list of the link.  A thread owns one column
// n; its neutron list for the link (at most 16 entries for the pf shell) is
// loaded once into registers and reused for all proton entries of the R rows.
// The per-ΔM coefficient table is stored twice (V and −V) so the neutron sign
// is folded into the table index.  No atomics; no scratch.
//
// Lanczos epilogue (optional): per-CTA partial sums of α = v·Hv (FP64) and
// the three-term correction w = Hv − β v_prev, so the re-orthogonalisation
// passes start from the Lanczos residual.
//
// Precision forms
//   FP64 plain : v, coefficients, accumulation FP64.
//   mixed      : v and coefficients FP32; FP32 partial sums per (row, link) and
//                per pp/nn entry, combined with Kahan compensation; the
//                one-body term, the epilogue and the output in FP64.
#include "device.cuh"
#include "hv_tile.cuh"
#include "lanczos.cuh"

namespace smgpu {

template <class TV, class TC, class Acc, int NT, int R, int MINB, bool DF>
__global__ void __launch_bounds__(NT, MINB) hv_tile_kernel(const HvArgs<TV, TC> a) {
  if (a.fl != nullptr && cta_gate(threadIdx.x == 0 && (a.fl->done || a.fl->exhausted))) return;
  const int task = blockIdx.x;
  const double beta = (a.vprev != nullptr) ? *a.beta : 0.0;
  hv_tile_rows<TV, TC, Acc, NT, R, DF>(a, a.v, a.w, a.vprev, a.tt.task_b[task], a.tt.task_p0[task], beta,
                                       a.alpha_part != nullptr ? a.alpha_part + task : nullptr);
}

// ---------------------------------------------------------------- dispatch
template <class TV, class TC, class Acc, bool DF>
static void launch_cfg(const HvConfig& cfg, const HvArgs<TV, TC>& a, cudaStream_t st) {
  const int grid = cfg.ntasks;
#define SMGPU_HV_CASE(NT_, R_, MB_)                                           \
  if (cfg.nt == NT_ && cfg.rows == R_ && cfg.minb == MB_) {                   \
    hv_tile_kernel<TV, TC, Acc, NT_, R_, MB_, DF><<<grid, NT_, 0, st>>>(a);   \
    return;                                                                   \
  }
  SMGPU_HV_CASE(128, 1, 1)
  SMGPU_HV_CASE(128, 2, 1)
  SMGPU_HV_CASE(128, 4, 1)
  SMGPU_HV_CASE(128, 8, 1)
  SMGPU_HV_CASE(128, 1, 8)
  SMGPU_HV_CASE(128, 2, 6)
  SMGPU_HV_CASE(128, 4, 6)
  SMGPU_HV_CASE(192, 2, 4)
  SMGPU_HV_CASE(256, 1, 1)
  SMGPU_HV_CASE(256, 2, 1)
  SMGPU_HV_CASE(256, 4, 1)
  SMGPU_HV_CASE(256, 2, 3)
  SMGPU_HV_CASE(256, 4, 3)
#undef SMGPU_HV_CASE
}

const HvConfig* hv_candidates(int* count) {
  // {threads, rows per CTA, -, min CTAs per SM (register cap)}
  static const HvConfig c[] = {{128, 1, 0, 1}, {128, 2, 0, 1}, {128, 4, 0, 1}, {128, 8, 0, 1}, {128, 1, 0, 8},
                               {128, 2, 0, 6}, {128, 4, 0, 6}, {192, 2, 0, 4}, {256, 1, 0, 1}, {256, 2, 0, 1},
                               {256, 4, 0, 1}, {256, 2, 0, 3}, {256, 4, 0, 3}};
  *count = (int)(sizeof(c) / sizeof(c[0]));
  return c;
}

void launch_hv_fp64(const DevTables& t, const TileTables& tt, const HvConfig& cfg, const double* ep,
                    const double* en, const CoefTables<double>& c, const double* v, double* w,
                    const HvEpilogue<double>& epi, cudaStream_t st) {
  HvArgs<double, double> a{t, tt, c, ep, en, v, w, epi.fl, epi.vprev, epi.beta, epi.alpha_part,
                           nullptr, nullptr, nullptr, nullptr};
  launch_cfg<double, double, AccF64, false>(cfg, a, st);
}

void launch_hv_mixed(const DevTables& t, const TileTables& tt, const HvConfig& cfg, const double* ep,
                     const double* en, const CoefTables<float>& c, const float* v, double* w,
                     const HvEpilogue<float>& epi, cudaStream_t st) {
  HvArgs<float, float> a{t, tt, c, ep, en, v, w, epi.fl, epi.vprev, epi.beta, epi.alpha_part,
                         nullptr, nullptr, nullptr, nullptr};
  launch_cfg<float, float, AccKahan, false>(cfg, a, st);
}

void launch_hv_mixed_df(const DevTables& t, const TileTables& tt, const HvConfig& cfg, const float2* ep2,
                        const float2* en2, const CoefTables<float>& c, const float* v, float* wh, float* wl,
                        const HvEpilogue<float>& epi, cudaStream_t st) {
  HvArgs<float, float> a{t, tt, c, nullptr, nullptr, v, nullptr, epi.fl, epi.vprev, epi.beta, epi.alpha_part,
                         wh, wl, ep2, en2};
  launch_cfg<float, float, AccKahan, true>(cfg, a, st);
}

}  // namespace smgpu
