// Device kernels of the thick-restart Lanczos driver (lanczos.cu).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include <cstdlib>

#include "device.cuh"

namespace smgpu {

// Reduction modes of k_reduce (what to do with the reduced sums).
enum ReduceMode {
  RED_STORE = 0,    // out[j] = sum_j
  RED_INVNORM = 5   // out[j] = 1/sqrt(sum_j)
};

// β from the norm before the subtraction (FP32-mixed forms): with the FP32
// basis V orthonormal up to its rounding E, ||w' - Σ h_j v_j||² = ||w'||² -
// Σ h_j² + hᵀE h, and when Σ h_j² <= kFastNorm ||w'||² the last term is below
// 1e-15 of the result.  Then the subtraction pass also forms β and the next
// basis vector, and the second-pass test and the scaling pass are skipped
// (no second pass can be needed: ||w''||² >= (1 - kFastNorm) ||w'||²).
constexpr double kFastNorm = 1e-8;
// The threshold a solve uses: kFastNorm, or -1 (never: every iteration takes
// the norm after the subtraction) with SMGPU_FASTNORM=0, which the tests use
// to cover both paths.
inline double fastnorm_threshold() {
  const char* e = std::getenv("SMGPU_FASTNORM");
  return (e && e[0] == '0') ? -1.0 : kFastNorm;
}

struct LanczosDev {
  int G;                // CTAs of the streaming reduction kernels
  int lm, ls, num_ev, nh;
  int64_t len;          // padded vector length
  int64_t mdim;
  double tol;
  int nalpha;           // CTAs of the H·v kernel (partials of α per iteration)
  double* T;            // lm x lm, column-major
  double* en;           // nh x num_ev
  double* alpha_part;   // lm x nalpha: per-iteration partials of α (H·v epilogue)
  double* pdot;         // (lm+2) x G: first-pass dot partials; slot m = ||w'||²
  double* pn1;          // G: ||w''||² partials after the first pass
  double* pdot2;        // (lm+2) x G: second-pass dot partials
  double* pn2;          // G: norm partials after the second pass
  double* partials;     // (max(lm, gram)+2) x G: general reductions
  double* h;            // lm + 2
  double* jacA;         // lm x lm
  double* jacZ;         // lm x lm
  double* evals;        // lm
  float* Yf;            // (lm-1) x ls: FP32 copy of the restart rotation
  float* wsplit;        // 2 x len: the residual w = hi + lo in double-float (FP32 basis only)
  double* gram;         // ls*(ls+1)/2 + ls (restart Gram matrix, packed)
  double* X;            // ls x ls (restart: inverse Cholesky factor)
  double* cvec;         // ls
  LanczosScalars* sc;
  LanczosFlags* fl;
  int alpha_df;         // 1: alpha_part holds double-float (hi, lo) float pairs (FP32-mixed H·v)
  double fastnorm;      // β from the norm before the subtraction when Σh² <= fastnorm ||w'||² (FP32 basis)
};

void launch_start_vector(const DevTables& t, uint64_t seed, double* w, cudaStream_t st);
void launch_convert(const double* a, float* b, int64_t len, cudaStream_t st);
template <class TX>
void launch_multidot(const LanczosDev& L, const TX* X, int m, const double* y, bool self, cudaStream_t st);
void launch_reduce(const LanczosDev& L, int m, ReduceMode mode, double* out, cudaStream_t st);
template <class TX>
void launch_scale_store(const LanczosDev& L, const double* w, TX* out, const double* scale, cudaStream_t st);

// One Lanczos iteration after the H·v (it0 = 0-based iteration index):
// w' = w - alpha v_it0, first CGS pass, conditional second pass, beta and v_{it0+1}.
template <class TX>
void launch_orth_iteration(const LanczosDev& L, TX* V, double* w, int it0, cudaStream_t st);
// The same for an FP32 basis with the residual kept in double-float, w = wh + wl.
void launch_orth_iteration_df(const LanczosDev& L, float* V, float* wh, float* wl, int it0, cudaStream_t st);
void launch_sturm(const LanczosDev& L, int it, int lock, cudaStream_t st);
// df: the double-float Jacobi (orders above kJacobiSmemN use FP64); refined:
// the FP64 Jacobi started from an FP32 Jacobi's eigenbasis (FP32-mixed
// solves, orders up to kJacobiRefineN); otherwise the plain FP64 Jacobi.
void launch_jacobi(const LanczosDev& L, int n, bool gate_on_done, bool df, bool refined, cudaStream_t st);
void launch_restart_small(const LanczosDev& L, cudaStream_t st);
template <class TX>
void launch_restart_rotate(const LanczosDev& L, const TX* V, TX* U, cudaStream_t st);
// df: FP32 vectors summed in double-float (SMGPU_MIXED_DF); otherwise FP64
template <class TX>
void launch_gram(const LanczosDev& L, const TX* U, const TX* vlast, bool df, cudaStream_t st);
// df: the partials of the FP32-basis Gram kernel ((hi, lo) pairs)
void launch_gram_reduce(const LanczosDev& L, bool df, cudaStream_t st);
// df: the double-float form on one warp (FP32-mixed solves, ls <= 32)
void launch_chol(const LanczosDev& L, bool df, cudaStream_t st);
// df: FP32 vectors combined in compensated FP32 (the FP32-mixed solves, whose
// updated basis is stored in FP32); otherwise FP64
template <class TX>
void launch_restart_apply(const LanczosDev& L, const TX* U, TX* V, bool df, cudaStream_t st);
template <class TX>
void launch_ritz(const LanczosDev& L, const TX* V, int elit, int nev, double* R, cudaStream_t st);
// J-projected Lanczos helpers: FP64 copies, y -= Σ h_j X_j, out = Σ c_j Q_j,
// and a one-CTA eigen-decomposition of a small matrix in device memory.
template <class TX>
void launch_widen(const TX* in, double* out, int64_t len, cudaStream_t st);
template <class TX>
void launch_narrow(const double* in, TX* out, int64_t len, cudaStream_t st);
template <class TX>
void launch_axpy_dev(const TX* X, int64_t ld, int m, const double* h, double* y, int64_t len, cudaStream_t st);
void launch_combine(const double* Q, int64_t ld, int m, const double* c, double* out, int64_t len, cudaStream_t st);
void launch_small_eig(const double* T, int n, double* A, double* Z, double* evals, cudaStream_t st);
template <class TX>
void launch_to_padded(const DevTables& t, const double* src, TX* dst, cudaStream_t st);
void launch_from_padded(const DevTables& t, const double* src, double* dst, cudaStream_t st);

}  // namespace smgpu
