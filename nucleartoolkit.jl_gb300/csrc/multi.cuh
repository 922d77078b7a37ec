// Multi-sample thick-restart Lanczos: S interaction samples that share one
// basis, iterated in lockstep on S-interleaved FP32 Krylov vectors
// (v[i*S + s]) with one multi-sample H·V per iteration.  Every sample keeps
// its own Lanczos matrix, convergence test, restart and flags; a sample that
// has converged is frozen (its basis and T are no longer written) while the
// others continue.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "device.cuh"

namespace smgpu {

struct MultiCtl {
  int all_done;    // every sample has converged (gate of all kernels)
  int ndone;       // samples that have converged
  int any_second;  // some sample takes the second Gram-Schmidt pass this iteration
  int pad;
};

struct MultiDev {
  int S, G, lm, ls, num_ev, nh, nalpha;
  int64_t len;   // padded vector length (rows); vectors hold len*S values
  int64_t mdim;
  double tol;
  double* T;           // S x lm x lm (column-major per sample)
  double* en;          // S x nh x num_ev
  double* alpha_part;  // lm x S x nalpha (H·V epilogue partials)
  double* part;        // max(lm+2, gram pairs) x S x G streaming partials
  double* h1;          // (lm+2) x S: first-pass dots, slot m = ||w'||²
  double* h2;          // (lm+2) x S: second-pass dots
  double* nrm1;        // S: ||w''||² after the first pass
  double* nrm2;        // S: after the second pass
  double* invb;        // S: 1/β of the live samples, 0 otherwise
  int* sec;            // S: second pass taken
  double* jacA;        // S x lm x lm
  double* jacZ;        // S x lm x lm
  double* evals;       // S x lm
  float* Yf;           // S x (lm-1) x ls (restart rotation, FP32)
  float* wsplit;       // 2 x len x S: the residual w = hi + lo in double-float (the iterations' w)
  float2* beta2;       // S: β of each sample as a double-float pair (H·V epilogue)
  double* gram;        // P x S (packed Gram matrices, sample innermost)
  double* X;           // S x ls x ls
  float* Xf;           // S x (ls*ls + ls): X then c, FP32
  double* cvec;        // S x ls
  LanczosFlags* fl;    // S
  MultiCtl* ctl;
};

void launch_m_start(int S, const DevTables& t, uint64_t seed, double* w, cudaStream_t st);
void launch_m_to_padded(int S, const DevTables& t, const double* src, double* w, cudaStream_t st);
void launch_m_to_padded_f(int S, const DevTables& t, const double* src, float* v, cudaStream_t st);
void launch_m_from_padded(int S, const DevTables& t, const double* w, double* dst, cudaStream_t st);
// V[0] = w / ||w|| per sample
void launch_m_init(const MultiDev& M, const double* w, float* V0, cudaStream_t st);
void launch_m_alpha(const MultiDev& M, int it0, cudaStream_t st);
void launch_m_sturm(const MultiDev& M, int k, int lock, cudaStream_t st);
// orthogonalisation, β and v_{it0+1} after the H·V and α of iteration it0
void launch_m_orth(const MultiDev& M, float* V, float* wh, float* wl, int it0, cudaStream_t st);
void launch_m_cycle_end(const MultiDev& M, cudaStream_t st);
void launch_m_restart(const MultiDev& M, float* V, float* U, cudaStream_t st);
// Ritz vectors of sample s: R (nev x len, FP64, padded) from jacA of that sample
void launch_m_jacobi_one(const MultiDev& M, int s, int n, cudaStream_t st);
void launch_m_ritz(const MultiDev& M, const float* V, int s, int elit, int nev, double* R, cudaStream_t st);

}  // namespace smgpu
