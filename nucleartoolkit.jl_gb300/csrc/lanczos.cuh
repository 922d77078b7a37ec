// Device kernels of the thick-restart Lanczos driver (lanczos.cu).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "device.cuh"

namespace smgpu {

// Reduction modes of k_reduce (what to do with the reduced sums).
enum ReduceMode {
  RED_STORE = 0,      // out[j] = sum_j
  RED_ALPHA = 1,      // T[it,it] = sum_0                     (it 0-based)
  RED_H = 2,          // h[j] = sum_j (j < m), nrm_old = sum_m
  RED_NRM_CHECK = 3,  // nrm = sum_0; second-pass flag = nrm < 0.5 * nrm_old
  RED_NRM = 4,        // nrm = sum_0 (second pass)
  RED_INVNORM = 5     // out[j] = 1/sqrt(sum_j)
};

// Scalars and flags that live in device memory (one block per handle).
struct LanczosScalars {
  double nrm_old;   // ||w||^2 before the orthogonalisation pass
  double nrm;       // ||w||^2 after the last pass
  double beta;
  double inv_beta;
  double pad[4];
};
struct LanczosFlags {
  int done;         // converged (set by the eigenvalue test)
  int elit;         // iteration (1-based) at which it stopped
  int second;       // second CGS pass requested
  int n_second;     // number of second passes taken (diagnostic)
  int bad;          // a device-side guard fired
  int exhausted;    // beta == 0: the Krylov space is exhausted
  int exh_k;        // size of T when that happened
  int pad;
};

struct LanczosDev {
  int G;                // CTAs of the reduction kernels
  int lm, ls, num_ev, nh;
  int64_t len;          // padded vector length
  int64_t mdim;
  double tol;
  double* T;            // lm x lm, column-major
  double* en;           // nh x num_ev
  double* partials;     // (lm+2) x G
  double* h;            // lm + 2
  double* jacA;         // lm x lm
  double* jacZ;         // lm x lm
  double* evals;        // lm
  double* gram;         // ls*(ls+1)/2 + ls (restart Gram matrix, packed)
  double* X;            // ls x ls (restart: inverse Cholesky factor)
  double* cvec;         // ls
  LanczosScalars* sc;
  LanczosFlags* fl;
};

void launch_start_vector(const DevTables& t, uint64_t seed, double* w, cudaStream_t st);
void launch_scale_store_plain(const double* a, float* b, int64_t len, cudaStream_t st);
template <class TX>
void launch_multidot(const LanczosDev& L, const TX* X, int m, const double* y, bool self, const int* gate,
                     cudaStream_t st);
void launch_reduce(const LanczosDev& L, int m, ReduceMode mode, double* out, int it, const int* gate, cudaStream_t st);
template <class TX>
void launch_multiaxpy(const LanczosDev& L, const TX* X, int m, double* y, const int* gate, cudaStream_t st);
void launch_beta(const LanczosDev& L, int it, cudaStream_t st);
template <class TX>
void launch_scale_store(const LanczosDev& L, const double* w, TX* out, const double* scale, const int* gate,
                        cudaStream_t st);
void launch_sturm(const LanczosDev& L, int it, int lock, cudaStream_t st);
void launch_jacobi(const LanczosDev& L, int n, bool gate_on_done, cudaStream_t st);
void launch_restart_small(const LanczosDev& L, cudaStream_t st);
template <class TX>
void launch_restart_rotate(const LanczosDev& L, const TX* V, TX* U, cudaStream_t st);
template <class TX>
void launch_gram(const LanczosDev& L, const TX* U, const TX* vlast, cudaStream_t st);
void launch_chol(const LanczosDev& L, cudaStream_t st);
template <class TX>
void launch_restart_apply(const LanczosDev& L, const TX* U, TX* V, cudaStream_t st);
template <class TX>
void launch_ritz(const LanczosDev& L, const TX* V, int elit, int nev, double* R, cudaStream_t st);
template <class TX>
void launch_to_padded(const DevTables& t, const double* src, TX* dst, cudaStream_t st);
void launch_from_padded(const DevTables& t, const double* src, double* dst, cudaStream_t st);

}  // namespace smgpu
