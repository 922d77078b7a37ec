// Batched thick-restart Lanczos: many independent shell-model problems of
// uneven dimension (each its own basis, tables and interaction) iterated in
// lockstep, FP32-mixed.  Every launch covers the whole batch: the H·v over
// the union of all problems' row tiles, the re-orthogonalisation over
// fixed-size chunks of the concatenated vectors (a chunk never crosses a
// problem), and the small per-problem kernels with one CTA per problem.
// A converged problem is frozen while the others continue.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "device.cuh"
#include "hv_tile.cuh"

namespace smgpu {

struct BatchProblemDev {
  HvArgs<float, float> a;  // tables and coefficients (vector fields unused)
  int64_t voff;            // offset of the problem's padded vector in the batch vector
  int64_t len;             // padded length (multiple of 4)
  int64_t mdim;
  int64_t moff;            // offset of the problem's unpadded vector in a concatenation of all problems
  int slot0, nslots;       // H·v tasks (α partial slots) of this problem
  int chunk0, nchunks;     // streaming chunks of this problem
};

struct BatchCtl {
  int all_done;  // every problem has converged
  int ndone;
  int sync_err;  // a grid barrier of the persistent cycle kernel ran out of its wait limit
  int pad1;
};

// Grid barrier state of the persistent cycle kernel (zeroed before each
// launch): CTAs arrive in groups of kSyncGroup on their own counters, the
// last arriver of a group on the top counter, and each group polls its own
// release word; every counter and release word has a 128-byte line to
// itself, so arrivals and polls spread over the L2 slices.
constexpr int kSyncGroup = 32;
constexpr int kSyncMaxGroups = 256;  // up to 8,192 CTAs
struct GridSync {
  unsigned count;  // top counter: groups arrived
  unsigned pad[31];
  unsigned group[kSyncMaxGroups][32];  // per-group arrival counter in word 0 of its line
  unsigned rel[kSyncMaxGroups][32];    // per-group release generation in word 0 of its line
};

// One restart cycle of the batched Lanczos as one persistent (cooperative)
// launch: iterations kstart .. lm-1, each phase of an iteration (H·v over
// a device task queue with the previous iteration's eigenvalue tests, the
// re-orthogonalisation passes, β and the next vector) separated by a grid
// barrier, and the last eigenvalue test.
struct BatchCycle {
  const int4* tasks;    // H·v tasks (problem, block, first row, α slot), largest first
  int ntasks;
  int* task_ctr;        // lm counters: the H·v task queue of each iteration (zeroed before the launch)
  int* hv_count;        // batched H·v iterations executed
  GridSync* gs;
  long long spin_limit; // polls of a barrier wait before it gives up (sync_err)
  int kstart, lock;
};

struct BatchDev {
  int nprob, lm, ls, num_ev, nh;
  double tol;
  double fastnorm;    // β from the norm before the subtraction when Σh² <= fastnorm ||w'||²
  int nchunks;        // chunks of the batch vector
  int nslots;         // H·v tasks
  int64_t LEN;        // batch vector length (slot stride of V and U)
  const BatchProblemDev* probs;
  const int4* chunks; // (problem, begin, end, -), local element indices, begin a multiple of 4
  double* T;          // nprob x lm x lm
  double* en;         // nprob x nh x num_ev
  double* alpha_part; // lm x nslots
  double* pdot;       // (lm+2) x nchunks
  double* pn1;        // nchunks
  double* pdot2;      // (lm+2) x nchunks
  double* pn2;        // nchunks
  double* part;       // gram pairs x nchunks
  double* jacA;       // nprob x lm x lm
  double* jacZ;
  double* evals;      // nprob x lm
  float* Yf;          // nprob x (lm-1) x ls
  float* wsplit;      // 2 x LEN: FP32 (hi, lo) split of w' (first re-orthogonalisation pass)
  double* X;          // nprob x ls x ls
  float* Xf;          // nprob x (ls*ls + ls)
  double* cvec;       // nprob x ls
  LanczosFlags* fl;   // nprob
  BatchCtl* ctl;
};

// H·v epilogue of a batched launch.
struct BatchEpi {
  const BatchCtl* ctl;       // gate (null: always run)
  const LanczosFlags* fl;    // per-problem gate (null: none)
  const float* vprev;        // batch vector of the previous Lanczos vector (null: no correction)
  const double* T;           // β_p = T[p*lm*lm + (it0-1)*lm + it0]
  int lm, it0;
  double* alpha_part;        // indexed by task slot (null: none)
  int* count;                // incremented once per launch while some problem runs (null: none)
};

constexpr int kBatchQM = 3;  // output columns per thread of the staged batch H·v bodies

struct BatchHvConfig {
  int nt, rows, minb;
  int staged;  // 1: the staged pn row body (hv_staged.cuh); 0: the row-tile body
};
const BatchHvConfig* hv_batch_candidates(int* count);
// Column capacity (threads x columns per thread) of a staged batch shape.
int hv_batch_staged_cols(const BatchHvConfig& c);
// tasks: (problem, block, first row, α slot), cand: index into hv_batch_candidates();
// smem: dynamic shared memory of a staged shape (the largest over the problems)
void launch_hv_batch(int cand, const BatchProblemDev* probs, const int4* tasks, int ntasks, const float* v, double* w,
                     const BatchEpi& epi, size_t smem, cudaStream_t st);
// One-time set-up of a staged shape's shared-memory size (before graph capture).
void hv_batch_prepare(int cand, size_t smem);

void launch_b_start(const BatchDev& B, uint64_t seed, double* w, cudaStream_t st);
void launch_b_to_padded(const BatchDev& B, const double* src, double* w, cudaStream_t st);  // src: problems' mdim concatenated
void launch_b_from_padded(const BatchDev& B, const double* w, double* dst, cudaStream_t st);
void launch_b_convert(const BatchDev& B, const double* w, float* v, cudaStream_t st);
void launch_b_init(const BatchDev& B, const double* w, float* V0, cudaStream_t st);
void launch_b_sturm(const BatchDev& B, int k, int lock, cudaStream_t st);
void launch_b_orth(const BatchDev& B, float* V, double* w, int it0, cudaStream_t st);
void launch_b_cycle_end(const BatchDev& B, cudaStream_t st);
// The persistent cycle kernel for the H·v launch shape `cand` (of
// hv_batch_candidates) with dynamic shared memory smem_hv for its H·v body.
// persist_supported: whether that shape has a persistent form.
bool persist_supported(int cand);
// Grid size (co-resident CTAs) of the persistent kernel, 0 when it cannot run.
int persist_grid(int cand, const BatchDev& B, size_t smem_hv);
void launch_b_persist_cycle(int cand, const BatchDev& B, float* V, double* w, const BatchCycle& C, size_t smem_hv,
                            int grid, cudaStream_t st);
void launch_b_restart(const BatchDev& B, float* V, float* U, cudaStream_t st);
// Ritz vectors of problem p: Jacobi of its T[0:n,0:n], then R (nev x len, FP64, padded)
void launch_b_jacobi_one(const BatchDev& B, int p, int n, cudaStream_t st);
void launch_b_ritz(const BatchDev& B, const float* V, int p, int elit, int nev, int64_t len, double* R,
                   cudaStream_t st);

}  // namespace smgpu
