// Batched H·v: one launch over the row tiles of every problem of a batch
// (operate_H!, src/ShellModel/lanczos_methods.jl:153-248, for many problems
// at once).  Each CTA takes one task (problem, block, first row, α slot) from
// a list sorted by estimated work, largest first, and runs either the
// row-tile body of hv.cu or the staged pn body of hv_staged.cu on that
// problem's tables and vector segment (FP32-mixed; the autotuner picks the
// launch shape, staged shapes only where every problem fits them).  The
// per-problem tables are read through a reference into a device array, so a
// CTA touches only the fields its rows use.
#include "batch.cuh"
#include "hv_staged.cuh"

namespace smgpu {

namespace {

template <int NT, int R, int MINB>
__global__ void __launch_bounds__(NT, MINB) hv_batch_kernel(const BatchProblemDev* __restrict__ probs,
                                                            const int4* __restrict__ tasks, const float* v,
                                                            double* w, const BatchEpi e) {
  const int4 tk = tasks[blockIdx.x];
  if (e.count != nullptr && blockIdx.x == 0 && threadIdx.x == 0 && !(e.ctl != nullptr && e.ctl->all_done))
    atomicAdd(e.count, 1);
  if (cta_gate(threadIdx.x == 0 && ((e.ctl != nullptr && e.ctl->all_done) ||
                                     (e.fl != nullptr && (e.fl[tk.x].done || e.fl[tk.x].exhausted)))))
    return;
  const BatchProblemDev& P = probs[tk.x];
  const int64_t off = P.voff;
  double beta = 0.0;
  const float* vprev = nullptr;
  if (e.vprev != nullptr) {
    vprev = e.vprev + off;
    beta = e.T[(int64_t)tk.x * e.lm * e.lm + (int64_t)(e.it0 - 1) * e.lm + e.it0];
  }
  hv_tile_rows<float, float, AccKahan, NT, R>(P.a, v + off, w + off, vprev, tk.y, tk.z, beta,
                                              e.alpha_part != nullptr ? e.alpha_part + tk.w : nullptr);
}

// The staged pn row body (hv_staged.cuh) on the batch's tasks.
template <int NT, int R, int MINB>
__global__ void __launch_bounds__(NT, MINB) hv_batch_staged_kernel(const BatchProblemDev* __restrict__ probs,
                                                                   const int4* __restrict__ tasks, const float* v,
                                                                   double* w, const BatchEpi e) {
  const int4 tk = tasks[blockIdx.x];
  if (e.count != nullptr && blockIdx.x == 0 && threadIdx.x == 0 && !(e.ctl != nullptr && e.ctl->all_done))
    atomicAdd(e.count, 1);
  if (cta_gate(threadIdx.x == 0 && ((e.ctl != nullptr && e.ctl->all_done) ||
                                     (e.fl != nullptr && (e.fl[tk.x].done || e.fl[tk.x].exhausted)))))
    return;
  const BatchProblemDev& P = probs[tk.x];
  const int64_t off = P.voff;
  double beta = 0.0;
  const float* vprev = nullptr;
  if (e.vprev != nullptr) {
    vprev = e.vprev + off;
    beta = e.T[(int64_t)tk.x * e.lm * e.lm + (int64_t)(e.it0 - 1) * e.lm + e.it0];
  }
  hv_staged_rows<NT, R, kBatchQM, false>(P.a, v + off, w + off, vprev, beta, tk.y, tk.z,
                                     e.alpha_part != nullptr ? e.alpha_part + tk.w : nullptr);
}

// {threads, rows, min CTAs per SM, staged}; launch_hv_batch and staged_case
// map each index to its template instance.
constexpr BatchHvConfig kBatchCand[] = {
    {32, 4, 1, 0},  {64, 2, 1, 0},  {64, 4, 1, 0},  {128, 1, 1, 0}, {128, 2, 1, 0}, {128, 4, 1, 0},
    {128, 2, 6, 0}, {256, 2, 1, 0}, {64, 1, 8, 1},  {128, 1, 4, 1}, {128, 1, 5, 1}, {128, 2, 3, 1},
};

template <int NT, int R, int MINB>
void launch_one(const BatchProblemDev* probs, const int4* tasks, int ntasks, const float* v, double* w,
                const BatchEpi& e, cudaStream_t st) {
  hv_batch_kernel<NT, R, MINB><<<ntasks, NT, 0, st>>>(probs, tasks, v, w, e);
}
template <int NT, int R, int MINB>
void launch_staged(const BatchProblemDev* probs, const int4* tasks, int ntasks, const float* v, double* w,
                   const BatchEpi& e, size_t smem, bool prepare, cudaStream_t st) {
  auto k = hv_batch_staged_kernel<NT, R, MINB>;
  if (prepare) SMGPU_CUDA_TRY(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  else k<<<ntasks, NT, smem, st>>>(probs, tasks, v, w, e);
}
void staged_case(int cand, const BatchProblemDev* probs, const int4* tasks, int ntasks, const float* v, double* w,
                 const BatchEpi& e, size_t smem, bool prepare, cudaStream_t st) {
  switch (cand) {
    case 8: launch_staged<64, 1, 8>(probs, tasks, ntasks, v, w, e, smem, prepare, st); break;
    case 9: launch_staged<128, 1, 4>(probs, tasks, ntasks, v, w, e, smem, prepare, st); break;
    case 10: launch_staged<128, 1, 5>(probs, tasks, ntasks, v, w, e, smem, prepare, st); break;
    default: launch_staged<128, 2, 3>(probs, tasks, ntasks, v, w, e, smem, prepare, st); break;
  }
}

}  // namespace

const BatchHvConfig* hv_batch_candidates(int* count) {
  *count = (int)(sizeof(kBatchCand) / sizeof(kBatchCand[0]));
  return kBatchCand;
}

int hv_batch_staged_cols(const BatchHvConfig& c) { return c.nt * kBatchQM; }

void hv_batch_prepare(int cand, size_t smem) {
  if (kBatchCand[cand].staged) staged_case(cand, nullptr, nullptr, 0, nullptr, nullptr, BatchEpi{}, smem, true, nullptr);
}

void launch_hv_batch(int cand, const BatchProblemDev* probs, const int4* tasks, int ntasks, const float* v, double* w,
                     const BatchEpi& e, size_t smem, cudaStream_t st) {
  if (ntasks <= 0) return;
  switch (cand) {
    case 0: launch_one<32, 4, 1>(probs, tasks, ntasks, v, w, e, st); break;
    case 1: launch_one<64, 2, 1>(probs, tasks, ntasks, v, w, e, st); break;
    case 2: launch_one<64, 4, 1>(probs, tasks, ntasks, v, w, e, st); break;
    case 3: launch_one<128, 1, 1>(probs, tasks, ntasks, v, w, e, st); break;
    case 4: launch_one<128, 2, 1>(probs, tasks, ntasks, v, w, e, st); break;
    case 5: launch_one<128, 4, 1>(probs, tasks, ntasks, v, w, e, st); break;
    case 6: launch_one<128, 2, 6>(probs, tasks, ntasks, v, w, e, st); break;
    case 7: launch_one<256, 2, 1>(probs, tasks, ntasks, v, w, e, st); break;
    default: staged_case(cand, probs, tasks, ntasks, v, w, e, smem, false, st); break;
  }
}

}  // namespace smgpu
