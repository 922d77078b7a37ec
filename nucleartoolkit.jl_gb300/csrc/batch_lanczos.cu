// Batched thick-restart Lanczos kernels (batch.cuh).  Per problem the
// algorithm and the kernel sequence are those of lanczos.cu — TRL
// (src/ShellModel/lanczos_methods.jl:1-91), diagonalize_T! (:250-258),
// ThickRestart (:260-307), ReORTH (shellmodel_main.jl:1005-1012) — for a
// whole batch of independent problems per launch:
//   * streaming kernels run one CTA per chunk of the concatenated vectors
//     (a chunk lies inside one problem) and write per-chunk partial sums;
//     every consumer sums the partials of its own problem in a fixed order,
//     so all CTAs of a problem agree bit for bit, as in lanczos.cu;
//   * small kernels (eigenvalue test, Jacobi, restart matrices, Cholesky)
//     run one CTA per problem.
// FP32 Krylov vectors, FP64 dot products, recurrences and small
// eigenproblems; FP32 Kahan sums for the restart rotation (the mixed form of
// lanczos.cu).
#include <algorithm>

#include "batch.cuh"
#include "hv_staged.cuh"
#include "hv_tile.cuh"
#include "lanczos_dev.cuh"

namespace smgpu {

namespace {
using namespace dev;

__device__ __forceinline__ void problem_finished(BatchCtl* ctl, int nprob) {
  if (atomicAdd(&ctl->ndone, 1) == nprob - 1) atomicExch(&ctl->all_done, 1);
}

// m sums out[j] = Σ_{q<n} p[j*stride + q], one warp per sum, into smem.
template <int NT>
__device__ __forceinline__ void sum_many_strided(const double* __restrict__ p, int64_t stride, int n, int m,
                                                 double* out) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  for (int j = wid; j < m; j += NT / 32) {
    double x = 0.0;
    for (int q = lane; q < n; q += 32) x += p[(int64_t)j * stride + q];
    x = warp_sum(x);
    if (lane == 0) out[j] = x;
  }
  __syncthreads();
}

// ------------------------------------------------------------------ vectors
__global__ void __launch_bounds__(kNT) k_b_start(const BatchDev B, uint64_t seed, double* __restrict__ w) {
  const int4 ch = B.chunks[blockIdx.x];
  const BatchProblemDev& P = B.probs[ch.x];
  const DevTables& t = P.a.t;
  for (int64_t i = ch.y + threadIdx.x; i < ch.z; i += kNT) {
    const int b = find_block(t.off_pad, t.nb, i);
    const int64_t loc = i - t.off_pad[b];
    const int st = t.stride[b];
    const int p = (int)(loc / st), n = (int)(loc % st);
    w[P.voff + i] = (n < t.nn[b]) ? start_elem(seed, t.tdims[b] + (int64_t)p * t.nn[b] + n) : 0.0;
  }
}

__global__ void __launch_bounds__(kNT) k_b_to_padded(const BatchDev B, const double* __restrict__ src,
                                                     double* __restrict__ w) {
  const int4 ch = B.chunks[blockIdx.x];
  const BatchProblemDev& P = B.probs[ch.x];
  const DevTables& t = P.a.t;
  for (int64_t i = ch.y + threadIdx.x; i < ch.z; i += kNT) {
    const int b = find_block(t.off_pad, t.nb, i);
    const int64_t loc = i - t.off_pad[b];
    const int st = t.stride[b];
    const int p = (int)(loc / st), n = (int)(loc % st);
    w[P.voff + i] = (n < t.nn[b]) ? src[P.moff + t.tdims[b] + (int64_t)p * t.nn[b] + n] : 0.0;
  }
}

__global__ void __launch_bounds__(kNT) k_b_from_padded(const BatchDev B, const double* __restrict__ w,
                                                       double* __restrict__ dst) {
  const int4 ch = B.chunks[blockIdx.x];
  const BatchProblemDev& P = B.probs[ch.x];
  const DevTables& t = P.a.t;
  for (int64_t i = ch.y + threadIdx.x; i < ch.z; i += kNT) {
    const int b = find_block(t.off_pad, t.nb, i);
    const int64_t loc = i - t.off_pad[b];
    const int st = t.stride[b];
    const int p = (int)(loc / st), n = (int)(loc % st);
    if (n < t.nn[b]) dst[P.moff + t.tdims[b] + (int64_t)p * t.nn[b] + n] = w[P.voff + i];
  }
}

__global__ void __launch_bounds__(kNT) k_b_convert(const double* __restrict__ w, float* __restrict__ v, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)kNT + threadIdx.x; i < n; i += (int64_t)gridDim.x * kNT) v[i] = (float)w[i];
}

// pn1[c] = ||w chunk||²
__global__ void __launch_bounds__(kNT) k_b_selfdot(const BatchDev B, const double* __restrict__ w) {
  __shared__ double red[kNT / 32];
  const int4 ch = B.chunks[blockIdx.x];
  const double* wb = w + B.probs[ch.x].voff;
  double x = 0.0;
  for (int64_t i = ch.y + threadIdx.x; i < ch.z; i += kNT) x = fma(wb[i], wb[i], x);
  x = block_sum_all<kNT>(x, red);
  if (threadIdx.x == 0) B.pn1[blockIdx.x] = x;
}

__global__ void __launch_bounds__(kNT) k_b_init_scale(const BatchDev B, const double* __restrict__ w,
                                                      float* __restrict__ v) {
  __shared__ double red[kNT / 32];
  const int4 ch = B.chunks[blockIdx.x];
  const BatchProblemDev& P = B.probs[ch.x];
  const double inv = 1.0 / sqrt(sum_partials_d2<kNT>(B.pn1 + P.chunk0, P.nchunks, red));
  for (int64_t i = ch.y + threadIdx.x; i < ch.z; i += kNT) v[P.voff + i] = (float)(w[P.voff + i] * inv);
}

// ------------------------------------------------------------ one iteration
// α (from the H·v partials of the problem), w' = w − α v_k, partials of
// v_j·w' (j <= it0) and of ||w'||² (slot it0+1).
template <int NT>
__device__ void b_orth_dot_body(const BatchDev& B, const int c, const float* __restrict__ V, double* w, int it0) {
  const int4 ch = B.chunks[c];
  if (cta_gate(threadIdx.x == 0 && (B.ctl->all_done || stopped(B.fl + ch.x)))) return;
  const BatchProblemDev& P = B.probs[ch.x];
  __shared__ double red[NT / 32];
  __shared__ double red8[(NT / 32) * 8];
  const double alpha = sum_partials_d2<NT>(B.alpha_part + (int64_t)it0 * B.nslots + P.slot0, P.nslots, red);
  const float* __restrict__ Vb = V + P.voff;
  const float* __restrict__ vk = Vb + (int64_t)it0 * B.LEN;
  double* wb = w + P.voff;
  const int m = it0 + 1;
  // w' = w - α v_k in FP64 once per element, split into an FP32 pair (kept
  // in wsplit for the later column blocks); the dots accumulate exact FP32
  // products in double-float on the FP32 pipe.
  float* __restrict__ wh = B.wsplit + P.voff;
  float* __restrict__ wl = B.wsplit + B.LEN + P.voff;
  // FP32 per-thread sums of the projections (a thread adds a handful of
  // products of one chunk; their rounding is far below the FP32 basis), the
  // CTA sums in double-float
  for (int j0 = 0; j0 <= m; j0 += 8) {
    float acc[8];
#pragma unroll
    for (int q = 0; q < 8; ++q) acc[q] = 0.f;
    #pragma unroll(NT <= 64 ? 2 : 1)  // 64-thread CTAs (persistent cycle): two trips' loads in flight
    for (int64_t i = ch.y + 4 * threadIdx.x; i < ch.z; i += 4 * NT) {
      float h[4], l[4];
      if (j0 == 0) {
        double wv[4], x[4];
        load4(wb + i, wv);
        load4(vk + i, x);
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          wv[u] = fma(-alpha, x[u], wv[u]);
          df_split(wv[u], h[u], l[u]);
        }
        store4(wb + i, wv);
        *reinterpret_cast<float4*>(wh + i) = make_float4(h[0], h[1], h[2], h[3]);
        *reinterpret_cast<float4*>(wl + i) = make_float4(l[0], l[1], l[2], l[3]);
      } else {
        const float4 a = *reinterpret_cast<const float4*>(wh + i);
        const float4 b = *reinterpret_cast<const float4*>(wl + i);
        h[0] = a.x; h[1] = a.y; h[2] = a.z; h[3] = a.w;
        l[0] = b.x; l[1] = b.y; l[2] = b.z; l[3] = b.w;
      }
#pragma unroll
      for (int q = 0; q < 8; ++q) {
        const int j = j0 + q;
        if (j < m) {
          const float4 x = *reinterpret_cast<const float4*>(Vb + (int64_t)j * B.LEN + i);
          acc[q] = __fmaf_rn(x.w, h[3], __fmaf_rn(x.z, h[2], __fmaf_rn(x.y, h[1], __fmaf_rn(x.x, h[0], acc[q]))));
        } else if (j == m) {
          acc[q] = __fmaf_rn(h[3], h[3], __fmaf_rn(h[2], h[2], __fmaf_rn(h[1], h[1], __fmaf_rn(h[0], h[0], acc[q]))));
        }
      }
    }
    // the eight sums in one double-float CTA reduction on the FP32 pipe
    DFAcc dacc[8];
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      dacc[q].hi = acc[q];
      dacc[q].lo = 0.f;
    }
    float2 s;
    block_sum_df<NT, 8>(dacc, red8, s);
    if (threadIdx.x < 8 && j0 + (int)threadIdx.x <= m)
      B.pdot[(int64_t)(j0 + threadIdx.x) * B.nchunks + c] = (double)s.x + (double)s.y;
  }
}

// Second-pass decision of the problem, identical in all its CTAs.
template <int NT>
__device__ __forceinline__ bool b_need_second(const BatchDev& B, const BatchProblemDev& P, int m, double* red) {
  const double n0 = sum_partials_d2<NT>(B.pdot + (int64_t)m * B.nchunks + P.chunk0, P.nchunks, red);
  const double n1 = sum_partials_d2<NT>(B.pn1 + P.chunk0, P.nchunks, red);
  return n1 < 0.5 * n0;
}

// w -= Σ_j h_j V_j over the chunk; pout[c] = ||w chunk||².
// (sum_h: form h_j = Σ ph[j][chunks of P] into hs first; else hs holds them)
template <int NT>
__device__ __forceinline__ void b_subtract(const BatchDev& B, const BatchProblemDev& P, const int c, const int4 ch,
                                           const float* __restrict__ V, double* w, int m,
                                           const double* __restrict__ ph, double* __restrict__ pout, double* hs,
                                           double* red, bool sum_h = true) {
  if (sum_h) sum_many_strided<NT>(ph + P.chunk0, B.nchunks, P.nchunks, m, hs);
  const float* __restrict__ Vb = V + P.voff;
  double* wb = w + P.voff;
  double nrm = 0.0;
  // Σ_j h_j V_j in double-float (h_j split once per CTA), one FP64
  // subtraction per element
  float* hh = reinterpret_cast<float*>(hs + m);
  float* hl = hh + m;
  for (int j = threadIdx.x; j < m; j += NT) df_split(hs[j], hh[j], hl[j]);
  __syncthreads();
  for (int64_t i = ch.y + 4 * threadIdx.x; i < ch.z; i += 4 * NT) {
    DFAcc s4[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) s4[u].init();
#pragma unroll(NT <= 64 ? 4 : 1)
    for (int j = 0; j < m; ++j) {
      const float4 x = *reinterpret_cast<const float4*>(Vb + (int64_t)j * B.LEN + i);
      const float a = hh[j], b = hl[j];
      s4[0].add_prod2(x.x, a, b);
      s4[1].add_prod2(x.y, a, b);
      s4[2].add_prod2(x.z, a, b);
      s4[3].add_prod2(x.w, a, b);
    }
    double t[4];
    load4(wb + i, t);
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      t[u] -= s4[u].get();
      nrm = fma(t[u], t[u], nrm);
    }
    store4(wb + i, t);
  }
  const double s = block_sum_d2<NT>(nrm, red);
  if (threadIdx.x == 0) pout[c] = s;
}

// The fast form of the first subtraction (h_j in hs): v_next = (w' -
// Σ_j h_j V_j) * inv over the chunk; the residual itself is not stored
// (the next H·v overwrites it).
template <int NT>
__device__ __forceinline__ void b_subtract_scale(const BatchDev& B, const BatchProblemDev& P, const int4 ch,
                                                 const float* __restrict__ V, const double* w, int m, double* hs,
                                                 const double inv, float* __restrict__ vn) {
  const float* __restrict__ Vb = V + P.voff;
  const double* wb = w + P.voff;
  float* hh = reinterpret_cast<float*>(hs + m);
  float* hl = hh + m;
  for (int j = threadIdx.x; j < m; j += NT) df_split(hs[j], hh[j], hl[j]);
  __syncthreads();
  for (int64_t i = ch.y + 4 * threadIdx.x; i < ch.z; i += 4 * NT) {
    DFAcc s4[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) s4[u].init();
#pragma unroll(NT <= 64 ? 4 : 1)
    for (int j = 0; j < m; ++j) {
      const float4 x = *reinterpret_cast<const float4*>(Vb + (int64_t)j * B.LEN + i);
      const float a = hh[j], b = hl[j];
      s4[0].add_prod2(x.x, a, b);
      s4[1].add_prod2(x.y, a, b);
      s4[2].add_prod2(x.z, a, b);
      s4[3].add_prod2(x.w, a, b);
    }
    double t[4];
    load4(wb + i, t);
    *reinterpret_cast<float4*>(vn + i) =
        make_float4((float)((t[0] - s4[0].get()) * inv), (float)((t[1] - s4[1].get()) * inv),
                    (float)((t[2] - s4[2].get()) * inv), (float)((t[3] - s4[3].get()) * inv));
  }
}

// β from the norm before the subtraction (B.fastnorm, normally kFastNorm, lanczos.cuh).
// w' -= Σ_j h_j V_j over the chunk (first pass).  Every CTA of the problem
// takes the same fast/slow decision from the same partial sums; the
// problem's first chunk records it (fastnorm) with β or exhaustion.
template <int NT>
__device__ void b_orth_axpy_body(const BatchDev& B, const int c, float* V, double* w, int it0) {
  const int4 ch = B.chunks[c];
  LanczosFlags* f = B.fl + ch.x;
  if (cta_gate(threadIdx.x == 0 && (B.ctl->all_done || stopped(f)))) return;
  extern __shared__ double hs[];
  __shared__ double red[NT / 32];
  const BatchProblemDev& P = B.probs[ch.x];
  const int m = it0 + 1;
  const double n0 = sum_partials_d2<NT>(B.pdot + (int64_t)m * B.nchunks + P.chunk0, P.nchunks, red);
  sum_many_strided<NT>(B.pdot + P.chunk0, B.nchunks, P.nchunks, m, hs);
  double hsq = 0.0;
  for (int j = 0; j < m; ++j) hsq = fma(hs[j], hs[j], hsq);
  const bool fast = n0 > 0.0 && hsq <= B.fastnorm * n0;
  if (!fast) {
    if (c == P.chunk0 && threadIdx.x == 0) f->fastnorm = 0;
    b_subtract<NT>(B, P, c, ch, V, w, m, B.pdot, B.pn1, hs, red, false);
    return;
  }
  const double beta = sqrt(n0 - hsq);
  const bool ok = beta < INFINITY;
  if (c == P.chunk0 && threadIdx.x == 0) {
    f->fastnorm = 1;
    double* T = B.T + (int64_t)ch.x * B.lm * B.lm;
    if (ok) {
      T[(int64_t)it0 * B.lm + it0 + 1] = beta;
      T[(int64_t)(it0 + 1) * B.lm + it0] = beta;
      f->second = 0;
    } else {
      f->exh_k = it0 + 1;
      f->exhausted = 1;
    }
  }
  if (!ok) return;
  b_subtract_scale<NT>(B, P, ch, V, w, m, hs, 1.0 / beta, V + (int64_t)(it0 + 1) * B.LEN + P.voff);
}

template <int NT>
__device__ void b_orth_dot2_body(const BatchDev& B, const int c, const float* __restrict__ V,
                                 const double* __restrict__ w, int it0) {
  const int4 ch = B.chunks[c];
  if (cta_gate(threadIdx.x == 0 && (B.ctl->all_done || stopped(B.fl + ch.x)))) return;
  if (cta_gate(threadIdx.x == 0 && *(volatile const int*)&B.fl[ch.x].fastnorm)) return;  // β already taken
  const BatchProblemDev& P = B.probs[ch.x];
  __shared__ double red[NT / 32];
  __shared__ double red8[(NT / 32) * 8];
  const int m = it0 + 1;
  if (!b_need_second<NT>(B, P, m, red)) return;
  const float* __restrict__ Vb = V + P.voff;
  const double* wb = w + P.voff;
  for (int j0 = 0; j0 < m; j0 += 8) {
    double acc[8];
#pragma unroll
    for (int q = 0; q < 8; ++q) acc[q] = 0.0;
    #pragma unroll(NT <= 64 ? 2 : 1)  // 64-thread CTAs (persistent cycle): two trips' loads in flight
    for (int64_t i = ch.y + 4 * threadIdx.x; i < ch.z; i += 4 * NT) {
      double wv[4];
      load4(wb + i, wv);
#pragma unroll
      for (int q = 0; q < 8; ++q)
        if (j0 + q < m) {
          double x[4];
          load4(Vb + (int64_t)(j0 + q) * B.LEN + i, x);
#pragma unroll
          for (int u = 0; u < 4; ++u) acc[q] = fma(x[u], wv[u], acc[q]);
        }
    }
    const double s = block_sum8<NT>(acc, red8);
    if (threadIdx.x < 8 && j0 + (int)threadIdx.x < m) B.pdot2[(int64_t)(j0 + threadIdx.x) * B.nchunks + c] = s;
  }
}

template <int NT>
__device__ void b_orth_axpy2_body(const BatchDev& B, const int c, const float* __restrict__ V, double* w, int it0) {
  const int4 ch = B.chunks[c];
  if (cta_gate(threadIdx.x == 0 && (B.ctl->all_done || stopped(B.fl + ch.x)))) return;
  if (cta_gate(threadIdx.x == 0 && *(volatile const int*)&B.fl[ch.x].fastnorm)) return;  // β already taken
  const BatchProblemDev& P = B.probs[ch.x];
  extern __shared__ double hs[];
  __shared__ double red[NT / 32];
  const int m = it0 + 1;
  if (!b_need_second<NT>(B, P, m, red)) return;
  b_subtract<NT>(B, P, c, ch, V, w, m, B.pdot2, B.pn2, hs, red);
}

// β = ||w||, T entries (by the problem's first CTA), v_{it0+1} = w/β.
template <int NT>
__device__ void b_orth_scale_body(const BatchDev& B, const int c, float* V, const double* __restrict__ w, int it0) {
  const int4 ch = B.chunks[c];
  LanczosFlags* f = B.fl + ch.x;
  if (cta_gate(threadIdx.x == 0 && (B.ctl->all_done || stopped(f) || *(volatile const int*)&f->fastnorm))) return;
  const BatchProblemDev& P = B.probs[ch.x];
  __shared__ double red[NT / 32];
  const int m = it0 + 1;
  const bool second = b_need_second<NT>(B, P, m, red);
  const double nrm = sum_partials_d2<NT>((second ? B.pn2 : B.pn1) + P.chunk0, P.nchunks, red);
  const double beta = sqrt(nrm);
  const bool ok = (beta > 0.0) && (beta < INFINITY);
  if (c == P.chunk0 && threadIdx.x == 0) {
    double* T = B.T + (int64_t)ch.x * B.lm * B.lm;
    if (ok) {
      T[(int64_t)it0 * B.lm + it0 + 1] = beta;
      T[(int64_t)(it0 + 1) * B.lm + it0] = beta;
      f->second = second ? 1 : 0;
      if (second) f->n_second += 1;
    } else {
      f->exh_k = it0 + 1;
      f->exhausted = 1;
    }
  }
  if (!ok) return;
  const double inv = 1.0 / beta;
  float* vn = V + (int64_t)(it0 + 1) * B.LEN + P.voff;
  const double* wb = w + P.voff;
  // four elements per thread and trip (chunk bounds are multiples of 4)
  #pragma unroll(NT <= 64 ? 4 : 1)
  for (int64_t i = ch.y + 4 * threadIdx.x; i < ch.z; i += 4 * NT) {
    double t[4];
    load4(wb + i, t);
    *reinterpret_cast<float4*>(vn + i) =
        make_float4((float)(t[0] * inv), (float)(t[1] * inv), (float)(t[2] * inv), (float)(t[3] * inv));
  }
}

// The chunk kernels of one iteration: one CTA per chunk.
__global__ void __launch_bounds__(kNT) k_b_orth_dot(const BatchDev B, const float* __restrict__ V, double* w, int it0) {
  b_orth_dot_body<kNT>(B, blockIdx.x, V, w, it0);
}
__global__ void __launch_bounds__(kNT) k_b_orth_axpy(const BatchDev B, float* V, double* w, int it0) {
  b_orth_axpy_body<kNT>(B, blockIdx.x, V, w, it0);
}
__global__ void __launch_bounds__(kNT) k_b_orth_dot2(const BatchDev B, const float* __restrict__ V,
                                                     const double* __restrict__ w, int it0) {
  b_orth_dot2_body<kNT>(B, blockIdx.x, V, w, it0);
}
__global__ void __launch_bounds__(kNT) k_b_orth_axpy2(const BatchDev B, const float* __restrict__ V, double* w,
                                                      int it0) {
  b_orth_axpy2_body<kNT>(B, blockIdx.x, V, w, it0);
}
__global__ void __launch_bounds__(kNT) k_b_orth_scale(const BatchDev B, float* V, const double* __restrict__ w,
                                                      int it0) {
  b_orth_scale_body<kNT>(B, blockIdx.x, V, w, it0);
}

// Eigenvalue test of every problem (one CTA each): α from the H·v partials,
// then sturm_step.
__device__ void b_sturm_body(const BatchDev& B, const int p, int k, int lock) {
  LanczosFlags* f = B.fl + p;
  // flags through L2 (in the persistent kernel other CTAs set them)
  volatile const LanczosFlags* vf = f;
  if (cta_gate(threadIdx.x == 0 && vf->done)) return;
  if (cta_gate(threadIdx.x == 0 && vf->exhausted && k > vf->exh_k)) {
    if (threadIdx.x == 0) {
      f->done = 1;
      f->elit = f->exh_k;
      problem_finished(B.ctl, B.nprob);
    }
    return;
  }
  const BatchProblemDev& P = B.probs[p];
  double* T = B.T + (int64_t)p * B.lm * B.lm;
  __shared__ double red[32];
  {
    double x = 0.0;
    const double* ap = B.alpha_part + (int64_t)(k - 1) * B.nslots + P.slot0;
    for (int i = threadIdx.x; i < P.nslots; i += blockDim.x) x += ap[i];
    x = warp_sum(x);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = x;
    __syncthreads();
    if (threadIdx.x == 0) {
      double s = 0.0;
      for (int wdx = 0; wdx < (int)(blockDim.x >> 5); ++wdx) s += red[wdx];
      T[(int64_t)(k - 1) * B.lm + (k - 1)] = s;
    }
    __syncthreads();
  }
  sturm_step(T, B.lm, k, lock, B.num_ev, B.en + (int64_t)p * B.nh * B.num_ev, B.nh, B.tol, P.mdim, f);
  if (threadIdx.x == 0 && f->done) problem_finished(B.ctl, B.nprob);
}
__global__ void k_b_sturm(const BatchDev B, int k, int lock) { b_sturm_body(B, blockIdx.x, k, lock); }

__global__ void k_b_cycle_end(const BatchDev B) {
  for (int p = threadIdx.x; p < B.nprob; p += blockDim.x) {
    LanczosFlags* f = B.fl + p;
    if (!f->done && f->exhausted) {
      f->done = 1;
      f->elit = f->exh_k;
      atomicAdd(&B.ctl->ndone, 1);
    }
  }
  __syncthreads();
  if (threadIdx.x == 0 && atomicAdd(&B.ctl->ndone, 0) >= B.nprob) B.ctl->all_done = 1;
}

// ------------------------------------------------------------------ restart
__global__ void __launch_bounds__(256) k_b_jacobi(const BatchDev B, int n, int gate) {
  const int p = blockIdx.x;
  if (gate && (B.ctl->all_done || stopped(B.fl + p))) return;
  const int64_t o = (int64_t)p * B.lm * B.lm;
  if (n <= kJacobiSmemN) jacobi_eig_df<256>(B.T + o, B.lm, n, B.jacA + o, B.evals + (int64_t)p * B.lm);
  else jacobi_eig<256>(B.T + o, B.lm, n, B.jacA + o, B.jacZ + o, B.evals + (int64_t)p * B.lm);
}

// Jacobi of one problem for its Ritz vectors (grid of one CTA).
__global__ void __launch_bounds__(256) k_b_jacobi_one(const BatchDev B, int p, int n) {
  const int64_t o = (int64_t)p * B.lm * B.lm;
  if (n <= kJacobiSmemN) jacobi_eig_df<256>(B.T + o, B.lm, n, B.jacA + o, B.evals + (int64_t)p * B.lm);
  else jacobi_eig<256>(B.T + o, B.lm, n, B.jacA + o, B.jacZ + o, B.evals + (int64_t)p * B.lm);
}

__global__ void k_b_restart_small(const BatchDev B) {
  const int p = blockIdx.x;
  if (B.ctl->all_done || stopped(B.fl + p)) return;
  const int lm = B.lm, ls = B.ls, m = lm - 1;
  double* T = B.T + (int64_t)p * lm * lm;
  const double* ev = B.evals + (int64_t)p * lm;
  const double* vs = B.jacA + (int64_t)p * lm * lm;
  float* yf = B.Yf + (int64_t)p * m * ls;
  for (int idx = threadIdx.x; idx < m * ls; idx += blockDim.x) yf[idx] = (float)vs[idx];
  __shared__ double beta;
  if (threadIdx.x == 0) beta = T[(int64_t)(lm - 1) * lm + (lm - 2)];
  __syncthreads();
  for (int idx = threadIdx.x; idx < lm * lm; idx += blockDim.x) T[idx] = 0.0;
  __syncthreads();
  for (int k = threadIdx.x; k < ls; k += blockDim.x) {
    T[(int64_t)k * lm + k] = ev[k];
    const double tmp = beta * vs[(int64_t)k * m + (m - 1)];
    T[(int64_t)k * lm + ls] = tmp;
    T[(int64_t)ls * lm + k] = tmp;
  }
}

// U_k = Σ_{j<m} Y[j,k] V_j over the chunk (FP32 products, Kahan sums).
__global__ void __launch_bounds__(kNT) k_b_rotate(const BatchDev B, const float* __restrict__ V,
                                                  float* __restrict__ U) {
  const int4 ch = B.chunks[blockIdx.x];
  if (cta_gate(threadIdx.x == 0 && (B.ctl->all_done || stopped(B.fl + ch.x)))) return;
  const BatchProblemDev& P = B.probs[ch.x];
  const int m = B.lm - 1, ls = B.ls;
  const float* __restrict__ Y = B.Yf + (int64_t)ch.x * m * ls;
  const float* __restrict__ Vb = V + P.voff;
  float* __restrict__ Ub = U + P.voff;
  for (int64_t i = ch.y + threadIdx.x; i < ch.z; i += kNT) {
    for (int k0 = 0; k0 < ls; k0 += 8) {
      KahanF acc[8];
#pragma unroll
      for (int q = 0; q < 8; ++q) acc[q].init();
      for (int j = 0; j < m; ++j) {
        const float x = Vb[(int64_t)j * B.LEN + i];
#pragma unroll
        for (int q = 0; q < 8; ++q)
          if (k0 + q < ls) acc[q].add(__fmul_rn(__ldg(Y + (int64_t)(k0 + q) * m + j), x));
      }
#pragma unroll
      for (int q = 0; q < 8; ++q)
        if (k0 + q < ls) Ub[(int64_t)(k0 + q) * B.LEN + i] = acc[q].get();
    }
  }
}

// The rotation with the basis read once: all ls <= 16 outputs of a thread's
// element in registers, the problem's Y in shared memory (rows padded to 16),
// groups of four terms summed with FMAs and the group sums compensated.
constexpr int kBRLS = 16;
__global__ void __launch_bounds__(kNT) k_b_rotate_r(const BatchDev B, const float* __restrict__ V,
                                                    float* __restrict__ U) {
  const int4 ch = B.chunks[blockIdx.x];
  if (cta_gate(threadIdx.x == 0 && (B.ctl->all_done || stopped(B.fl + ch.x)))) return;
  const BatchProblemDev& P = B.probs[ch.x];
  const int m = B.lm - 1, ls = B.ls;
  extern __shared__ float ys[];  // m x kBRLS
  const float* __restrict__ Y = B.Yf + (int64_t)ch.x * m * ls;
  for (int idx = threadIdx.x; idx < m * kBRLS; idx += kNT) {
    const int j = idx / kBRLS, k = idx % kBRLS;
    ys[idx] = k < ls ? Y[(int64_t)k * m + j] : 0.f;
  }
  __syncthreads();
  const float* __restrict__ Vb = V + P.voff;
  float* __restrict__ Ub = U + P.voff;
  for (int64_t i = ch.y + threadIdx.x; i < ch.z; i += kNT) {
    KahanF acc[kBRLS];
#pragma unroll
    for (int k = 0; k < kBRLS; ++k) acc[k].init();
    int j = 0;
    for (; j + 4 <= m; j += 4) {
      float x[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) x[u] = Vb[(int64_t)(j + u) * B.LEN + i];
      const float4* y0 = reinterpret_cast<const float4*>(ys + (j + 0) * kBRLS);
      const float4* y1 = reinterpret_cast<const float4*>(ys + (j + 1) * kBRLS);
      const float4* y2 = reinterpret_cast<const float4*>(ys + (j + 2) * kBRLS);
      const float4* y3 = reinterpret_cast<const float4*>(ys + (j + 3) * kBRLS);
#pragma unroll
      for (int q = 0; q < kBRLS / 4; ++q) {
        const float4 a = y0[q], b = y1[q], c = y2[q], d = y3[q];
        acc[4 * q].add(__fmaf_rn(d.x, x[3], __fmaf_rn(c.x, x[2], __fmaf_rn(b.x, x[1], __fmul_rn(a.x, x[0])))));
        acc[4 * q + 1].add(__fmaf_rn(d.y, x[3], __fmaf_rn(c.y, x[2], __fmaf_rn(b.y, x[1], __fmul_rn(a.y, x[0])))));
        acc[4 * q + 2].add(__fmaf_rn(d.z, x[3], __fmaf_rn(c.z, x[2], __fmaf_rn(b.z, x[1], __fmul_rn(a.z, x[0])))));
        acc[4 * q + 3].add(__fmaf_rn(d.w, x[3], __fmaf_rn(c.w, x[2], __fmaf_rn(b.w, x[1], __fmul_rn(a.w, x[0])))));
      }
    }
    for (; j < m; ++j) {
      const float x = Vb[(int64_t)j * B.LEN + i];
      const float4* y4 = reinterpret_cast<const float4*>(ys + j * kBRLS);
#pragma unroll
      for (int q = 0; q < kBRLS / 4; ++q) {
        const float4 y = y4[q];
        acc[4 * q].add_prod(y.x, x);
        acc[4 * q + 1].add_prod(y.y, x);
        acc[4 * q + 2].add_prod(y.z, x);
        acc[4 * q + 3].add_prod(y.w, x);
      }
    }
#pragma unroll
    for (int k = 0; k < kBRLS; ++k)
      if (k < ls) Ub[(int64_t)k * B.LEN + i] = acc[k].get();
  }
}

// The apply with the problem's U values of a thread's element in registers.
__global__ void __launch_bounds__(kNT) k_b_apply_r(const BatchDev B, const float* __restrict__ U,
                                                   float* __restrict__ V) {
  const int4 ch = B.chunks[blockIdx.x];
  if (cta_gate(threadIdx.x == 0 && (B.ctl->all_done || stopped(B.fl + ch.x)))) return;
  const BatchProblemDev& P = B.probs[ch.x];
  const int ls = B.ls, lm = B.lm;
  __shared__ float xf[kBRLS * kBRLS + kBRLS];
  const float* __restrict__ xg = B.Xf + (int64_t)ch.x * (ls * ls + ls);
  for (int idx = threadIdx.x; idx < ls * ls + ls; idx += kNT) xf[idx] = xg[idx];
  __syncthreads();
  const float* __restrict__ Ub = U + P.voff;
  float* __restrict__ Vb = V + P.voff;
  for (int64_t i = ch.y + threadIdx.x; i < ch.z; i += kNT) {
    float u[kBRLS];
#pragma unroll
    for (int j = 0; j < kBRLS; ++j) u[j] = j < ls ? Ub[(int64_t)j * B.LEN + i] : 0.f;
    KahanF last;
    last.init();
    last.add(Vb[(int64_t)(lm - 1) * B.LEN + i]);
#pragma unroll
    for (int k = 0; k < kBRLS; ++k) {
      if (k >= ls) break;
      KahanF q;
      q.init();
#pragma unroll
      for (int j = 0; j <= k; ++j) q.add_prod(xf[k * ls + j], u[j]);
      const float qv = q.get();
      Vb[(int64_t)k * B.LEN + i] = qv;
      last.add_prod(-xf[ls * ls + k], qv);
    }
    Vb[(int64_t)ls * B.LEN + i] = last.get();
  }
}

// The Gram partials with one thread per pair (ls <= 16): tiles of 128
// elements with padded rows (no bank conflicts), double-buffered through
// registers, FP32 sums per tile added in double-float.
__global__ void __launch_bounds__(kNT) k_b_gram_r(const BatchDev B, const float* __restrict__ U,
                                                  const float* __restrict__ Vlast) {
  const int c = blockIdx.x;
  const int4 ch = B.chunks[c];
  if (cta_gate(threadIdx.x == 0 && (B.ctl->all_done || stopped(B.fl + ch.x)))) return;
  const BatchProblemDev& P = B.probs[ch.x];
  constexpr int TILE = 128, TS = TILE + 1;
  constexpr int LD = ((kBRLS + 1) * TILE + kNT - 1) / kNT;
  extern __shared__ float gt[];  // 2 x (ls+1) x TS
  const int ls = B.ls, nv = ls + 1;
  const int NP = ls * (ls + 1) / 2 + ls;
  const float* __restrict__ Ub = U + P.voff;
  const float* __restrict__ vl = Vlast + P.voff;
  const bool act = (int)threadIdx.x < NP;
  int k = 0, l = 0;
  if (act) gram_pair(threadIdx.x, ls, k, l);
  DFAcc acc;
  acc.init();
  float st[LD];
  auto load = [&](int64_t t0) {
#pragma unroll
    for (int u = 0; u < LD; ++u) {
      const int idx = threadIdx.x + u * kNT;
      const int j = idx / TILE, x = idx % TILE;
      float val = 0.f;
      if (j < nv && t0 + x < ch.z) val = (j < ls) ? Ub[(int64_t)j * B.LEN + t0 + x] : vl[t0 + x];
      st[u] = val;
    }
  };
  auto store = [&](int buf) {
    float* tl = gt + buf * nv * TS;
#pragma unroll
    for (int u = 0; u < LD; ++u) {
      const int idx = threadIdx.x + u * kNT;
      const int j = idx / TILE, x = idx % TILE;
      if (j < nv) tl[j * TS + x] = st[u];
    }
  };
  int buf = 0;
  if (ch.y < ch.z) {
    load(ch.y);
    store(0);
  }
  __syncthreads();
  for (int64_t t0 = ch.y; t0 < ch.z; t0 += TILE) {
    const bool more = t0 + TILE < ch.z;
    if (more) load(t0 + TILE);
    const float* tl = gt + buf * nv * TS;
    if (act) {
      const int cnt = (int)min((int64_t)TILE, ch.z - t0);
      float p0 = 0.f, p1 = 0.f;
      int x = 0;
      for (; x + 1 < cnt; x += 2) {
        p0 = __fmaf_rn(tl[k * TS + x], tl[l * TS + x], p0);
        p1 = __fmaf_rn(tl[k * TS + x + 1], tl[l * TS + x + 1], p1);
      }
      if (x < cnt) p0 = __fmaf_rn(tl[k * TS + x], tl[l * TS + x], p0);
      df_add(acc.hi, acc.lo, __fadd_rn(p0, p1), 0.f);
    }
    if (more) store(buf ^ 1);
    __syncthreads();
    buf ^= 1;
  }
  if (act) B.part[(int64_t)threadIdx.x * B.nchunks + c] = acc.get();
}

// Each problem's Cholesky on one warp in double-float (chol_df_warp); the
// Gram entries summed over the problem's chunks first.
__global__ void __launch_bounds__(32) k_b_chol_df(const BatchDev B) {
  const int p = blockIdx.x;
  if (B.ctl->all_done || stopped(B.fl + p)) return;  // one warp: uniform
  const BatchProblemDev& P = B.probs[p];
  const int ls = B.ls;
  const int NP = ls * (ls + 1) / 2 + ls;
  __shared__ double g[32 * 33 / 2 + 32];
  for (int pr = threadIdx.x; pr < NP; pr += 32) {
    double x = 0.0;
    const double* src = B.part + (int64_t)pr * B.nchunks + P.chunk0;
    for (int q = 0; q < P.nchunks; ++q) x += src[q];
    g[pr] = x;
  }
  __syncwarp();
  double* X = B.X + (int64_t)p * ls * ls;
  double* cv = B.cvec + (int64_t)p * ls;
  float* xf = B.Xf + (int64_t)p * (ls * ls + ls);
  const bool bad = chol_df_warp(
      ls, [&](int idx) { return g[idx]; },
      [&](int j, int i, double x) {
        X[j * ls + i] = x;
        xf[j * ls + i] = (float)x;
      },
      [&](int k, double c) {
        cv[k] = c;
        xf[ls * ls + k] = (float)c;
      });
  if (threadIdx.x == 0 && bad) B.fl[p].bad = 1;
}

// Chunk partials of the Gram matrix of U and of U_k·v_last (pair order of
// k_gram), double-float sums: part[pair*nchunks + c].
__global__ void __launch_bounds__(kNT) k_b_gram(const BatchDev B, const float* __restrict__ U,
                                                const float* __restrict__ Vlast) {
  const int c = blockIdx.x;
  const int4 ch = B.chunks[c];
  if (cta_gate(threadIdx.x == 0 && (B.ctl->all_done || stopped(B.fl + ch.x)))) return;
  const BatchProblemDev& P = B.probs[ch.x];
  constexpr int TILE = 64;
  extern __shared__ float tl[];  // (ls+1) x TILE
  const int ls = B.ls;
  const int NP = ls * (ls + 1) / 2 + ls;
  const float* __restrict__ Ub = U + P.voff;
  const float* __restrict__ vl = Vlast + P.voff;
  for (int c0 = 0; c0 < NP; c0 += 8 * kNT) {
    DFAcc dacc[8];
    int kk[8], ll[8];
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      dacc[q].init();
      const int pr = c0 + threadIdx.x + q * kNT;
      kk[q] = 0;
      ll[q] = 0;
      if (pr < NP) gram_pair(pr, ls, kk[q], ll[q]);
    }
    for (int64_t t0 = ch.y; t0 < ch.z; t0 += TILE) {
      const int cnt = (int)min((int64_t)TILE, ch.z - t0);
      for (int idx = threadIdx.x; idx < (ls + 1) * TILE; idx += kNT) {
        const int j = idx / TILE, x = idx % TILE;
        float val = 0.f;
        if (x < cnt) val = (j < ls) ? Ub[(int64_t)j * B.LEN + t0 + x] : vl[t0 + x];
        tl[idx] = val;
      }
      __syncthreads();
#pragma unroll
      for (int q = 0; q < 8; ++q) {
        const int pr = c0 + threadIdx.x + q * kNT;
        if (pr >= NP) break;
        for (int x = 0; x < cnt; ++x) dacc[q].add_prod(tl[kk[q] * TILE + x], tl[ll[q] * TILE + x]);
      }
      __syncthreads();
    }
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      const int pr = c0 + threadIdx.x + q * kNT;
      if (pr < NP) B.part[(int64_t)pr * B.nchunks + c] = dacc[q].get();
    }
  }
}

// Per problem: Gram matrix from the chunk partials, Cholesky G = RᵀR,
// X = R⁻¹, c = Xᵀ g (as k_chol), FP32 copies for k_b_apply.
__global__ void k_b_chol(const BatchDev B) {
  const int p = blockIdx.x;
  if (B.ctl->all_done || stopped(B.fl + p)) return;
  const BatchProblemDev& P = B.probs[p];
  const int ls = B.ls;
  const int NP = ls * (ls + 1) / 2 + ls;
  extern __shared__ double sh[];
  double* g = sh;        // NP
  double* R = sh + NP;   // ls x ls
  for (int pr = threadIdx.x; pr < NP; pr += blockDim.x) {
    double x = 0.0;
    const double* src = B.part + (int64_t)pr * B.nchunks + P.chunk0;
    for (int q = 0; q < P.nchunks; ++q) x += src[q];
    g[pr] = x;
  }
  __syncthreads();
  if (threadIdx.x != 0) return;
  double* X = B.X + (int64_t)p * ls * ls;
  double* cv = B.cvec + (int64_t)p * ls;
  float* xf = B.Xf + (int64_t)p * (ls * ls + ls);
  auto Gm = [&](int k, int l) {  // k <= l
    int off = 0;
    for (int r = 0; r < k; ++r) off += ls - r;
    return g[off + (l - k)];
  };
  for (int j = 0; j < ls; ++j) {
    for (int i = 0; i <= j; ++i) {
      double t = Gm(i, j);
      for (int k = 0; k < i; ++k) t -= R[j * ls + k] * R[i * ls + k];
      if (i == j) {
        if (!(t > 0.0)) {
          B.fl[p].bad = 1;
          t = 1e-300;
        }
        R[j * ls + j] = sqrt(t);
      } else {
        R[j * ls + i] = t / R[i * ls + i];
      }
    }
  }
  for (int j = 0; j < ls; ++j) {
    for (int i = ls - 1; i >= 0; --i) {
      double t = (i == j) ? 1.0 : 0.0;
      for (int k = i + 1; k <= j; ++k) t -= R[k * ls + i] * X[j * ls + k];
      X[j * ls + i] = (i <= j) ? t / R[i * ls + i] : 0.0;
    }
  }
  const int gofs = ls * (ls + 1) / 2;
  for (int k = 0; k < ls; ++k) {
    double t = 0.0;
    for (int j = 0; j <= k; ++j) t += X[k * ls + j] * g[gofs + j];
    cv[k] = t;
  }
  for (int idx = 0; idx < ls * ls; ++idx) xf[idx] = (float)X[idx];
  for (int k = 0; k < ls; ++k) xf[ls * ls + k] = (float)cv[k];
}

// V_k = Σ_{j<=k} X[j,k] U_j (k < ls);  V_ls = V_{lm-1} − Σ_k c_k V_k.
__global__ void __launch_bounds__(kNT) k_b_apply(const BatchDev B, const float* __restrict__ U,
                                                 float* __restrict__ V) {
  const int4 ch = B.chunks[blockIdx.x];
  if (cta_gate(threadIdx.x == 0 && (B.ctl->all_done || stopped(B.fl + ch.x)))) return;
  const BatchProblemDev& P = B.probs[ch.x];
  const int ls = B.ls, lm = B.lm;
  const float* __restrict__ xf = B.Xf + (int64_t)ch.x * (ls * ls + ls);
  const float* __restrict__ Ub = U + P.voff;
  float* __restrict__ Vb = V + P.voff;
  for (int64_t i = ch.y + threadIdx.x; i < ch.z; i += kNT) {
    KahanF last;
    last.init();
    last.add(Vb[(int64_t)(lm - 1) * B.LEN + i]);
    for (int k = 0; k < ls; ++k) {
      KahanF q;
      q.init();
      for (int j = 0; j <= k; ++j) q.add(__fmul_rn(__ldg(xf + k * ls + j), Ub[(int64_t)j * B.LEN + i]));
      const float qv = q.get();
      Vb[(int64_t)k * B.LEN + i] = qv;
      last.add(__fmul_rn(-__ldg(xf + ls * ls + k), qv));
    }
    Vb[(int64_t)ls * B.LEN + i] = last.get();
  }
}

// R_e = Σ_{k<elit} Y[k,e] V_k of problem p (its chunks), FP64, padded.
__global__ void __launch_bounds__(kNT) k_b_ritz(const BatchDev B, const float* __restrict__ V, int p, int elit,
                                                int nev, double* __restrict__ R) {
  const BatchProblemDev& P = B.probs[p];
  const double* __restrict__ Y = B.jacA + (int64_t)p * B.lm * B.lm;
  const float* __restrict__ Vb = V + P.voff;
  for (int64_t i = blockIdx.x * (int64_t)kNT + threadIdx.x; i < P.len; i += (int64_t)gridDim.x * kNT) {
    for (int e = 0; e < nev; ++e) {
      double t = 0.0;
      for (int k = 0; k < elit; ++k) t = fma(Y[(int64_t)e * elit + k], (double)Vb[(int64_t)k * B.LEN + i], t);
      R[(int64_t)e * P.len + i] = t;
    }
  }
}

size_t jacobi_smem(int n) { return jacobi_smem_bytes(n); }

// ------------------------------------------------------- persistent cycle
// A gpu-scope load that sees the L2 value without acquire semantics: the
// barrier polls with it, so a waiting CTA does not invalidate the L1 cache
// its SM's other CTAs are still working from; one fence after the wait
// gives the acquire.
__device__ __forceinline__ int ld_relaxed_s32(const int* p) {
  int v;
  asm volatile("ld.relaxed.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ unsigned ld_relaxed_u32(const unsigned* p) {
  unsigned v;
  asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

// Grid barrier of the cooperative cycle kernel.  Thread 0 of each CTA
// arrives on its group's counter; the last arriver of a group resets that
// counter and arrives on the top counter; the last group to arrive resets
// the top counter and writes the next generation into every group's release
// word, which the group's CTAs poll.  (A thousand CTAs arriving on, and
// polling, one address serialise for tens of microseconds.)  Every wait is
// bounded: after C.spin_limit polls the CTA records sync_err and the kernel
// unwinds (every CTA leaves at its next barrier), so a lost CTA costs an
// error status, not a hang.  Returns false when the kernel is to stop.
__device__ __forceinline__ void st_relaxed_u32(unsigned* p, unsigned v) {
  asm volatile("st.relaxed.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ bool grid_sync(const BatchCycle& C, BatchCtl* ctl) {
  __shared__ int s_ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    int ok = 1;
    const unsigned grp = blockIdx.x / kSyncGroup;
    const unsigned ngroups = (gridDim.x + kSyncGroup - 1) / kSyncGroup;
    const unsigned in_grp = min((unsigned)kSyncGroup, gridDim.x - grp * kSyncGroup);
    // the group's release word cannot advance before this CTA arrives
    const unsigned g = ld_relaxed_u32(&C.gs->rel[grp][0]);
    __threadfence();
    bool last = false;
    if (atomicAdd(&C.gs->group[grp][0], 1u) == in_grp - 1) {
      __threadfence();  // the group's writes, seen through its counter, before the top arrival
      atomicExch(&C.gs->group[grp][0], 0u);
      last = atomicAdd(&C.gs->count, 1u) == ngroups - 1;
    }
    if (last) {
      __threadfence();
      atomicExch(&C.gs->count, 0u);
      __threadfence();
      for (unsigned q = 0; q < ngroups; ++q) st_relaxed_u32(&C.gs->rel[q][0], g + 1u);
    } else {
      long long polls = 0;
      while (ld_relaxed_u32(&C.gs->rel[grp][0]) == g) {
        if (++polls > C.spin_limit) {
          ok = 0;
          atomicExch(&ctl->sync_err, 1);
          break;
        }
        __nanosleep(32);
      }
    }
    __threadfence();
    if (*(volatile int*)&ctl->sync_err) ok = 0;
    s_ok = ok;
  }
  __syncthreads();
  return s_ok != 0;
}

// The eigenvalue tests of iteration k, problem p by CTA floor(p·nb/nprob):
// spread over the grid (the tests are FP64-heavy, and CTAs of adjacent
// indices may share an SM).
__device__ void b_sturm_spread(const BatchDev& B, int nb, int k, int lock) {
  const int c = blockIdx.x;
  const int pb = (int)(((long long)c * B.nprob + nb - 1) / nb), pe = (int)(((long long)(c + 1) * B.nprob + nb - 1) / nb);
  for (int p = pb; p < pe; ++p) b_sturm_body(B, p, k, lock);
}

// Which passes after the subtraction this iteration needs, the same in every
// CTA (it reads the flags and partials the subtraction pass completed):
// bit 0, some running problem took the slow form (its β still to come, in
// the scaling pass); bit 1, one of those may take the second Gram-Schmidt
// pass (b_need_second's test with a margin for the summation order; the
// chunk passes then decide per problem exactly).
template <int NT>
__device__ int passes_needed(const BatchDev& B, int m) {
  __shared__ int s_need;
  if (threadIdx.x == 0) s_need = 0;
  __syncthreads();
  for (int p = threadIdx.x; p < B.nprob; p += NT) {
    const LanczosFlags* f = B.fl + p;
    if (stopped(f) || *(volatile const int*)&f->fastnorm) continue;
    const BatchProblemDev& P = B.probs[p];
    double n0 = 0.0, n1 = 0.0;
    for (int q = 0; q < P.nchunks; ++q) {
      n0 += B.pdot[(int64_t)m * B.nchunks + P.chunk0 + q];
      n1 += B.pn1[P.chunk0 + q];
    }
    atomicOr(&s_need, (n1 < 0.5 * n0 * (1.0 + 1e-6)) ? 3 : 1);
  }
  __syncthreads();
  const int need = s_need;
  __syncthreads();
  return need;
}

// One H·v task (the body of hv_batch_staged_kernel / hv_batch_kernel).  Not
// inlined: compiled on its own, the row body gets the register allocation it
// has in those kernels (inlined into the cycle kernel it shares registers
// with the cycle's live state; measured 8 % slower over the batched solve).
template <int NT, int R, bool STAGED>
__device__ __noinline__ void b_hv_task(const BatchDev& B, const int4 tk, const float* v, double* w,
                                          const float* vprev_all, int it0, double* alpha_part) {
  if (cta_gate(threadIdx.x == 0 && (B.fl[tk.x].done || B.fl[tk.x].exhausted))) return;
  const BatchProblemDev& P = B.probs[tk.x];
  const int64_t off = P.voff;
  double beta = 0.0;
  const float* vprev = nullptr;
  if (vprev_all != nullptr) {
    vprev = vprev_all + off;
    beta = B.T[(int64_t)tk.x * B.lm * B.lm + (int64_t)(it0 - 1) * B.lm + it0];
  }
  if constexpr (STAGED)
    hv_staged_rows<NT, R, kBatchQM, false>(P.a, v + off, w + off, vprev, beta, tk.y, tk.z, alpha_part + tk.w);
  else
    hv_tile_rows<float, float, AccKahan, NT, R>(P.a, v + off, w + off, vprev, tk.y, tk.z, beta, alpha_part + tk.w);
}

// Registers capped as the H·v shapes of the graph form (64 threads: 8 CTAs
// per SM; 128 threads: 4).
template <int NT, int R, bool STAGED>
__global__ void __launch_bounds__(NT, 512 / NT) k_b_cycle(const BatchDev B, float* V, double* w, const BatchCycle C) {
  __shared__ int s_task, s_want;
  const int nb = gridDim.x;
  for (int it = C.kstart; it <= B.lm - 1; ++it) {
    const int it0 = it - 1;
    // phase A: the previous iteration's eigenvalue tests (one CTA per
    // problem), then the H·v row tasks from this iteration's queue
    if (it > C.kstart) b_sturm_spread(B, nb, it - 1, C.lock);
    if (blockIdx.x == 0 && threadIdx.x == 0 && !*(volatile int*)&B.ctl->all_done) atomicAdd(C.hv_count, 1);
    const float* vprev = (it0 > C.lock) ? V + (int64_t)(it0 - 1) * B.LEN : nullptr;
    double* ap = B.alpha_part + (int64_t)it0 * B.nslots;
    // tasks are taken kGrab at a time (one atomic per kGrab tasks keeps
    // the queue counter off the critical path) until the last two tasks per
    // CTA, then singly (a CTA holding kGrab of the last tasks would hold up
    // the end of the phase)
    constexpr int kGrab = 4;
    while (true) {
      __syncthreads();
      if (threadIdx.x == 0) {
        const int want = ld_relaxed_s32(C.task_ctr + it0) < C.ntasks - 2 * nb ? kGrab : 1;
        s_task = atomicAdd(C.task_ctr + it0, want);
        s_want = want;
      }
      __syncthreads();
      const int t0 = s_task;
      if (t0 >= C.ntasks) break;
      const int t1 = min(C.ntasks, t0 + s_want);
      for (int task = t0; task < t1; ++task)
        b_hv_task<NT, R, STAGED>(B, C.tasks[task], V + (int64_t)it0 * B.LEN, w, vprev, it0, ap);
    }
    if (!grid_sync(C, B.ctl)) return;
    if (*(volatile int*)&B.ctl->all_done) return;  // set only in phase A: the same for every CTA
    // the re-orthogonalisation passes, β and the next vector (chunk phases)
    for (int c = blockIdx.x; c < B.nchunks; c += nb) b_orth_dot_body<NT>(B, c, V, w, it0);
    if (!grid_sync(C, B.ctl)) return;
    for (int c = blockIdx.x; c < B.nchunks; c += nb) b_orth_axpy_body<NT>(B, c, V, w, it0);
    if (!grid_sync(C, B.ctl)) return;
    // the second pass and the scaling pass only when some running problem
    // needs them (the same decision in every CTA)
    const int need = passes_needed<NT>(B, it0 + 1);
    if (need & 2) {
      for (int c = blockIdx.x; c < B.nchunks; c += nb) b_orth_dot2_body<NT>(B, c, V, w, it0);
      if (!grid_sync(C, B.ctl)) return;
      for (int c = blockIdx.x; c < B.nchunks; c += nb) b_orth_axpy2_body<NT>(B, c, V, w, it0);
      if (!grid_sync(C, B.ctl)) return;
    }
    if (need & 1) {
      for (int c = blockIdx.x; c < B.nchunks; c += nb) b_orth_scale_body<NT>(B, c, V, w, it0);
      if (!grid_sync(C, B.ctl)) return;
    }
  }
  b_sturm_spread(B, nb, B.lm - 1, C.lock);
}

// cand (index into hv_batch_candidates) -> persistent instance
template <int NT, int R, bool STAGED>
struct PersistKernel {
  static void* fn() { return (void*)k_b_cycle<NT, R, STAGED>; }
};
void* persist_fn(int cand) {
  switch (cand) {
    case 3: return PersistKernel<128, 1, false>::fn();
    case 4: return PersistKernel<128, 2, false>::fn();
    case 6: return PersistKernel<128, 2, false>::fn();
    case 8: return PersistKernel<64, 1, true>::fn();
    case 9: return PersistKernel<128, 1, true>::fn();
    case 10: return PersistKernel<128, 1, true>::fn();
    default: return nullptr;
  }
}
int persist_nt(int cand) { return cand == 8 ? 64 : 128; }
size_t persist_smem(const BatchDev& B, size_t smem_hv) {
  size_t m = smem_hv;
  m = std::max(m, sizeof(double) * (3 * (size_t)B.lm + B.num_ev));  // eigenvalue test
  m = std::max(m, 2 * sizeof(double) * (size_t)(B.lm + 1));         // h_j and their splits
  return m;
}
}  // namespace

bool persist_supported(int cand) { return persist_fn(cand) != nullptr; }

int persist_grid(int cand, const BatchDev& B, size_t smem_hv) {
  void* f = persist_fn(cand);
  if (!f) return 0;
  const size_t smem = persist_smem(B, smem_hv);
  int dev = 0, sms = 0, coop = 0, per_sm = 0;
  SMGPU_CUDA_TRY(cudaGetDevice(&dev));
  SMGPU_CUDA_TRY(cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev));
  if (!coop) return 0;
  SMGPU_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  SMGPU_CUDA_TRY(cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  SMGPU_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, f, persist_nt(cand), smem));
  return std::min(per_sm * sms, kSyncGroup * kSyncMaxGroups);
}

void launch_b_persist_cycle(int cand, const BatchDev& B, float* V, double* w, const BatchCycle& C, size_t smem_hv,
                            int grid, cudaStream_t st) {
  void* f = persist_fn(cand);
  if (!f || grid <= 0) throw CudaError{cudaErrorInvalidConfiguration, "persistent cycle kernel", __FILE__, __LINE__};
  BatchDev b = B;
  float* v = V;
  double* ww = w;
  BatchCycle c = C;
  void* args[] = {&b, &v, &ww, &c};
  SMGPU_CUDA_TRY(cudaLaunchCooperativeKernel(f, dim3(grid), dim3(persist_nt(cand)), args, persist_smem(B, smem_hv), st));
}

// ------------------------------------------------------------------ launchers
void launch_b_start(const BatchDev& B, uint64_t seed, double* w, cudaStream_t st) {
  k_b_start<<<B.nchunks, kNT, 0, st>>>(B, seed, w);
}
void launch_b_to_padded(const BatchDev& B, const double* src, double* w, cudaStream_t st) {
  k_b_to_padded<<<B.nchunks, kNT, 0, st>>>(B, src, w);
}
void launch_b_from_padded(const BatchDev& B, const double* w, double* dst, cudaStream_t st) {
  k_b_from_padded<<<B.nchunks, kNT, 0, st>>>(B, w, dst);
}
void launch_b_convert(const BatchDev& B, const double* w, float* v, cudaStream_t st) {
  int64_t g = (B.LEN + kNT - 1) / kNT;
  if (g > 152 * 8) g = 152 * 8;
  k_b_convert<<<(int)(g < 1 ? 1 : g), kNT, 0, st>>>(w, v, B.LEN);
}
void launch_b_init(const BatchDev& B, const double* w, float* V0, cudaStream_t st) {
  k_b_selfdot<<<B.nchunks, kNT, 0, st>>>(B, w);
  k_b_init_scale<<<B.nchunks, kNT, 0, st>>>(B, w, V0);
}
void launch_b_sturm(const BatchDev& B, int k, int lock, cudaStream_t st) {
  int threads = ((B.num_ev * kLPE + 31) / 32) * 32;
  if (threads > 1024) threads = 1024;
  if (threads < 32) threads = 32;
  const size_t shm = sizeof(double) * (3 * (size_t)B.lm + B.num_ev);
  k_b_sturm<<<B.nprob, threads, shm, st>>>(B, k, lock);
}
void launch_b_orth(const BatchDev& B, float* V, double* w, int it0, cudaStream_t st) {
  const size_t hsh = 2 * sizeof(double) * (size_t)(it0 + 1);  // h_j and their FP32 splits
  k_b_orth_dot<<<B.nchunks, kNT, 0, st>>>(B, V, w, it0);
  k_b_orth_axpy<<<B.nchunks, kNT, hsh, st>>>(B, V, w, it0);
  k_b_orth_dot2<<<B.nchunks, kNT, 0, st>>>(B, V, w, it0);
  k_b_orth_axpy2<<<B.nchunks, kNT, hsh, st>>>(B, V, w, it0);
  k_b_orth_scale<<<B.nchunks, kNT, 0, st>>>(B, V, w, it0);
}
void launch_b_cycle_end(const BatchDev& B, cudaStream_t st) { k_b_cycle_end<<<1, 256, 0, st>>>(B); }
void launch_b_restart(const BatchDev& B, float* V, float* U, cudaStream_t st) {
  const int m = B.lm - 1, ls = B.ls;
  const int NP = ls * (ls + 1) / 2 + ls;
  k_b_jacobi<<<B.nprob, 256, jacobi_smem(m), st>>>(B, m, 1);
  k_b_restart_small<<<B.nprob, 256, 0, st>>>(B);
  const bool reg = ls <= kBRLS && sizeof(float) * (size_t)m * kBRLS <= 48 * 1024;
  if (reg) k_b_rotate_r<<<B.nchunks, kNT, sizeof(float) * m * kBRLS, st>>>(B, V, U);
  else k_b_rotate<<<B.nchunks, kNT, 0, st>>>(B, V, U);
  if (ls <= kBRLS && NP <= kNT)
    k_b_gram_r<<<B.nchunks, kNT, sizeof(float) * 2 * (ls + 1) * 129, st>>>(B, U, V + (int64_t)(B.lm - 1) * B.LEN);
  else
    k_b_gram<<<B.nchunks, kNT, sizeof(float) * (ls + 1) * 64, st>>>(B, U, V + (int64_t)(B.lm - 1) * B.LEN);
  if (ls <= 32) k_b_chol_df<<<B.nprob, 32, 0, st>>>(B);
  else k_b_chol<<<B.nprob, 128, sizeof(double) * (NP + ls * ls), st>>>(B);
  if (reg) k_b_apply_r<<<B.nchunks, kNT, 0, st>>>(B, U, V);
  else k_b_apply<<<B.nchunks, kNT, 0, st>>>(B, U, V);
}
void launch_b_jacobi_one(const BatchDev& B, int p, int n, cudaStream_t st) {
  k_b_jacobi_one<<<1, 256, jacobi_smem(n), st>>>(B, p, n);
}
void launch_b_ritz(const BatchDev& B, const float* V, int p, int elit, int nev, int64_t len, double* R,
                   cudaStream_t st) {
  int64_t g = (len + kNT - 1) / kNT;
  if (g > 152 * 4) g = 152 * 4;
  k_b_ritz<<<(int)(g < 1 ? 1 : g), kNT, 0, st>>>(B, V, p, elit, nev, R);
}

}  // namespace smgpu
