// Thick-restart Lanczos on the GPU: the device half of TRL
// (src/ShellModel/lanczos_methods.jl:1-91), diagonalize_T! (:250-258),
// ThickRestart (:260-307), ReORTH (shellmodel_main.jl:1005-1012) and the Ritz
// vector assembly (shellmodel_main.jl:208-224).
//
// Every kernel reads its gate from device memory (LanczosFlags), so a whole
// restart cycle can be captured in one CUDA graph: once the convergence test
// sets `done`, the remaining kernels of the cycle return immediately.
//
// One iteration after the H·v (whose epilogue already produced per-CTA
// partials of α and w = Hv − β v_prev):
//   orth_dot   : α (summed by every CTA from the partials), w' = w − α v_k,
//                partials of h_j = v_j·w' and of ||w'||²
//   orth_axpy  : h (summed per CTA), w'' = w' − Σ h_j v_j, partials of ||w''||²
//   orth_dot2 / orth_axpy2 : second classical Gram-Schmidt pass, taken only
//                when ||w''||² < ||w'||²/2 (Daniel-Gragg-Kaufman-Stewart test)
//   orth_scale : β = ||w||, T entries, v_{k+1} = w/β
// Reductions are deterministic: a fixed grid writes per-CTA partial sums and
// every consumer adds them in the same fixed order, so all CTAs agree bit for
// bit on α, h, β and the second-pass decision.
//
// FP64 is used for all dot products, the orthogonalisation, the small
// eigenproblems and the Ritz vectors.  Krylov vectors are stored as TX
// (double in the plain form, float in the mixed form); in the mixed form the
// restart's basis rotation runs in FP32 with Kahan-compensated sums (its
// result is stored in FP32) and is re-orthonormalised in FP64 (Cholesky QR).
#include <cfloat>

#include "lanczos.cuh"
#include "lanczos_dev.cuh"

namespace smgpu {

namespace {
using namespace dev;


__global__ void k_start_vector(DevTables t, uint64_t seed, double* __restrict__ w) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < t.len_pad;
       i += (int64_t)gridDim.x * blockDim.x) {
    int b = find_block(t.off_pad, t.nb, i);
    int64_t loc = i - t.off_pad[b];
    int st = t.stride[b];
    int p = (int)(loc / st), n = (int)(loc % st);
    w[i] = (n < t.nn[b]) ? start_elem(seed, t.tdims[b] + (int64_t)p * t.nn[b] + n) : 0.0;
  }
}

__global__ void k_convert(const double* __restrict__ a, float* __restrict__ b, int64_t len) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < len; i += (int64_t)gridDim.x * blockDim.x)
    b[i] = (float)a[i];
}

template <class TX>
__global__ void k_to_padded(DevTables t, const double* __restrict__ src, TX* __restrict__ dst) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < t.len_pad;
       i += (int64_t)gridDim.x * blockDim.x) {
    int b = find_block(t.off_pad, t.nb, i);
    int64_t loc = i - t.off_pad[b];
    int st = t.stride[b];
    int p = (int)(loc / st), n = (int)(loc % st);
    dst[i] = (n < t.nn[b]) ? (TX)src[t.tdims[b] + (int64_t)p * t.nn[b] + n] : (TX)0;
  }
}
__global__ void k_from_padded(DevTables t, const double* __restrict__ src, double* __restrict__ dst) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < t.len_pad;
       i += (int64_t)gridDim.x * blockDim.x) {
    int b = find_block(t.off_pad, t.nb, i);
    int64_t loc = i - t.off_pad[b];
    int st = t.stride[b];
    int p = (int)(loc / st), n = (int)(loc % st);
    if (n < t.nn[b]) dst[t.tdims[b] + (int64_t)p * t.nn[b] + n] = src[i];
  }
}

// partials[j*G + cta] = Σ_{i in chunk} X_j[i]·y[i]  (j < m);  j = m: y·y if self.
template <class TX>
__global__ void __launch_bounds__(kNT) k_multidot(const TX* __restrict__ X, int64_t ld, int m,
                                                  const double* __restrict__ y, int64_t len, int self,
                                                  double* __restrict__ partials, int G) {
  __shared__ double red8[(kNT / 32) * 8];
  int64_t cb, ce;
  chunk_of(len, G, cb, ce);
  const int mt = m + (self ? 1 : 0);
  for (int j0 = 0; j0 < mt; j0 += 8) {
    double acc[8];
#pragma unroll
    for (int q = 0; q < 8; ++q) acc[q] = 0.0;
    for (int64_t i = cb + threadIdx.x; i < ce; i += kNT) {
      const double yi = y[i];
#pragma unroll
      for (int q = 0; q < 8; ++q) {
        const int j = j0 + q;
        if (j < m) acc[q] = fma(widen(X[(int64_t)j * ld + i]), yi, acc[q]);
        else if (j == m && self) acc[q] = fma(yi, yi, acc[q]);
      }
    }
    const double s = block_sum8<kNT>(acc, red8);
    if (threadIdx.x < 8 && j0 + (int)threadIdx.x < mt) partials[(int64_t)(j0 + threadIdx.x) * G + blockIdx.x] = s;
  }
}

// out[j] = f(Σ_g partials[j*G+g]), one warp per j.
__global__ void __launch_bounds__(kNT) k_reduce(const double* __restrict__ partials, int G, int m, int mode,
                                                double* __restrict__ out) {
  __shared__ double res[1024];
  for (int j0 = 0; j0 < m; j0 += 1024) {
    const int mm = min(1024, m - j0);
    sum_partials_many<kNT>(partials + (int64_t)j0 * G, G, mm, res);
    for (int j = threadIdx.x; j < mm; j += kNT) out[j0 + j] = (mode == RED_INVNORM) ? 1.0 / sqrt(res[j]) : res[j];
    __syncthreads();
  }
}

template <class TX>
__global__ void __launch_bounds__(kNT) k_scale_store(const double* __restrict__ w, TX* __restrict__ out,
                                                     const double* __restrict__ scale, int64_t len) {
  const double s = *scale;
  for (int64_t i = blockIdx.x * (int64_t)kNT + threadIdx.x; i < len; i += (int64_t)gridDim.x * kNT)
    out[i] = (TX)(w[i] * s);
}

// ------------------------------------------------------------ orthogonalisation
template <class TX>
__global__ void __launch_bounds__(kNT) k_orth_dot(const TX* __restrict__ V, int64_t ld, int it0, double* w,
                                                  const double* __restrict__ alpha_part, int nalpha,
                                                  double* __restrict__ pdot, int G, const LanczosFlags* fl) {
  if (cta_gate(threadIdx.x == 0 && stopped(fl))) return;
  __shared__ double red[kNT / 32];
  __shared__ double red8[(kNT / 32) * 8];
  const double alpha = sum_partials<kNT>(alpha_part + (int64_t)it0 * nalpha, nalpha, red);
  const TX* __restrict__ vk = V + (int64_t)it0 * ld;
  const int m = it0 + 1;
  int64_t cb, ce;
  chunk_of(ld, G, cb, ce);
  for (int j0 = 0; j0 <= m; j0 += 8) {
    double acc[8];
#pragma unroll
    for (int q = 0; q < 8; ++q) acc[q] = 0.0;
    for (int64_t i = cb + 4 * threadIdx.x; i < ce; i += 4 * kNT) {
      double wv[4];
      load4(w + i, wv);
      if (j0 == 0) {
        double x[4];
        load4(vk + i, x);
#pragma unroll
        for (int u = 0; u < 4; ++u) wv[u] = fma(-alpha, x[u], wv[u]);
        store4(w + i, wv);
      }
#pragma unroll
      for (int q = 0; q < 8; ++q) {
        const int j = j0 + q;
        if (j < m) {
          double x[4];
          load4(V + (int64_t)j * ld + i, x);
#pragma unroll
          for (int u = 0; u < 4; ++u) acc[q] = fma(x[u], wv[u], acc[q]);
        } else if (j == m) {
#pragma unroll
          for (int u = 0; u < 4; ++u) acc[q] = fma(wv[u], wv[u], acc[q]);
        }
      }
    }
    const double s = block_sum8<kNT>(acc, red8);
    if (threadIdx.x < 8 && j0 + (int)threadIdx.x <= m) pdot[(int64_t)(j0 + threadIdx.x) * G + blockIdx.x] = s;
  }
}

// Second-pass decision, identical in every CTA: ||w''||² < ||w'||² / 2.
__device__ __forceinline__ bool need_second(const double* pdot, const double* pn1, int m, int G, double* red) {
  const double n0 = sum_partials<kNT>(pdot + (int64_t)m * G, G, red);
  const double n1 = sum_partials<kNT>(pn1, G, red);
  return n1 < 0.5 * n0;
}

// w -= Σ_j h_j V_j with h_j = Σ_g ph[j*G+g];  pout[cta] = ||w_chunk||².
template <class TX>
__device__ __forceinline__ void orth_subtract(const TX* __restrict__ V, int64_t ld, int m, double* w,
                                              const double* __restrict__ ph, double* __restrict__ pout, int G,
                                              double* hs, double* red, bool sum_h = true) {
  if (sum_h) sum_partials_many<kNT>(ph, G, m, hs);  // else hs holds the h_j
  int64_t cb, ce;
  chunk_of(ld, G, cb, ce);
  double nrm = 0.0;
  for (int64_t i = cb + 4 * threadIdx.x; i < ce; i += 4 * kNT) {
    double t[4];
    load4(w + i, t);
    for (int j = 0; j < m; ++j) {
      double x[4];
      load4(V + (int64_t)j * ld + i, x);
      const double hj = hs[j];
#pragma unroll
      for (int u = 0; u < 4; ++u) t[u] = fma(-hj, x[u], t[u]);
    }
    store4(w + i, t);
#pragma unroll
    for (int u = 0; u < 4; ++u) nrm = fma(t[u], t[u], nrm);
  }
  double s = block_sum_all<kNT>(nrm, red);
  if (threadIdx.x == 0) pout[blockIdx.x] = s;
}

// First subtraction.  FP32 basis: when the projections are small
// (L.fastnorm, normally kFastNorm) β comes from the norm before the subtraction and this pass also
// writes T's β, the scalars and v_{it0+1} (fastnorm = 1; the second-pass and
// scaling kernels then return at once); every CTA takes the same decision
// from the same partial sums.
template <class TX>
__global__ void __launch_bounds__(kNT) k_orth_axpy(const TX* __restrict__ V, int64_t ld, int it0, double* w,
                                                   const double* __restrict__ pdot, double* __restrict__ pn1, int G,
                                                   TX* __restrict__ vnext, double* T, int lm, LanczosScalars* sc,
                                                   LanczosFlags* fl, double fastnorm) {
  if (cta_gate(threadIdx.x == 0 && stopped(fl))) return;
  extern __shared__ double hs[];
  __shared__ double red[kNT / 32];
  const int m = it0 + 1;
  if constexpr (sizeof(TX) == 4) {
    const double n0 = sum_partials<kNT>(pdot + (int64_t)m * G, G, red);
    sum_partials_many<kNT>(pdot, G, m, hs);
    double hsq = 0.0;
    for (int j = 0; j < m; ++j) hsq = fma(hs[j], hs[j], hsq);
    const bool fast = n0 > 0.0 && hsq <= fastnorm * n0;
    if (blockIdx.x == 0 && threadIdx.x == 0) fl->fastnorm = fast ? 1 : 0;
    if (fast) {
      const double beta = sqrt(n0 - hsq);
      if (blockIdx.x == 0 && threadIdx.x == 0) {
        T[(int64_t)it0 * lm + it0 + 1] = beta;
        T[(int64_t)(it0 + 1) * lm + it0] = beta;
        sc->beta = beta;
        sc->inv_beta = 1.0 / beta;
        fl->second = 0;
      }
      const double inv = 1.0 / beta;
      int64_t cb, ce;
      chunk_of(ld, G, cb, ce);
      for (int64_t i = cb + 4 * threadIdx.x; i < ce; i += 4 * kNT) {
        double t[4];
        load4(w + i, t);
        for (int j = 0; j < m; ++j) {
          double x[4];
          load4(V + (int64_t)j * ld + i, x);
          const double hj = hs[j];
#pragma unroll
          for (int u = 0; u < 4; ++u) t[u] = fma(-hj, x[u], t[u]);
        }
        *reinterpret_cast<float4*>(vnext + i) =
            make_float4((float)(t[0] * inv), (float)(t[1] * inv), (float)(t[2] * inv), (float)(t[3] * inv));
      }
      return;
    }
    orth_subtract<TX>(V, ld, m, w, pdot, pn1, G, hs, red, false);
  } else {
    orth_subtract<TX>(V, ld, m, w, pdot, pn1, G, hs, red);
  }
}

// Whether the first subtraction already finished the iteration (FP32 basis).
template <class TX>
__device__ __forceinline__ bool took_fastnorm(const LanczosFlags* fl) {
  if constexpr (sizeof(TX) == 4) return *(volatile const int*)&fl->fastnorm != 0;
  return false;
}

template <class TX>
__global__ void __launch_bounds__(kNT) k_orth_dot2(const TX* __restrict__ V, int64_t ld, int it0,
                                                   const double* __restrict__ w, const double* __restrict__ pdot,
                                                   const double* __restrict__ pn1, double* __restrict__ pdot2,
                                                   int G, const LanczosFlags* fl) {
  if (cta_gate(threadIdx.x == 0 && (stopped(fl) || took_fastnorm<TX>(fl)))) return;
  __shared__ double red[kNT / 32];
  __shared__ double red8[(kNT / 32) * 8];
  const int m = it0 + 1;
  if (!need_second(pdot, pn1, m, G, red)) return;
  int64_t cb, ce;
  chunk_of(ld, G, cb, ce);
  for (int j0 = 0; j0 < m; j0 += 8) {
    double acc[8];
#pragma unroll
    for (int q = 0; q < 8; ++q) acc[q] = 0.0;
    for (int64_t i = cb + 4 * threadIdx.x; i < ce; i += 4 * kNT) {
      double wv[4];
      load4(w + i, wv);
#pragma unroll
      for (int q = 0; q < 8; ++q)
        if (j0 + q < m) {
          double x[4];
          load4(V + (int64_t)(j0 + q) * ld + i, x);
#pragma unroll
          for (int u = 0; u < 4; ++u) acc[q] = fma(x[u], wv[u], acc[q]);
        }
    }
    const double s = block_sum8<kNT>(acc, red8);
    if (threadIdx.x < 8 && j0 + (int)threadIdx.x < m) pdot2[(int64_t)(j0 + threadIdx.x) * G + blockIdx.x] = s;
  }
}

template <class TX>
__global__ void __launch_bounds__(kNT) k_orth_axpy2(const TX* __restrict__ V, int64_t ld, int it0, double* w,
                                                    const double* __restrict__ pdot,
                                                    const double* __restrict__ pn1,
                                                    const double* __restrict__ pdot2, double* __restrict__ pn2,
                                                    int G, const LanczosFlags* fl) {
  if (cta_gate(threadIdx.x == 0 && (stopped(fl) || took_fastnorm<TX>(fl)))) return;
  extern __shared__ double hs[];
  __shared__ double red[kNT / 32];
  const int m = it0 + 1;
  if (!need_second(pdot, pn1, m, G, red)) return;
  orth_subtract<TX>(V, ld, m, w, pdot2, pn2, G, hs, red);
}

// β = ||w||, T[it0+1,it0] = T[it0,it0+1] = β, v_{it0+1} = w/β.  A zero β means
// the Krylov space is exhausted: stop with the current T.
template <class TX>
__global__ void __launch_bounds__(kNT) k_orth_scale(const double* __restrict__ w, TX* __restrict__ vnext,
                                                    const double* __restrict__ pdot,
                                                    const double* __restrict__ pn1,
                                                    const double* __restrict__ pn2, int G, int it0, double* T,
                                                    int lm, int64_t len, LanczosScalars* sc, LanczosFlags* fl) {
  if (cta_gate(threadIdx.x == 0 && (stopped(fl) || took_fastnorm<TX>(fl)))) return;
  __shared__ double red[kNT / 32];
  const int m = it0 + 1;
  const bool second = need_second(pdot, pn1, m, G, red);
  const double nrm = sum_partials<kNT>(second ? pn2 : pn1, G, red);
  const double beta = sqrt(nrm);
  const bool ok = (beta > 0.0) && (beta < INFINITY);
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    if (ok) {
      T[(int64_t)it0 * lm + it0 + 1] = beta;
      T[(int64_t)(it0 + 1) * lm + it0] = beta;
      sc->beta = beta;
      sc->inv_beta = 1.0 / beta;
      fl->second = second ? 1 : 0;
      if (second) fl->n_second += 1;
    } else {
      fl->exh_k = it0 + 1;
      fl->exhausted = 1;
    }
  }
  if (!ok) return;
  const double inv = 1.0 / beta;
  for (int64_t i = blockIdx.x * (int64_t)kNT + threadIdx.x; i < len; i += (int64_t)gridDim.x * kNT)
    vnext[i] = (TX)(w[i] * inv);
}

// ---------------------------------------- FP32 basis, double-float residual
// The FP32-mixed solve keeps w = wh + wl as a double-float pair: every
// vector-length operation below runs on the FP32 pipe (exact FP32 products
// by fused two-products, sums in double-float), and so do the CTA reductions
// and the per-CTA partials (stored as (hi, lo) float pairs in the FP64 partial
// arrays, α partials of the H·v epilogue included); FP64 is left to one
// thread's scalar work (β, the second-pass test).
// 512-thread CTAs, two per SM: the streams need the memory-level parallelism.
constexpr int kONT = 512;

// α (from the H·v partials), w' = w − α v_k, partials of v_j·w' (j <= it0)
// and of ||w'||² (slot it0+1).
__global__ void __launch_bounds__(kONT, 2) k_orth_dot_df(const float* __restrict__ V, int64_t ld, int it0,
                                                         float* __restrict__ wh, float* __restrict__ wl,
                                                         const double* __restrict__ alpha_part, int nalpha,
                                                         double* __restrict__ pdot, int G, const LanczosFlags* fl) {
  if (cta_gate(threadIdx.x == 0 && stopped(fl))) return;
  __shared__ double red[kONT / 32];
  __shared__ double red8[(kONT / 32) * 8];
  const float2 alpha = sum_partials_df<kONT>(reinterpret_cast<const float2*>(alpha_part) + (int64_t)it0 * nalpha,
                                             nalpha, reinterpret_cast<float2*>(red));
  const float aH = -alpha.x, aL = -alpha.y;
  const float* __restrict__ vk = V + (int64_t)it0 * ld;
  const int m = it0 + 1;
  int64_t cb, ce;
  chunk_of(ld, G, cb, ce);
  // blocks of 16 basis vectors per pass over the chunk.  The per-thread sums
  // are FP32 (a thread adds ~16 products of one chunk; the rounding they
  // leave in h_j is ~1e-10 ||w||, far below the FP32 basis itself), the CTA
  // sums double-float.
  constexpr int JB = 16;
  for (int j0 = 0; j0 <= m; j0 += JB) {
    float acc[JB];
#pragma unroll
    for (int q = 0; q < JB; ++q) acc[q] = 0.f;
    for (int64_t i = cb + 4 * threadIdx.x; i < ce; i += 4 * kONT) {
      const float4 a = *reinterpret_cast<const float4*>(wh + i);
      const float4 b = *reinterpret_cast<const float4*>(wl + i);
      float h[4] = {a.x, a.y, a.z, a.w}, l[4] = {b.x, b.y, b.z, b.w};
      if (j0 == 0) {
        const float4 x = *reinterpret_cast<const float4*>(vk + i);
        df_fma(h[0], l[0], x.x, aH, aL);
        df_fma(h[1], l[1], x.y, aH, aL);
        df_fma(h[2], l[2], x.z, aH, aL);
        df_fma(h[3], l[3], x.w, aH, aL);
        *reinterpret_cast<float4*>(wh + i) = make_float4(h[0], h[1], h[2], h[3]);
        *reinterpret_cast<float4*>(wl + i) = make_float4(l[0], l[1], l[2], l[3]);
      }
#pragma unroll
      for (int q = 0; q < JB; ++q) {
        const int j = j0 + q;
        if (j < m) {
          const float4 x = *reinterpret_cast<const float4*>(V + (int64_t)j * ld + i);
          acc[q] = __fmaf_rn(x.w, h[3], __fmaf_rn(x.z, h[2], __fmaf_rn(x.y, h[1], __fmaf_rn(x.x, h[0], acc[q]))));
        } else if (j == m) {
          acc[q] = __fmaf_rn(h[3], h[3], __fmaf_rn(h[2], h[2], __fmaf_rn(h[1], h[1], __fmaf_rn(h[0], h[0], acc[q]))));
        }
      }
    }
#pragma unroll
    for (int g = 0; g < JB / 8; ++g) {
      if (j0 + 8 * g > m) break;
      DFAcc d[8];
#pragma unroll
      for (int q = 0; q < 8; ++q) {
        d[q].hi = acc[8 * g + q];
        d[q].lo = 0.f;
      }
      float2 s;
      block_sum_df<kONT, 8>(d, red8, s);
      const int j = j0 + 8 * g + (int)threadIdx.x;
      if (threadIdx.x < 8 && j <= m) reinterpret_cast<float2*>(pdot)[(int64_t)j * G + blockIdx.x] = s;
    }
  }
}

// w -= Σ_j h_j V_j (h_j = Σ_g ph[j*G+g], split once per CTA); pout[cta] = ||w chunk||².
__device__ __forceinline__ void orth_subtract_df(const float* __restrict__ V, int64_t ld, int m,
                                                 float* __restrict__ wh, float* __restrict__ wl,
                                                 const double* __restrict__ ph, double* __restrict__ pout, int G,
                                                 double* hs, double* red) {
  float* hh = reinterpret_cast<float*>(hs + m + 2);
  float* hl = hh + m;
  sum_partials_many_df<kONT>(reinterpret_cast<const float2*>(ph), G, m, hh, hl);
  int64_t cb, ce;
  chunk_of(ld, G, cb, ce);
  DFAcc nrm;
  nrm.init();
  for (int64_t i = cb + 4 * threadIdx.x; i < ce; i += 4 * kONT) {
    DFAcc s4[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) s4[u].init();
    for (int j = 0; j < m; ++j) {
      const float4 x = *reinterpret_cast<const float4*>(V + (int64_t)j * ld + i);
      const float a = hh[j], b = hl[j];
      s4[0].add_prod2(x.x, a, b);
      s4[1].add_prod2(x.y, a, b);
      s4[2].add_prod2(x.z, a, b);
      s4[3].add_prod2(x.w, a, b);
    }
    const float4 a = *reinterpret_cast<const float4*>(wh + i);
    const float4 b = *reinterpret_cast<const float4*>(wl + i);
    float h[4] = {a.x, a.y, a.z, a.w}, l[4] = {b.x, b.y, b.z, b.w};
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      df_add(h[u], l[u], -s4[u].hi, -s4[u].lo);
      nrm.add_prod2(h[u], h[u], 2.0f * l[u]);
    }
    *reinterpret_cast<float4*>(wh + i) = make_float4(h[0], h[1], h[2], h[3]);
    *reinterpret_cast<float4*>(wl + i) = make_float4(l[0], l[1], l[2], l[3]);
  }
  DFAcc n1[1] = {nrm};
  float2 s;
  block_sum_df<kONT, 1>(n1, red, s);
  if (threadIdx.x == 0) reinterpret_cast<float2*>(pout)[blockIdx.x] = s;
}

__global__ void __launch_bounds__(kONT, 2) k_orth_axpy_df(const float* __restrict__ V, int64_t ld, int it0, float* wh,
                                                      float* wl, const double* __restrict__ pdot,
                                                      double* __restrict__ pn1, int G, LanczosScalars* sc,
                                                      const LanczosFlags* fl) {
  if (cta_gate(threadIdx.x == 0 && stopped(fl))) return;
  extern __shared__ double hs[];
  __shared__ double red[kONT / 32];
  const int m = it0 + 1;
  if (blockIdx.x == 0) {
    // ||w − α v_k||² (slot m of the first-pass partials), for the second-pass test
    const float2 n0 = sum_partials_df<kONT>(reinterpret_cast<const float2*>(pdot) + (int64_t)m * G, G,
                                            reinterpret_cast<float2*>(red));
    if (threadIdx.x == 0) sc->w_norm2 = (double)n0.x + (double)n0.y;
  }
  orth_subtract_df(V, ld, m, wh, wl, pdot, pn1, G, hs, red);
}

// Second-pass decision of the double-float solve: ||w''||² < ||w'||² / 2.
// The sum in double-float; one thread compares in FP64 and broadcasts.
__device__ __forceinline__ bool need_second_df(const LanczosScalars* sc, const double* pn1, int G, double* red) {
  const float2 n1 = sum_partials_df<kONT>(reinterpret_cast<const float2*>(pn1), G, reinterpret_cast<float2*>(red));
  return cta_gate(threadIdx.x == 0 && (double)n1.x + (double)n1.y < 0.5 * sc->w_norm2);
}

__global__ void __launch_bounds__(kONT, 2) k_orth_dot2_df(const float* __restrict__ V, int64_t ld, int it0,
                                                      const float* __restrict__ wh, const float* __restrict__ wl,
                                                      const LanczosScalars* sc,
                                                      const double* __restrict__ pn1, double* __restrict__ pdot2,
                                                      int G, const LanczosFlags* fl) {
  if (cta_gate(threadIdx.x == 0 && stopped(fl))) return;
  __shared__ double red[kONT / 32];
  const int m = it0 + 1;
  if (!need_second_df(sc, pn1, G, red)) return;
  __shared__ double red8[(kONT / 32) * 8];
  int64_t cb, ce;
  chunk_of(ld, G, cb, ce);
  for (int j0 = 0; j0 < m; j0 += 8) {
    DFAcc acc[8];
#pragma unroll
    for (int q = 0; q < 8; ++q) acc[q].init();
    for (int64_t i = cb + 4 * threadIdx.x; i < ce; i += 4 * kONT) {
      const float4 a = *reinterpret_cast<const float4*>(wh + i);
      const float4 b = *reinterpret_cast<const float4*>(wl + i);
#pragma unroll
      for (int q = 0; q < 8; ++q)
        if (j0 + q < m) {
          const float4 x = *reinterpret_cast<const float4*>(V + (int64_t)(j0 + q) * ld + i);
          acc[q].add_prod2(x.x, a.x, b.x);
          acc[q].add_prod2(x.y, a.y, b.y);
          acc[q].add_prod2(x.z, a.z, b.z);
          acc[q].add_prod2(x.w, a.w, b.w);
        }
    }
    float2 s;
    block_sum_df<kONT, 8>(acc, red8, s);
    if (threadIdx.x < 8 && j0 + (int)threadIdx.x < m)
      reinterpret_cast<float2*>(pdot2)[(int64_t)(j0 + threadIdx.x) * G + blockIdx.x] = s;
  }
}

__global__ void __launch_bounds__(kONT, 2) k_orth_axpy2_df(const float* __restrict__ V, int64_t ld, int it0, float* wh,
                                                       float* wl, const LanczosScalars* sc,
                                                       const double* __restrict__ pn1,
                                                       const double* __restrict__ pdot2, double* __restrict__ pn2,
                                                       int G, const LanczosFlags* fl) {
  if (cta_gate(threadIdx.x == 0 && stopped(fl))) return;
  extern __shared__ double hs[];
  __shared__ double red[kONT / 32];
  const int m = it0 + 1;
  if (!need_second_df(sc, pn1, G, red)) return;
  orth_subtract_df(V, ld, m, wh, wl, pdot2, pn2, G, hs, red);
}

// β = ||w||, T entries, v_{it0+1} = w/β rounded to FP32 (as k_orth_scale).
__global__ void __launch_bounds__(kONT, 2) k_orth_scale_df(const float* __restrict__ wh, const float* __restrict__ wl,
                                                       float* __restrict__ vnext, const double* __restrict__ pn1,
                                                       const double* __restrict__ pn2, int G, int it0, double* T,
                                                       int lm, int64_t len, LanczosScalars* sc, LanczosFlags* fl) {
  if (cta_gate(threadIdx.x == 0 && stopped(fl))) return;
  __shared__ double red[kONT / 32];
  __shared__ float s_inv[2];
  const bool second = need_second_df(sc, pn1, G, red);
  const float2 nrm =
      sum_partials_df<kONT>(reinterpret_cast<const float2*>(second ? pn2 : pn1), G, reinterpret_cast<float2*>(red));
  // β and 1/β by one thread (FP64), broadcast as a double-float pair
  bool ok0 = false;
  if (threadIdx.x == 0) {
    const double beta = sqrt((double)nrm.x + (double)nrm.y);
    ok0 = (beta > 0.0) && (beta < INFINITY);
    if (blockIdx.x == 0) {
      if (ok0) {
        T[(int64_t)it0 * lm + it0 + 1] = beta;
        T[(int64_t)(it0 + 1) * lm + it0] = beta;
        sc->beta = beta;
        sc->inv_beta = 1.0 / beta;
        fl->second = second ? 1 : 0;
        if (second) fl->n_second += 1;
      } else {
        fl->exh_k = it0 + 1;
        fl->exhausted = 1;
      }
    }
    if (ok0) df_from_double(1.0 / beta, s_inv[0], s_inv[1]);
  }
  if (!cta_gate(ok0)) return;
  const float ih = s_inv[0], il = s_inv[1];
  for (int64_t i = 4 * (blockIdx.x * (int64_t)kONT + threadIdx.x); i < len; i += 4 * (int64_t)gridDim.x * kONT) {
    const float4 h = *reinterpret_cast<const float4*>(wh + i);
    const float4 l = *reinterpret_cast<const float4*>(wl + i);
    *reinterpret_cast<float4*>(vnext + i) =
        make_float4(__fmaf_rn(h.x, ih, __fmaf_rn(l.x, ih, __fmul_rn(h.x, il))),
                    __fmaf_rn(h.y, ih, __fmaf_rn(l.y, ih, __fmul_rn(h.y, il))),
                    __fmaf_rn(h.z, ih, __fmaf_rn(l.z, ih, __fmul_rn(h.z, il))),
                    __fmaf_rn(h.w, ih, __fmaf_rn(l.w, ih, __fmul_rn(h.w, il))));
  }
}


// Lowest eigenvalues (diagonalize_T!, lanczos_methods.jl:250-258): α from the
// H·v epilogue partials, then sturm_step.
__global__ void k_sturm(double* __restrict__ T, int lm, int k, int lock, int num_ev, double* en, int nh,
                        double tol, int64_t mdim, const double* __restrict__ alpha_part, int nalpha,
                        int alpha_df, LanczosFlags* fl) {
  if (cta_gate(threadIdx.x == 0 && fl->done)) return;
  if (cta_gate(threadIdx.x == 0 && fl->exhausted && k > fl->exh_k)) {
    // the Krylov space ended at exh_k; T_k was never completed
    if (threadIdx.x == 0) { fl->done = 1; fl->elit = fl->exh_k; }
    return;
  }
  __shared__ double red[32];
  const int tid = threadIdx.x;
  // α of this iteration from the H·v epilogue partials
  {
    double x = 0.0;
    if (alpha_df) {  // double-float (hi, lo) partials of the FP32-mixed H·v
      const float2* ap = reinterpret_cast<const float2*>(alpha_part) + (int64_t)(k - 1) * nalpha;
      for (int i = tid; i < nalpha; i += blockDim.x) x += (double)ap[i].x + (double)ap[i].y;
    } else {
      for (int i = tid; i < nalpha; i += blockDim.x) x += alpha_part[(int64_t)(k - 1) * nalpha + i];
    }
    x = warp_sum(x);
    if ((tid & 31) == 0) red[tid >> 5] = x;
    __syncthreads();
    if (tid == 0) {
      double s = 0.0;
      for (int wdx = 0; wdx < (int)(blockDim.x >> 5); ++wdx) s += red[wdx];
      T[(int64_t)(k - 1) * lm + (k - 1)] = s;
    }
    __syncthreads();
  }
  sturm_step(T, lm, k, lock, num_ev, en, nh, tol, mdim, fl);
}

// Eigenvectors of T[0:n,0:n] (ThickRestart / Ritz vectors), gated on the flags.
template <int NT>
__global__ void __launch_bounds__(NT) k_jacobi(const double* __restrict__ T, int ldt, int n, double* A, double* Z,
                                               double* evals, const LanczosFlags* fl, int gate) {
  if (gate && stopped(fl)) return;
  jacobi_eig<NT>(T, ldt, n, A, Z, evals);
}
template <int NT>
__global__ void __launch_bounds__(NT) k_jacobi_refined(const double* __restrict__ T, int ldt, int n, double* A,
                                                       double* evals, const LanczosFlags* fl, int gate) {
  if (gate && stopped(fl)) return;
  jacobi_eig_refined<NT>(T, ldt, n, A, evals);
}
template <int NT>
__global__ void __launch_bounds__(NT) k_jacobi_df(const double* __restrict__ T, int ldt, int n, double* A,
                                                  double* evals, const LanczosFlags* fl, int gate) {
  if (gate && stopped(fl)) return;
  jacobi_eig_df<NT>(T, ldt, n, A, evals);
}

// ThickRestart's small part (lanczos_methods.jl:261-271): new arrowhead T.
__global__ void k_restart_small(double* T, int lm, int ls, const double* evals, const double* vecs, float* vecs_f,
                                const LanczosFlags* fl) {
  if (stopped(fl)) return;
  const int m = lm - 1;
  for (int idx = threadIdx.x; idx < m * ls; idx += blockDim.x) vecs_f[idx] = (float)vecs[idx];
  __shared__ double beta;
  if (threadIdx.x == 0) beta = T[(int64_t)(lm - 1) * lm + (lm - 2)];
  __syncthreads();
  for (int idx = threadIdx.x; idx < lm * lm; idx += blockDim.x) T[idx] = 0.0;
  __syncthreads();
  for (int k = threadIdx.x; k < ls; k += blockDim.x) {
    T[(int64_t)k * lm + k] = evals[k];
    double tmp = beta * vecs[(int64_t)k * m + (m - 1)];
    T[(int64_t)k * lm + ls] = tmp;
    T[(int64_t)ls * lm + k] = tmp;
  }
}

// U_k = Σ_{j<m} Y[j,k] V_j  (k < ls).  FP64 for the plain form; FP32 with
// Kahan sums for the mixed form (the result is stored in FP32).
template <class TX>
__global__ void __launch_bounds__(kNT) k_restart_rotate(const TX* __restrict__ V, TX* __restrict__ U,
                                                        const double* __restrict__ Y, const float* __restrict__ Yf,
                                                        int m, int ls, int64_t len,
                                                        const LanczosFlags* __restrict__ fl) {
  if (stopped(fl)) return;
  // Y (m x ls, column-major) is small and read through L1
  for (int64_t i = blockIdx.x * (int64_t)kNT + threadIdx.x; i < len; i += (int64_t)gridDim.x * kNT) {
    for (int k0 = 0; k0 < ls; k0 += 8) {
      if constexpr (sizeof(TX) == 4) {
        KahanF acc[8];
#pragma unroll
        for (int q = 0; q < 8; ++q) acc[q].init();
        for (int j = 0; j < m; ++j) {
          const float x = (float)V[(int64_t)j * len + i];
#pragma unroll
          for (int q = 0; q < 8; ++q)
            if (k0 + q < ls) acc[q].add(__fmul_rn(__ldg(Yf + (int64_t)(k0 + q) * m + j), x));
        }
#pragma unroll
        for (int q = 0; q < 8; ++q)
          if (k0 + q < ls) U[(int64_t)(k0 + q) * len + i] = (TX)acc[q].get();
      } else {
        double acc[8];
#pragma unroll
        for (int q = 0; q < 8; ++q) acc[q] = 0.0;
        for (int j = 0; j < m; ++j) {
          const double x = (double)V[(int64_t)j * len + i];
#pragma unroll
          for (int q = 0; q < 8; ++q)
            if (k0 + q < ls) acc[q] = fma(__ldg(Y + (int64_t)(k0 + q) * m + j), x, acc[q]);
        }
#pragma unroll
        for (int q = 0; q < 8; ++q)
          if (k0 + q < ls) U[(int64_t)(k0 + q) * len + i] = (TX)acc[q];
      }
    }
  }
}

// FP32-mixed forms of the restart streams: every basis vector is read once,
// products compensated (Kahan with the product inside the fused step).
//   rotate: U_k = Σ_{j<m} Y[j,k] V_j, one element per thread, all ls outputs
//           in registers, Y broadcast from shared memory (rows padded to 16).
constexpr int kRLS = 16;  // largest ls of the register-resident restart kernels
__global__ void __launch_bounds__(kNT) k_restart_rotate_f(const float* __restrict__ V, float* __restrict__ U,
                                                          const float* __restrict__ Yf, int m, int ls, int64_t len,
                                                          const LanczosFlags* __restrict__ fl) {
  if (cta_gate(threadIdx.x == 0 && stopped(fl))) return;
  extern __shared__ float ys[];  // m x kRLS: ys[j*kRLS + k] = Y[j,k]
  for (int idx = threadIdx.x; idx < m * kRLS; idx += kNT) {
    const int j = idx / kRLS, k = idx % kRLS;
    ys[idx] = k < ls ? Yf[(int64_t)k * m + j] : 0.f;
  }
  __syncthreads();
  for (int64_t i = blockIdx.x * (int64_t)kNT + threadIdx.x; i < len; i += (int64_t)gridDim.x * kNT) {
    KahanF acc[kRLS];
#pragma unroll
    for (int k = 0; k < kRLS; ++k) acc[k].init();
    int j = 0;
    for (; j + 4 <= m; j += 4) {
      float x[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) x[u] = V[(int64_t)(j + u) * len + i];
      // the four terms of a group summed with plain FMAs, the group sums
      // compensated (half the operations of a compensated step per term)
      const float4* y0 = reinterpret_cast<const float4*>(ys + (j + 0) * kRLS);
      const float4* y1 = reinterpret_cast<const float4*>(ys + (j + 1) * kRLS);
      const float4* y2 = reinterpret_cast<const float4*>(ys + (j + 2) * kRLS);
      const float4* y3 = reinterpret_cast<const float4*>(ys + (j + 3) * kRLS);
#pragma unroll
      for (int q = 0; q < kRLS / 4; ++q) {
        const float4 a = y0[q], b = y1[q], c = y2[q], d = y3[q];
        acc[4 * q].add(__fmaf_rn(d.x, x[3], __fmaf_rn(c.x, x[2], __fmaf_rn(b.x, x[1], __fmul_rn(a.x, x[0])))));
        acc[4 * q + 1].add(__fmaf_rn(d.y, x[3], __fmaf_rn(c.y, x[2], __fmaf_rn(b.y, x[1], __fmul_rn(a.y, x[0])))));
        acc[4 * q + 2].add(__fmaf_rn(d.z, x[3], __fmaf_rn(c.z, x[2], __fmaf_rn(b.z, x[1], __fmul_rn(a.z, x[0])))));
        acc[4 * q + 3].add(__fmaf_rn(d.w, x[3], __fmaf_rn(c.w, x[2], __fmaf_rn(b.w, x[1], __fmul_rn(a.w, x[0])))));
      }
    }
    for (; j < m; ++j) {
      const float x = V[(int64_t)j * len + i];
      const float4* y4 = reinterpret_cast<const float4*>(ys + j * kRLS);
#pragma unroll
      for (int q = 0; q < kRLS / 4; ++q) {
        const float4 y = y4[q];
        acc[4 * q].add_prod(y.x, x);
        acc[4 * q + 1].add_prod(y.y, x);
        acc[4 * q + 2].add_prod(y.z, x);
        acc[4 * q + 3].add_prod(y.w, x);
      }
    }
#pragma unroll
    for (int k = 0; k < kRLS; ++k)
      if (k < ls) U[(int64_t)k * len + i] = acc[k].get();
  }
}

//   apply: V_k = Σ_{j<=k} X[j,k] U_j, V_ls = V_{lm-1} − Σ_k c_k V_k; the ls
//          values of U in registers.
__global__ void __launch_bounds__(kNT) k_restart_apply_f(const float* __restrict__ U, float* __restrict__ V,
                                                         const double* __restrict__ X,
                                                         const double* __restrict__ cvec, int ls, int lm,
                                                         int64_t len, const LanczosFlags* __restrict__ fl) {
  if (cta_gate(threadIdx.x == 0 && stopped(fl))) return;
  __shared__ float xf[kRLS * kRLS + kRLS];
  for (int idx = threadIdx.x; idx < ls * ls; idx += kNT) xf[idx] = (float)X[idx];
  for (int idx = threadIdx.x; idx < ls; idx += kNT) xf[ls * ls + idx] = (float)cvec[idx];
  __syncthreads();
  for (int64_t i = blockIdx.x * (int64_t)kNT + threadIdx.x; i < len; i += (int64_t)gridDim.x * kNT) {
    float u[kRLS];
#pragma unroll
    for (int j = 0; j < kRLS; ++j) u[j] = j < ls ? U[(int64_t)j * len + i] : 0.f;
    KahanF last;
    last.init();
    last.add(V[(int64_t)(lm - 1) * len + i]);
#pragma unroll
    for (int k = 0; k < kRLS; ++k) {
      if (k >= ls) break;
      KahanF q;
      q.init();
#pragma unroll
      for (int j = 0; j <= k; ++j) q.add_prod(xf[k * ls + j], u[j]);
      const float qv = q.get();
      V[(int64_t)k * len + i] = qv;
      last.add_prod(-xf[ls * ls + k], qv);
    }
    V[(int64_t)ls * len + i] = last.get();
  }
}

//   Gram: tiles of 128 elements of the ls+1 vectors staged in shared memory,
//         double-buffered through registers (the next tile's loads are in
//         flight while the current one is multiplied); one thread per pair,
//         FP32 sums per tile added in double-float, partials as (hi, lo)
//         pairs.
__global__ void __launch_bounds__(kNT) k_gram_f(const float* __restrict__ U, const float* __restrict__ vl, int ls,
                                                int64_t len, double* __restrict__ partials, int G,
                                                const LanczosFlags* __restrict__ fl) {
  if (cta_gate(threadIdx.x == 0 && stopped(fl))) return;
  constexpr int TILE = 128;
  constexpr int TS = TILE + 1;
  constexpr int LD = ((kRLS + 1) * TILE + kNT - 1) / kNT;  // elements a thread stages per tile
  extern __shared__ float gt[];                 // 2 x (ls+1) x TS
  const int nv = ls + 1;
  const int P = ls * (ls + 1) / 2 + ls;
  int64_t cb, ce;
  chunk_of(len, G, cb, ce);
  int k = 0, l = 0;
  const bool act = (int)threadIdx.x < P;
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
      if (j < nv && t0 + x < ce) val = (j < ls) ? U[(int64_t)j * len + t0 + x] : vl[t0 + x];
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
  if (cb < ce) {
    load(cb);
    store(0);
  }
  __syncthreads();
  for (int64_t t0 = cb; t0 < ce; t0 += TILE) {
    const bool more = t0 + TILE < ce;
    if (more) load(t0 + TILE);
    const float* tl = gt + buf * nv * TS;
    if (act) {
      // the tile's products summed in FP32 (128 terms of O(1/len) each), the
      // tile sums added in double-float
      const int cnt = (int)min((int64_t)TILE, ce - t0);
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
  if (act) reinterpret_cast<float2*>(partials)[(int64_t)threadIdx.x * G + blockIdx.x] = make_float2(acc.hi, acc.lo);
}

__global__ void __launch_bounds__(kNT) k_gram_reduce_f(const double* __restrict__ partials, int G, int P,
                                                       double* __restrict__ out, const LanczosFlags* fl) {
  if (cta_gate(threadIdx.x == 0 && stopped(fl))) return;
  __shared__ float hh[1024], hl[1024];
  for (int j0 = 0; j0 < P; j0 += 1024) {
    const int mm = min(1024, P - j0);
    sum_partials_many_df<kNT>(reinterpret_cast<const float2*>(partials) + (int64_t)j0 * G, G, mm, hh, hl);
    for (int j = threadIdx.x; j < mm; j += kNT) out[j0 + j] = (double)hh[j] + (double)hl[j];
    __syncthreads();
  }
}

// Gram matrix of U (upper triangle, packed row by row) and U_k·v_last.
// Entry order: pairs (k,l) with k <= l in row-major order, then g_k.
// FP64 for FP64 vectors; for FP32 vectors FP64 (F64, the FP32-mixed form) or
// double-float (the double-float form when ls exceeds the register kernels).
template <class TX, bool F64>
__global__ void __launch_bounds__(kNT) k_gram(const TX* __restrict__ U, const TX* __restrict__ vl, int ls,
                                              int64_t len, double* __restrict__ partials, int G,
                                              const LanczosFlags* __restrict__ fl) {
  if (stopped(fl)) return;
  constexpr int TILE = 64;
  constexpr int TS = TILE + 1;  // padded row: the 32 lanes of a warp read 32 different rows
  extern __shared__ double tile[];  // (ls+1) x TS of TX
  TX* tl = reinterpret_cast<TX*>(tile);
  const int P = ls * (ls + 1) / 2 + ls;
  int64_t cb, ce;
  chunk_of(len, G, cb, ce);
  double acc[8] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
  DFAcc dacc[8];
#pragma unroll
  for (int q = 0; q < 8; ++q) dacc[q].init();
  for (int64_t t0 = cb; t0 < ce; t0 += TILE) {
    const int cnt = (int)min((int64_t)TILE, ce - t0);
    for (int idx = threadIdx.x; idx < (ls + 1) * TILE; idx += kNT) {
      int j = idx / TILE, x = idx % TILE;
      TX val = (TX)0;
      if (x < cnt) val = (j < ls) ? U[(int64_t)j * len + t0 + x] : vl[t0 + x];
      tl[j * TS + x] = val;
    }
    __syncthreads();
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      int pr = threadIdx.x + q * kNT;
      if (pr >= P) break;
      int k, l;
      gram_pair(pr, ls, k, l);
      if constexpr (sizeof(TX) == 4 && !F64) {
        for (int x = 0; x < cnt; ++x) dacc[q].add_prod(tl[k * TS + x], tl[l * TS + x]);
      } else {
        // (the product of two FP32 numbers is exact in FP64)
        double s = acc[q];
        for (int x = 0; x < cnt; ++x) s = fma(widen(tl[k * TS + x]), widen(tl[l * TS + x]), s);
        acc[q] = s;
      }
    }
    __syncthreads();
  }
#pragma unroll
  for (int q = 0; q < 8; ++q) {
    int pr = threadIdx.x + q * kNT;
    if (pr < P) partials[(int64_t)pr * G + blockIdx.x] = (sizeof(TX) == 4 && !F64) ? dacc[q].get() : acc[q];
  }
}

__global__ void __launch_bounds__(kNT) k_gram_reduce(const double* __restrict__ partials, int G, int P,
                                                     double* __restrict__ out, const LanczosFlags* fl) {
  if (stopped(fl)) return;
  __shared__ double res[1024];
  for (int j0 = 0; j0 < P; j0 += 1024) {
    const int mm = min(1024, P - j0);
    sum_partials_many<kNT>(partials + (int64_t)j0 * G, G, mm, res);
    for (int j = threadIdx.x; j < mm; j += kNT) out[j0 + j] = res[j];
    __syncthreads();
  }
}

// Cholesky G = RᵀR, X = R⁻¹ (upper), c = Xᵀ g.  Single thread (ls is small).
__global__ void k_chol(const double* __restrict__ gram, int ls, double* X, double* cvec, LanczosFlags* fl) {
  if (stopped(fl) || threadIdx.x != 0) return;
  extern __shared__ double R[];  // ls x ls, column-major
  auto G = [&](int k, int l) {  // k <= l
    int off = 0;
    for (int r = 0; r < k; ++r) off += ls - r;
    return gram[off + (l - k)];
  };
  for (int j = 0; j < ls; ++j) {
    for (int i = 0; i <= j; ++i) {
      double s = G(i, j);
      for (int k = 0; k < i; ++k) s -= R[j * ls + k] * R[i * ls + k];
      if (i == j) {
        if (!(s > 0.0)) { fl->bad = 1; s = 1e-300; }
        R[j * ls + j] = sqrt(s);
      } else {
        R[j * ls + i] = s / R[i * ls + i];
      }
    }
  }
  for (int j = 0; j < ls; ++j) {
    for (int i = ls - 1; i >= 0; --i) {
      double s = (i == j) ? 1.0 : 0.0;
      for (int k = i + 1; k <= j; ++k) s -= R[k * ls + i] * X[j * ls + k];
      X[j * ls + i] = (i <= j) ? s / R[i * ls + i] : 0.0;
    }
  }
  const int gofs = ls * (ls + 1) / 2;
  for (int k = 0; k < ls; ++k) {
    double s = 0.0;
    for (int j = 0; j <= k; ++j) s += X[k * ls + j] * gram[gofs + j];
    cvec[k] = s;
  }
}

// The same Cholesky and inverse in double-float on one warp (chol_df_warp).
__global__ void __launch_bounds__(32) k_chol_df(const double* __restrict__ gram, int ls, double* X, double* cvec,
                                                LanczosFlags* fl) {
  if (stopped(fl)) return;  // one warp: every lane reads the same flags
  const bool bad = chol_df_warp(
      ls, [&](int idx) { return gram[idx]; }, [&](int j, int i, double x) { X[j * ls + i] = x; },
      [&](int k, double c) { cvec[k] = c; });
  if (threadIdx.x == 0 && bad) fl->bad = 1;
}

// V_k = Σ_{j<=k} X[j,k] U_j (k < ls);  V_ls = V_{lm-1} - Σ_k c_k V_k.
// FP64 sums, except for FP32 vectors with !F64 (the double-float form when ls
// exceeds the register kernels): FP32 products with Kahan sums.
template <class TX, bool F64>
__global__ void __launch_bounds__(kNT) k_restart_apply(const TX* __restrict__ U, TX* __restrict__ V,
                                                       const double* __restrict__ X, const double* __restrict__ cvec,
                                                       int ls, int lm, int64_t len,
                                                       const LanczosFlags* __restrict__ fl) {
  if (stopped(fl)) return;
  extern __shared__ double xs[];  // ls*ls + ls doubles, then the same as floats
  float* xf = (float*)(xs + ls * ls + ls);
  for (int idx = threadIdx.x; idx < ls * ls; idx += kNT) {
    xs[idx] = X[idx];
    xf[idx] = (float)X[idx];
  }
  for (int idx = threadIdx.x; idx < ls; idx += kNT) {
    xs[ls * ls + idx] = cvec[idx];
    xf[ls * ls + idx] = (float)cvec[idx];
  }
  __syncthreads();
  for (int64_t i = blockIdx.x * (int64_t)kNT + threadIdx.x; i < len; i += (int64_t)gridDim.x * kNT) {
    if constexpr (sizeof(TX) == 4 && !F64) {
      // X is the identity up to O(1e-7); FP32 products, Kahan sums
      KahanF last;
      last.init();
      last.add((float)V[(int64_t)(lm - 1) * len + i]);
      for (int k = 0; k < ls; ++k) {
        KahanF q;
        q.init();
        for (int j = 0; j <= k; ++j) q.add(__fmul_rn(xf[k * ls + j], (float)U[(int64_t)j * len + i]));
        const float qv = q.get();
        V[(int64_t)k * len + i] = (TX)qv;
        last.add(__fmul_rn(-xf[ls * ls + k], qv));
      }
      V[(int64_t)ls * len + i] = (TX)last.get();
    } else {
      double last = widen(V[(int64_t)(lm - 1) * len + i]);
      for (int k = 0; k < ls; ++k) {
        double q = 0.0;
        for (int j = 0; j <= k; ++j) q = fma(xs[k * ls + j], widen(U[(int64_t)j * len + i]), q);
        V[(int64_t)k * len + i] = (TX)q;
        last = fma(-xs[ls * ls + k], q, last);
      }
      V[(int64_t)ls * len + i] = (TX)last;
    }
  }
}

// R_e = Σ_{k<elit} Y[k,e] V_k  (shellmodel_main.jl:210-214), FP64.
template <class TX>
__global__ void __launch_bounds__(kNT) k_ritz(const TX* __restrict__ V, const double* __restrict__ Y, int elit,
                                              int nev, double* __restrict__ R, int64_t len) {
  for (int64_t i = blockIdx.x * (int64_t)kNT + threadIdx.x; i < len; i += (int64_t)gridDim.x * kNT) {
    for (int e = 0; e < nev; ++e) {
      double s = 0.0;
      for (int k = 0; k < elit; ++k) s = fma(Y[(int64_t)e * elit + k], (double)V[(int64_t)k * len + i], s);
      R[(int64_t)e * len + i] = s;
    }
  }
}

// ---------------------------------------------------------------------------
// Vector helpers of the J-projected Lanczos (lanczos_methods.jl:93-151).
template <class TX>
__global__ void __launch_bounds__(kNT) k_widen(const TX* __restrict__ in, double* __restrict__ out, int64_t len) {
  for (int64_t i = blockIdx.x * (int64_t)kNT + threadIdx.x; i < len; i += (int64_t)gridDim.x * kNT)
    out[i] = (double)in[i];
}
template <class TX>
__global__ void __launch_bounds__(kNT) k_narrow(const double* __restrict__ in, TX* __restrict__ out, int64_t len) {
  for (int64_t i = blockIdx.x * (int64_t)kNT + threadIdx.x; i < len; i += (int64_t)gridDim.x * kNT)
    out[i] = (TX)in[i];
}
// y -= Σ_{j<m} h_j X_j  (h on the device)
template <class TX>
__global__ void __launch_bounds__(kNT) k_axpy_dev(const TX* __restrict__ X, int64_t ld, int m,
                                                  const double* __restrict__ h, double* __restrict__ y, int64_t len) {
  for (int64_t i = blockIdx.x * (int64_t)kNT + threadIdx.x; i < len; i += (int64_t)gridDim.x * kNT) {
    double t = y[i];
    for (int j = 0; j < m; ++j) t = fma(-h[j], (double)X[(int64_t)j * ld + i], t);
    y[i] = t;
  }
}
// out = Σ_{j<m} c_j Q_j  (c on the device, column stride cst)
__global__ void __launch_bounds__(kNT) k_combine(const double* __restrict__ Q, int64_t ld, int m,
                                                 const double* __restrict__ c, double* __restrict__ out,
                                                 int64_t len) {
  for (int64_t i = blockIdx.x * (int64_t)kNT + threadIdx.x; i < len; i += (int64_t)gridDim.x * kNT) {
    double t = 0.0;
    for (int j = 0; j < m; ++j) t = fma(c[j], Q[(int64_t)j * ld + i], t);
    out[i] = t;
  }
}

// Eigen-decomposition of a small symmetric matrix in device memory (column-
// major n x n, ld n): one CTA of parallel Jacobi.
__global__ void __launch_bounds__(256) k_small_eig(const double* __restrict__ T, int n, double* A, double* Z,
                                                   double* evals) {
  jacobi_eig<256>(T, n, n, A, Z, evals);
}

inline int grid_for(int64_t len) {
  int64_t g = (len + kNT - 1) / kNT;
  if (g > 152 * 8) g = 152 * 8;
  if (g < 1) g = 1;
  return (int)g;
}
}  // namespace

// ------------------------------------------------------------------ launchers
void launch_convert(const double* a, float* b, int64_t len, cudaStream_t st) {
  k_convert<<<grid_for(len), kNT, 0, st>>>(a, b, len);
}
void launch_start_vector(const DevTables& t, uint64_t seed, double* w, cudaStream_t st) {
  k_start_vector<<<grid_for(t.len_pad), kNT, 0, st>>>(t, seed, w);
}
template <class TX>
void launch_to_padded(const DevTables& t, const double* src, TX* dst, cudaStream_t st) {
  k_to_padded<TX><<<grid_for(t.len_pad), kNT, 0, st>>>(t, src, dst);
}
void launch_from_padded(const DevTables& t, const double* src, double* dst, cudaStream_t st) {
  k_from_padded<<<grid_for(t.len_pad), kNT, 0, st>>>(t, src, dst);
}
template <class TX>
void launch_multidot(const LanczosDev& L, const TX* X, int m, const double* y, bool self, cudaStream_t st) {
  k_multidot<TX><<<L.G, kNT, 0, st>>>(X, L.len, m, y, L.len, self ? 1 : 0, L.partials, L.G);
}
void launch_reduce(const LanczosDev& L, int m, ReduceMode mode, double* out, cudaStream_t st) {
  k_reduce<<<1, kNT, 0, st>>>(L.partials, L.G, m, (int)mode, out);
}
template <class TX>
void launch_scale_store(const LanczosDev& L, const double* w, TX* out, const double* scale, cudaStream_t st) {
  k_scale_store<TX><<<grid_for(L.len), kNT, 0, st>>>(w, out, scale, L.len);
}
template <class TX>
void launch_orth_iteration(const LanczosDev& L, TX* V, double* w, int it0, cudaStream_t st) {
  const int m = it0 + 1;
  const size_t hsh = sizeof(double) * (size_t)m;
  k_orth_dot<TX><<<L.G, kNT, 0, st>>>(V, L.len, it0, w, L.alpha_part, L.nalpha, L.pdot, L.G, L.fl);
  k_orth_axpy<TX><<<L.G, kNT, hsh, st>>>(V, L.len, it0, w, L.pdot, L.pn1, L.G, V + (int64_t)(it0 + 1) * L.len, L.T,
                                         L.lm, L.sc, L.fl, L.fastnorm);
  k_orth_dot2<TX><<<L.G, kNT, 0, st>>>(V, L.len, it0, w, L.pdot, L.pn1, L.pdot2, L.G, L.fl);
  k_orth_axpy2<TX><<<L.G, kNT, hsh, st>>>(V, L.len, it0, w, L.pdot, L.pn1, L.pdot2, L.pn2, L.G, L.fl);
  k_orth_scale<TX><<<L.G, kNT, 0, st>>>(w, V + (int64_t)(it0 + 1) * L.len, L.pdot, L.pn1, L.pn2, L.G, it0, L.T,
                                        L.lm, L.len, L.sc, L.fl);
}
void launch_orth_iteration_df(const LanczosDev& L, float* V, float* wh, float* wl, int it0, cudaStream_t st) {
  const int m = it0 + 1;
  const size_t hsh = sizeof(double) * (size_t)(m + 2) + 2 * sizeof(float) * (size_t)m;  // h_j, their FP32 splits
  // one wave of two CTAs per SM, less one SM: the eigenvalue test running
  // beside them finds room without delaying a CTA to a second wave
  const int G = L.G > 4 ? L.G - 2 : L.G;
  k_orth_dot_df<<<G, kONT, 0, st>>>(V, L.len, it0, wh, wl, L.alpha_part, L.nalpha, L.pdot, G, L.fl);
  k_orth_axpy_df<<<G, kONT, hsh, st>>>(V, L.len, it0, wh, wl, L.pdot, L.pn1, G, L.sc, L.fl);
  k_orth_dot2_df<<<G, kONT, 0, st>>>(V, L.len, it0, wh, wl, L.sc, L.pn1, L.pdot2, G, L.fl);
  k_orth_axpy2_df<<<G, kONT, hsh, st>>>(V, L.len, it0, wh, wl, L.sc, L.pn1, L.pdot2, L.pn2, G, L.fl);
  k_orth_scale_df<<<G, kONT, 0, st>>>(wh, wl, V + (int64_t)(it0 + 1) * L.len, L.pn1, L.pn2, G, it0, L.T, L.lm,
                                      L.len, L.sc, L.fl);
}
void launch_sturm(const LanczosDev& L, int it, int lock, cudaStream_t st) {
  int threads = ((L.num_ev * kLPE + 31) / 32) * 32;
  if (threads > 1024) threads = 1024;
  if (threads < 32) threads = 32;
  size_t shm = sizeof(double) * (3 * (size_t)L.lm + L.num_ev);
  k_sturm<<<1, threads, shm, st>>>(L.T, L.lm, it, lock, L.num_ev, L.en, L.nh, L.tol, L.mdim, L.alpha_part, L.nalpha,
                                   L.alpha_df, L.fl);
}
void launch_jacobi(const LanczosDev& L, int n, bool gate_on_done, bool df, bool refined, cudaStream_t st) {
  const size_t shm = jacobi_smem_bytes(n);
  if (df && n <= kJacobiSmemN)
    k_jacobi_df<256><<<1, 256, shm, st>>>(L.T, L.lm, n, L.jacA, L.evals, L.fl, gate_on_done ? 1 : 0);
  else if (refined && n <= kJacobiRefineN)
    k_jacobi_refined<256><<<1, 256, jacobi_refined_smem_bytes(n), st>>>(L.T, L.lm, n, L.jacA, L.evals, L.fl,
                                                                       gate_on_done ? 1 : 0);
  else
    k_jacobi<256><<<1, 256, shm, st>>>(L.T, L.lm, n, L.jacA, L.jacZ, L.evals, L.fl, gate_on_done ? 1 : 0);
}
void launch_restart_small(const LanczosDev& L, cudaStream_t st) {
  k_restart_small<<<1, 256, 0, st>>>(L.T, L.lm, L.ls, L.evals, L.jacA, L.Yf, L.fl);
}
template <class TX>
void launch_restart_rotate(const LanczosDev& L, const TX* V, TX* U, cudaStream_t st) {
  int m = L.lm - 1;
  if constexpr (sizeof(TX) == 4) {
    if (L.ls <= kRLS && sizeof(float) * (size_t)m * kRLS <= 48 * 1024) {
      k_restart_rotate_f<<<grid_for(L.len), kNT, sizeof(float) * m * kRLS, st>>>(V, U, L.Yf, m, L.ls, L.len, L.fl);
      return;
    }
  }
  k_restart_rotate<TX><<<grid_for(L.len), kNT, 0, st>>>(V, U, L.jacA, L.Yf, m, L.ls, L.len, L.fl);
}
template <class TX>
void launch_gram(const LanczosDev& L, const TX* U, const TX* vlast, bool df, cudaStream_t st) {
  if constexpr (sizeof(TX) == 4) {
    if (df && L.ls <= kRLS && L.ls * (L.ls + 1) / 2 + L.ls <= kNT) {
      k_gram_f<<<L.G, kNT, sizeof(float) * 2 * (L.ls + 1) * 129, st>>>(U, vlast, L.ls, L.len, L.partials, L.G, L.fl);
      return;
    }
    if (df) {
      k_gram<TX, false><<<L.G, kNT, sizeof(double) * (L.ls + 1) * 65, st>>>(U, vlast, L.ls, L.len, L.partials, L.G,
                                                                            L.fl);
      return;
    }
  }
  k_gram<TX, true><<<L.G, kNT, sizeof(double) * (L.ls + 1) * 65, st>>>(U, vlast, L.ls, L.len, L.partials, L.G, L.fl);
}
void launch_gram_reduce(const LanczosDev& L, bool df, cudaStream_t st) {
  const int P = L.ls * (L.ls + 1) / 2 + L.ls;
  if (df && L.ls <= kRLS && P <= kNT) k_gram_reduce_f<<<1, kNT, 0, st>>>(L.partials, L.G, P, L.gram, L.fl);
  else k_gram_reduce<<<1, kNT, 0, st>>>(L.partials, L.G, P, L.gram, L.fl);
}
void launch_chol(const LanczosDev& L, bool df, cudaStream_t st) {
  if (df && L.ls <= 32) k_chol_df<<<1, 32, 0, st>>>(L.gram, L.ls, L.X, L.cvec, L.fl);
  else k_chol<<<1, 32, sizeof(double) * L.ls * L.ls, st>>>(L.gram, L.ls, L.X, L.cvec, L.fl);
}
template <class TX>
void launch_restart_apply(const LanczosDev& L, const TX* U, TX* V, bool df, cudaStream_t st) {
  const size_t shm = (sizeof(double) + sizeof(float)) * (L.ls * L.ls + L.ls);
  if constexpr (sizeof(TX) == 4) {
    if (df && L.ls <= kRLS) {
      k_restart_apply_f<<<grid_for(L.len), kNT, 0, st>>>(U, V, L.X, L.cvec, L.ls, L.lm, L.len, L.fl);
      return;
    }
    if (df) {
      k_restart_apply<TX, false><<<grid_for(L.len), kNT, shm, st>>>(U, V, L.X, L.cvec, L.ls, L.lm, L.len, L.fl);
      return;
    }
  }
  k_restart_apply<TX, true><<<grid_for(L.len), kNT, shm, st>>>(U, V, L.X, L.cvec, L.ls, L.lm, L.len, L.fl);
}
template <class TX>
void launch_ritz(const LanczosDev& L, const TX* V, int elit, int nev, double* R, cudaStream_t st) {
  k_ritz<TX><<<grid_for(L.len), kNT, 0, st>>>(V, L.jacA, elit, nev, R, L.len);
}

template <class TX>
void launch_widen(const TX* in, double* out, int64_t len, cudaStream_t st) {
  k_widen<TX><<<grid_for(len), kNT, 0, st>>>(in, out, len);
}
template <class TX>
void launch_narrow(const double* in, TX* out, int64_t len, cudaStream_t st) {
  k_narrow<TX><<<grid_for(len), kNT, 0, st>>>(in, out, len);
}
template <class TX>
void launch_axpy_dev(const TX* X, int64_t ld, int m, const double* h, double* y, int64_t len, cudaStream_t st) {
  k_axpy_dev<TX><<<grid_for(len), kNT, 0, st>>>(X, ld, m, h, y, len);
}
void launch_combine(const double* Q, int64_t ld, int m, const double* c, double* out, int64_t len, cudaStream_t st) {
  k_combine<<<grid_for(len), kNT, 0, st>>>(Q, ld, m, c, out, len);
}
void launch_small_eig(const double* T, int n, double* A, double* Z, double* evals, cudaStream_t st) {
  const size_t shm = jacobi_smem_bytes(n);
  k_small_eig<<<1, 256, shm, st>>>(T, n, A, Z, evals);
}

#define SMGPU_INST(TX)                                                                                       \
  template void launch_to_padded<TX>(const DevTables&, const double*, TX*, cudaStream_t);                    \
  template void launch_multidot<TX>(const LanczosDev&, const TX*, int, const double*, bool, cudaStream_t);   \
  template void launch_scale_store<TX>(const LanczosDev&, const double*, TX*, const double*, cudaStream_t);   \
  template void launch_orth_iteration<TX>(const LanczosDev&, TX*, double*, int, cudaStream_t);               \
  template void launch_restart_rotate<TX>(const LanczosDev&, const TX*, TX*, cudaStream_t);                  \
  template void launch_gram<TX>(const LanczosDev&, const TX*, const TX*, bool, cudaStream_t);                \
  template void launch_restart_apply<TX>(const LanczosDev&, const TX*, TX*, bool, cudaStream_t);             \
  template void launch_ritz<TX>(const LanczosDev&, const TX*, int, int, double*, cudaStream_t);               \
  template void launch_widen<TX>(const TX*, double*, int64_t, cudaStream_t);                                 \
  template void launch_narrow<TX>(const double*, TX*, int64_t, cudaStream_t);                                \
  template void launch_axpy_dev<TX>(const TX*, int64_t, int, const double*, double*, int64_t, cudaStream_t);
SMGPU_INST(double)
SMGPU_INST(float)
#undef SMGPU_INST

}  // namespace smgpu
