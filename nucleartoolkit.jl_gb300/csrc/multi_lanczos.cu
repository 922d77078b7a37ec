// Multi-sample thick-restart Lanczos kernels (multi.cuh).  Per sample the
// algorithm is that of lanczos.cu — TRL (src/ShellModel/lanczos_methods.jl:
// 1-91), diagonalize_T! (:250-258), ThickRestart (:260-307), the Ritz vectors
// (shellmodel_main.jl:208-224) — run for S samples at once, the way prepEC
// (src/ShellModel/eigenvector_continuation.jl:140-177) runs TRL once per
// interaction sample on a shared basis.
//
// Layout: Krylov vectors are FP32, interleaved sample-innermost (slot j,
// row i, sample s at V[j*len*S + i*S + s]); w is FP64 in the same layout.
// Streaming kernels give each thread four consecutive samples of one row
// (one 16-byte load per vector), so all S samples of a row are read with
// S/4 coalesced loads.  Reductions: per-CTA partials per (slot, sample),
// then one warp per sum in a separate small kernel; all orders are fixed,
// so the results are deterministic.
//
// Gating: every kernel returns when all samples have converged
// (MultiCtl::all_done); per-sample work is skipped for samples whose flags
// say done/exhausted, so a converged sample's basis and T stay as they were
// when it converged.
#include "lanczos_dev.cuh"
#include "multi.cuh"

namespace smgpu {

namespace {
using namespace dev;

__device__ __forceinline__ bool lane_stopped(const LanczosFlags* fl, int s) { return fl[s].done || fl[s].exhausted; }

__device__ __forceinline__ void lane_finished(MultiCtl* ctl, int S) {
  if (atomicAdd(&ctl->ndone, 1) == S - 1) atomicExch(&ctl->all_done, 1);
}

inline int grid_for(int64_t n) {
  int64_t g = (n + kNT - 1) / kNT;
  if (g > 152 * 8) g = 152 * 8;
  if (g < 1) g = 1;
  return (int)g;
}

// Reduce acc[q][u] (slot q, sample 4*(tid%Q)+u) over the CTA and write
// part[((slot0+q)*S + s)*G + cta] for q < nq.  red: (kNT/32)*NQ*S doubles.
template <int S, int NQ>
__device__ __forceinline__ void reduce_slots(double (&acc)[NQ][4], int nq, double* red, double* __restrict__ part,
                                             int slot0, int G) {
  constexpr int Q = S / 4;
#pragma unroll
  for (int q = 0; q < NQ; ++q)
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      double x = acc[q][u];
#pragma unroll
      for (int o = Q; o < 32; o <<= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
      acc[q][u] = x;
    }
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  __syncthreads();
  if (lane < Q) {
#pragma unroll
    for (int q = 0; q < NQ; ++q)
#pragma unroll
      for (int u = 0; u < 4; ++u) red[(wid * NQ + q) * S + 4 * lane + u] = acc[q][u];
  }
  __syncthreads();
  for (int c = threadIdx.x; c < nq * S; c += kNT) {
    const int q = c / S, s = c % S;
    double x = 0.0;
    for (int w = 0; w < kNT / 32; ++w) x += red[(w * NQ + q) * S + s];
    part[((int64_t)(slot0 + q) * S + s) * G + blockIdx.x] = x;
  }
}

// reduce_slots for double-float accumulators: shuffles in double-float on the
// FP32 pipe, FP64 only for the per-warp totals.
template <int S, int NQ>
__device__ __forceinline__ void reduce_slots_df(DFAcc (&acc)[NQ][4], int nq, double* red, double* __restrict__ part,
                                                int slot0, int G) {
  constexpr int Q = S / 4;
#pragma unroll
  for (int q = 0; q < NQ; ++q)
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      float h = acc[q][u].hi, l = acc[q][u].lo;
#pragma unroll
      for (int o = Q; o < 32; o <<= 1) {
        const float oh = __shfl_xor_sync(0xffffffffu, h, o);
        const float ol = __shfl_xor_sync(0xffffffffu, l, o);
        df_add(h, l, oh, ol);
      }
      acc[q][u].hi = h;
      acc[q][u].lo = l;
    }
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  __syncthreads();
  if (lane < Q) {
#pragma unroll
    for (int q = 0; q < NQ; ++q)
#pragma unroll
      for (int u = 0; u < 4; ++u) red[(wid * NQ + q) * S + 4 * lane + u] = acc[q][u].get();
  }
  __syncthreads();
  for (int c = threadIdx.x; c < nq * S; c += kNT) {
    const int q = c / S, s = c % S;
    double x = 0.0;
    for (int w = 0; w < kNT / 32; ++w) x += red[(w * NQ + q) * S + s];
    part[((int64_t)(slot0 + q) * S + s) * G + blockIdx.x] = x;
  }
}

// ------------------------------------------------------------------ vectors
__global__ void k_m_start(DevTables t, int S, uint64_t seed, double* __restrict__ w) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < t.len_pad;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int b = find_block(t.off_pad, t.nb, i);
    const int64_t loc = i - t.off_pad[b];
    const int st = t.stride[b];
    const int p = (int)(loc / st), n = (int)(loc % st);
    const double x = (n < t.nn[b]) ? start_elem(seed, t.tdims[b] + (int64_t)p * t.nn[b] + n) : 0.0;
    for (int s = 0; s < S; ++s) w[i * S + s] = x;
  }
}

// src: S vectors of mdim (sample-major, unpadded) -> interleaved padded
template <class TX>
__global__ void k_m_to_padded(DevTables t, int S, const double* __restrict__ src, TX* __restrict__ dst) {
  const int64_t mdim = t.tdims[t.nb];
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < t.len_pad;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int b = find_block(t.off_pad, t.nb, i);
    const int64_t loc = i - t.off_pad[b];
    const int st = t.stride[b];
    const int p = (int)(loc / st), n = (int)(loc % st);
    const bool in = n < t.nn[b];
    const int64_t g = t.tdims[b] + (int64_t)p * t.nn[b] + n;
    for (int s = 0; s < S; ++s) dst[i * S + s] = in ? (TX)src[(int64_t)s * mdim + g] : (TX)0;
  }
}

__global__ void k_m_from_padded(DevTables t, int S, const double* __restrict__ w, double* __restrict__ dst) {
  const int64_t mdim = t.tdims[t.nb];
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < t.len_pad;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int b = find_block(t.off_pad, t.nb, i);
    const int64_t loc = i - t.off_pad[b];
    const int st = t.stride[b];
    const int p = (int)(loc / st), n = (int)(loc % st);
    if (n >= t.nn[b]) continue;
    const int64_t g = t.tdims[b] + (int64_t)p * t.nn[b] + n;
    for (int s = 0; s < S; ++s) dst[(int64_t)s * mdim + g] = w[i * S + s];
  }
}

// part[s*G + cta] = ||w_s chunk||²
template <int S>
__global__ void __launch_bounds__(kNT) k_m_selfdot(const double* __restrict__ w, int64_t len, double* part, int G) {
  constexpr int Q = S / 4, RPP = kNT / Q;
  __shared__ double red[(kNT / 32) * S];
  const int q = threadIdx.x % Q, r = threadIdx.x / Q;
  int64_t cb, ce;
  chunk_of(len, G, cb, ce);
  double acc[1][4] = {{0.0, 0.0, 0.0, 0.0}};
  for (int64_t i = cb + r; i < ce; i += RPP) {
    double x[4];
    load4(w + i * S + 4 * q, x);
#pragma unroll
    for (int u = 0; u < 4; ++u) acc[0][u] = fma(x[u], x[u], acc[0][u]);
  }
  reduce_slots<S, 1>(acc, 1, red, part, 0, G);
}

template <int S>
__global__ void __launch_bounds__(kNT) k_m_scale_init(const double* __restrict__ w, float* __restrict__ v,
                                                      const double* __restrict__ nrm, int64_t len) {
  const int64_t n = len * S;
  for (int64_t e = blockIdx.x * (int64_t)kNT + threadIdx.x; e < n; e += (int64_t)gridDim.x * kNT) {
    const double inv = 1.0 / sqrt(nrm[e % S]);
    v[e] = (float)(w[e] * inv);
  }
}

// out[c] = Σ_g part[c*G + g], one warp per c.  gate: 0 none, 1 all_done,
// 2 all_done or no second pass.
__global__ void __launch_bounds__(kNT) k_m_reduce(const double* __restrict__ part, int G, int count,
                                                  double* __restrict__ out, const MultiCtl* ctl, int gate) {
  if (gate >= 1 && ctl->all_done) return;
  if (gate == 2 && !ctl->any_second) return;
  const int c = (int)((blockIdx.x * (int64_t)kNT + threadIdx.x) >> 5);
  const int lane = threadIdx.x & 31;
  if (c >= count) return;
  double x = 0.0;
  for (int g = lane; g < G; g += 32) x += part[(int64_t)c * G + g];
  x = warp_sum(x);
  if (lane == 0) out[c] = x;
}

// ------------------------------------------------------------ one iteration
// α_s = Σ partials of the H·V epilogue -> T_s[it0][it0]
__global__ void k_m_alpha(const double* __restrict__ alpha_part, int nalpha, double* T, int lm, int it0,
                          const LanczosFlags* fl, const MultiCtl* ctl) {
  const int s = blockIdx.x;
  if (cta_gate(threadIdx.x == 0 && (ctl->all_done || lane_stopped(fl, s)))) return;
  __shared__ double red[kNT / 32];
  const double a = sum_partials<kNT>(alpha_part + (int64_t)s * nalpha, nalpha, red);
  if (threadIdx.x == 0) T[(int64_t)s * lm * lm + (int64_t)it0 * lm + it0] = a;
}

__global__ void k_m_sturm(double* T, int lm, int k, int lock, int num_ev, double* en, int nh, double tol,
                          int64_t mdim, LanczosFlags* fl, MultiCtl* ctl, int S) {
  const int s = blockIdx.x;
  LanczosFlags* f = fl + s;
  if (cta_gate(threadIdx.x == 0 && f->done)) return;
  if (cta_gate(threadIdx.x == 0 && f->exhausted && k > f->exh_k)) {
    if (threadIdx.x == 0) {
      f->done = 1;
      f->elit = f->exh_k;
      lane_finished(ctl, S);
    }
    return;
  }
  sturm_step(T + (int64_t)s * lm * lm, lm, k, lock, num_ev, en + (int64_t)s * nh * num_ev, nh, tol, mdim, f);
  if (threadIdx.x == 0 && f->done) lane_finished(ctl, S);
}

// First pass (first = 1): α_s (T diagonal), w' = w − α v_k, partials of
// V_j·w' (j <= it0) and of ||w'||² (slot it0+1); second pass (first = 0):
// partials of V_j·w (j <= it0).  w = wh + wl in double-float, interleaved as V;
// all vector arithmetic on the FP32 pipe.
template <int S>
__global__ void __launch_bounds__(kNT) k_m_dot_df(const float* __restrict__ V, int64_t len, int it0,
                                                  float* __restrict__ wh, float* __restrict__ wl,
                                                  const double* __restrict__ T, int lm, double* __restrict__ part,
                                                  int G, const LanczosFlags* fl, const MultiCtl* ctl, int first) {
  if (cta_gate(threadIdx.x == 0 && (ctl->all_done || (!first && !ctl->any_second)))) return;
  constexpr int Q = S / 4, RPP = kNT / Q;
  __shared__ double red[(kNT / 32) * 8 * S];
  const int q = threadIdx.x % Q, r = threadIdx.x / Q, s0 = 4 * q;
  const int64_t LS = len * S;
  float aH[4], aL[4];
#pragma unroll
  for (int u = 0; u < 4; ++u) {
    const double al = (first && !lane_stopped(fl, s0 + u)) ? T[(int64_t)(s0 + u) * lm * lm + (int64_t)it0 * lm + it0] : 0.0;
    df_from_double(-al, aH[u], aL[u]);
  }
  const int m = it0 + 1;
  const int mt = first ? m + 1 : m;
  const float* __restrict__ vk = V + (int64_t)it0 * LS;
  int64_t cb, ce;
  chunk_of(len, G, cb, ce);
  // FP32 per-thread sums (a thread adds a few products of one chunk per
  // sample; their rounding is far below the FP32 basis), double-float CTA sums
  for (int j0 = 0; j0 < mt; j0 += 8) {
    float acc[8][4];
#pragma unroll
    for (int q8 = 0; q8 < 8; ++q8)
#pragma unroll
      for (int u = 0; u < 4; ++u) acc[q8][u] = 0.f;
    for (int64_t i = cb + r; i < ce; i += RPP) {
      const int64_t e = i * S + s0;
      const float4 a4 = *reinterpret_cast<const float4*>(wh + e);
      const float4 b4 = *reinterpret_cast<const float4*>(wl + e);
      float h[4] = {a4.x, a4.y, a4.z, a4.w}, l[4] = {b4.x, b4.y, b4.z, b4.w};
      if (first && j0 == 0) {
        const float4 x = *reinterpret_cast<const float4*>(vk + e);
        df_fma(h[0], l[0], x.x, aH[0], aL[0]);
        df_fma(h[1], l[1], x.y, aH[1], aL[1]);
        df_fma(h[2], l[2], x.z, aH[2], aL[2]);
        df_fma(h[3], l[3], x.w, aH[3], aL[3]);
        *reinterpret_cast<float4*>(wh + e) = make_float4(h[0], h[1], h[2], h[3]);
        *reinterpret_cast<float4*>(wl + e) = make_float4(l[0], l[1], l[2], l[3]);
      }
#pragma unroll
      for (int q8 = 0; q8 < 8; ++q8) {
        const int j = j0 + q8;
        if (j < m) {
          const float4 x = *reinterpret_cast<const float4*>(V + (int64_t)j * LS + e);
          acc[q8][0] = __fmaf_rn(x.x, h[0], acc[q8][0]);
          acc[q8][1] = __fmaf_rn(x.y, h[1], acc[q8][1]);
          acc[q8][2] = __fmaf_rn(x.z, h[2], acc[q8][2]);
          acc[q8][3] = __fmaf_rn(x.w, h[3], acc[q8][3]);
        } else if (first && j == m) {
#pragma unroll
          for (int u = 0; u < 4; ++u) acc[q8][u] = __fmaf_rn(h[u], h[u], acc[q8][u]);
        }
      }
    }
    DFAcc dacc[8][4];
#pragma unroll
    for (int q8 = 0; q8 < 8; ++q8)
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        dacc[q8][u].hi = acc[q8][u];
        dacc[q8][u].lo = 0.f;
      }
    reduce_slots_df<S, 8>(dacc, min(8, mt - j0), red, part, j0, G);
  }
}

// w_s -= Σ_j h[j*S+s] V_j,s for the live samples (second pass: only those
// with sec[s]); part[s*G + cta] = ||w_s chunk||².  Double-float w, the h_j
// split once per CTA into FP32 pairs (dynamic shared memory: 2·m·S floats).
template <int S>
__global__ void __launch_bounds__(kNT) k_m_axpy_df(const float* __restrict__ V, int64_t len, int m,
                                                   float* __restrict__ wh, float* __restrict__ wl,
                                                   const double* __restrict__ h, double* __restrict__ part, int G,
                                                   const LanczosFlags* fl, const MultiCtl* ctl,
                                                   const int* __restrict__ sec) {
  if (cta_gate(threadIdx.x == 0 && (ctl->all_done || (sec != nullptr && !ctl->any_second)))) return;
  constexpr int Q = S / 4, RPP = kNT / Q;
  extern __shared__ float hsf[];  // m*S high parts, then m*S low parts
  __shared__ double red[(kNT / 32) * S];
  float* hh = hsf;
  float* hl = hsf + m * S;
  for (int c = threadIdx.x; c < m * S; c += kNT) {
    const int s = c % S;
    const bool use = !lane_stopped(fl, s) && (sec == nullptr || sec[s] != 0);
    df_from_double(use ? h[c] : 0.0, hh[c], hl[c]);
  }
  __syncthreads();
  const int q = threadIdx.x % Q, r = threadIdx.x / Q, s0 = 4 * q;
  const int64_t LS = len * S;
  int64_t cb, ce;
  chunk_of(len, G, cb, ce);
  DFAcc nrm[1][4];
#pragma unroll
  for (int u = 0; u < 4; ++u) nrm[0][u].init();
  for (int64_t i = cb + r; i < ce; i += RPP) {
    const int64_t e = i * S + s0;
    DFAcc s4[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) s4[u].init();
    for (int j = 0; j < m; ++j) {
      const float4 x = *reinterpret_cast<const float4*>(V + (int64_t)j * LS + e);
      const int c = j * S + s0;
      s4[0].add_prod2(x.x, hh[c], hl[c]);
      s4[1].add_prod2(x.y, hh[c + 1], hl[c + 1]);
      s4[2].add_prod2(x.z, hh[c + 2], hl[c + 2]);
      s4[3].add_prod2(x.w, hh[c + 3], hl[c + 3]);
    }
    const float4 a4 = *reinterpret_cast<const float4*>(wh + e);
    const float4 b4 = *reinterpret_cast<const float4*>(wl + e);
    float hv[4] = {a4.x, a4.y, a4.z, a4.w}, lv[4] = {b4.x, b4.y, b4.z, b4.w};
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      df_add(hv[u], lv[u], -s4[u].hi, -s4[u].lo);
      nrm[0][u].add_prod2(hv[u], hv[u], 2.0f * lv[u]);
    }
    *reinterpret_cast<float4*>(wh + e) = make_float4(hv[0], hv[1], hv[2], hv[3]);
    *reinterpret_cast<float4*>(wl + e) = make_float4(lv[0], lv[1], lv[2], lv[3]);
  }
  reduce_slots_df<S, 1>(nrm, 1, red, part, 0, G);
}

// Second-pass decision per sample: ||w''||² < ||w'||² / 2.
__global__ void k_m_decide(const double* __restrict__ h1, const double* __restrict__ nrm1, int m, int* sec,
                           const LanczosFlags* fl, MultiCtl* ctl, int S) {
  if (__shfl_sync(0xffffffffu, ctl->all_done, 0)) return;
  const int s = threadIdx.x;
  bool sc = false;
  if (s < S && !lane_stopped(fl, s)) sc = nrm1[s] < 0.5 * h1[(int64_t)m * S + s];
  if (s < S) sec[s] = sc ? 1 : 0;
  const unsigned any = __ballot_sync(0xffffffffu, sc);
  if (s == 0) ctl->any_second = any != 0u ? 1 : 0;
}

// β_s, T entries, 1/β_s (0 for frozen or exhausted samples).
__global__ void k_m_beta(double* T, int lm, int it0, const double* __restrict__ nrm1, const double* __restrict__ nrm2,
                         const int* __restrict__ sec, double* invb, float2* beta2, LanczosFlags* fl,
                         const MultiCtl* ctl, int S) {
  if (ctl->all_done) return;
  const int s = threadIdx.x;
  if (s >= S) return;
  LanczosFlags* f = fl + s;
  if (f->done || f->exhausted) {
    invb[s] = 0.0;
    return;
  }
  const bool second = sec[s] != 0;
  const double beta = sqrt(second ? nrm2[s] : nrm1[s]);
  const bool ok = (beta > 0.0) && (beta < INFINITY);
  double* Ts = T + (int64_t)s * lm * lm;
  if (ok) {
    Ts[(int64_t)it0 * lm + it0 + 1] = beta;
    Ts[(int64_t)(it0 + 1) * lm + it0] = beta;
    invb[s] = 1.0 / beta;
    float bh, bl;
    df_from_double(beta, bh, bl);
    beta2[s] = make_float2(bh, bl);
    f->second = second ? 1 : 0;
    if (second) f->n_second += 1;
  } else {
    f->exh_k = it0 + 1;
    f->exhausted = 1;
    invb[s] = 0.0;
  }
}

// v_{it0+1} = w / β per live sample (w = wh + wl; 1/β split per thread)
template <int S>
__global__ void __launch_bounds__(kNT) k_m_scale_df(const float* __restrict__ wh, const float* __restrict__ wl,
                                                    float* __restrict__ vnext, const double* __restrict__ invb,
                                                    int64_t len, const MultiCtl* ctl) {
  if (ctl->all_done) return;
  constexpr int Q = S / 4;
  const int64_t n4 = len * Q;
  const int64_t g0 = blockIdx.x * (int64_t)kNT + threadIdx.x;
  const int s0 = 4 * (int)(g0 % Q);  // the grid stride is a multiple of Q: fixed per thread
  float ibh[4], ibl[4];
  bool live[4], all = true;
#pragma unroll
  for (int u = 0; u < 4; ++u) {
    const double ib = invb[s0 + u];
    live[u] = ib != 0.0;
    all = all && live[u];
    df_from_double(ib, ibh[u], ibl[u]);
  }
  for (int64_t g = g0; g < n4; g += (int64_t)gridDim.x * kNT) {
    const int64_t e = 4 * g;
    const float4 a4 = *reinterpret_cast<const float4*>(wh + e);
    const float4 b4 = *reinterpret_cast<const float4*>(wl + e);
    const float h[4] = {a4.x, a4.y, a4.z, a4.w}, l[4] = {b4.x, b4.y, b4.z, b4.w};
    float y[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) y[u] = __fmaf_rn(h[u], ibh[u], __fmaf_rn(l[u], ibh[u], __fmul_rn(h[u], ibl[u])));
    if (all) {
      *reinterpret_cast<float4*>(vnext + e) = make_float4(y[0], y[1], y[2], y[3]);
    } else {
#pragma unroll
      for (int u = 0; u < 4; ++u)
        if (live[u]) vnext[e + u] = y[u];
    }
  }
}

// Samples whose Krylov space ended in the last iteration of a cycle finish here.
__global__ void k_m_cycle_end(LanczosFlags* fl, MultiCtl* ctl, int S) {
  const int s = threadIdx.x;
  if (s < S) {
    LanczosFlags* f = fl + s;
    if (!f->done && f->exhausted) {
      f->done = 1;
      f->elit = f->exh_k;
      atomicAdd(&ctl->ndone, 1);
    }
  }
  __syncwarp();
  if (s == 0 && atomicAdd(&ctl->ndone, 0) >= S) ctl->all_done = 1;
}

// ------------------------------------------------------------------ restart
__global__ void __launch_bounds__(256) k_m_jacobi(const double* __restrict__ T, int lm, int n, double* A, double* Z,
                                                  double* evals, const LanczosFlags* fl, const MultiCtl* ctl,
                                                  int gate) {
  const int s = blockIdx.x;
  if (gate && (ctl->all_done || lane_stopped(fl, s))) return;
  const int64_t o = (int64_t)s * lm * lm;
  if (n <= kJacobiSmemN) jacobi_eig_df<256>(T + o, lm, n, A + o, evals + (int64_t)s * lm);
  else jacobi_eig<256>(T + o, lm, n, A + o, Z + o, evals + (int64_t)s * lm);
}

// ThickRestart's small part (lanczos_methods.jl:261-271) per sample.
__global__ void k_m_restart_small(double* T, int lm, int ls, const double* evals, const double* vecs, float* Yf,
                                  const LanczosFlags* fl, const MultiCtl* ctl) {
  const int s = blockIdx.x;
  if (ctl->all_done || lane_stopped(fl, s)) return;
  const int m = lm - 1;
  double* Ts = T + (int64_t)s * lm * lm;
  const double* ev = evals + (int64_t)s * lm;
  const double* vs = vecs + (int64_t)s * lm * lm;
  float* yf = Yf + (int64_t)s * m * ls;
  for (int idx = threadIdx.x; idx < m * ls; idx += blockDim.x) yf[idx] = (float)vs[idx];
  __shared__ double beta;
  if (threadIdx.x == 0) beta = Ts[(int64_t)(lm - 1) * lm + (lm - 2)];
  __syncthreads();
  for (int idx = threadIdx.x; idx < lm * lm; idx += blockDim.x) Ts[idx] = 0.0;
  __syncthreads();
  for (int k = threadIdx.x; k < ls; k += blockDim.x) {
    Ts[(int64_t)k * lm + k] = ev[k];
    const double tmp = beta * vs[(int64_t)k * m + (m - 1)];
    Ts[(int64_t)k * lm + ls] = tmp;
    Ts[(int64_t)ls * lm + k] = tmp;
  }
}

// U_k,s = Σ_{j<m} Y_s[j,k] V_j,s: FP32 products, Kahan sums.  The grid
// stride is a multiple of S, so every thread stays on one sample.
template <int S>
__global__ void __launch_bounds__(kNT) k_m_rotate(const float* __restrict__ V, float* __restrict__ U,
                                                  const float* __restrict__ Yf, int m, int ls, int64_t len,
                                                  const LanczosFlags* __restrict__ fl, const MultiCtl* ctl,
                                                  int use_smem) {
  if (ctl->all_done) return;
  // 8 outputs per pass; the pass's slice of every sample's Y staged in shared
  // memory as [j][q][s] (the lanes of a warp read consecutive samples)
  // (staged when it fits, use_smem; otherwise read through L1)
  extern __shared__ float ysh[];  // m * 8 * S
  const int s = threadIdx.x % S;
  const bool live = !lane_stopped(fl, s);
  const int64_t LS = len * S;
  for (int k0 = 0; k0 < ls; k0 += 8) {
    if (use_smem) {
      __syncthreads();
      for (int idx = threadIdx.x; idx < m * 8 * S; idx += kNT) {
        const int ss = idx % S, q = (idx / S) % 8, j = idx / (8 * S);
        ysh[idx] = (k0 + q < ls) ? Yf[(int64_t)ss * m * ls + (int64_t)(k0 + q) * m + j] : 0.f;
      }
      __syncthreads();
    }
    if (!live) continue;
    const float* __restrict__ Ys = Yf + (int64_t)s * m * ls;
    for (int64_t e = blockIdx.x * (int64_t)kNT + threadIdx.x; e < LS; e += (int64_t)gridDim.x * kNT) {
      KahanF acc[8];
#pragma unroll
      for (int q = 0; q < 8; ++q) acc[q].init();
      for (int j = 0; j < m; ++j) {
        const float x = V[(int64_t)j * LS + e];
        if (use_smem) {
          const float* yj = ysh + j * 8 * S + s;
#pragma unroll
          for (int q = 0; q < 8; ++q) acc[q].add(__fmul_rn(yj[q * S], x));
        } else {
#pragma unroll
          for (int q = 0; q < 8; ++q)
            if (k0 + q < ls) acc[q].add(__fmul_rn(__ldg(Ys + (int64_t)(k0 + q) * m + j), x));
        }
      }
#pragma unroll
      for (int q = 0; q < 8; ++q)
        if (k0 + q < ls) U[(int64_t)(k0 + q) * LS + e] = acc[q].get();
    }
  }
}

// The same rotation with the basis read once: all ls <= 16 outputs of a
// thread's element in registers, compensated FMA sums, every sample's Y in
// shared memory as [j][s][16] (a thread reads its sample's row as float4s).
constexpr int kMRLS = 16;
template <int S>
__global__ void __launch_bounds__(kNT) k_m_rotate_r(const float* __restrict__ V, float* __restrict__ U,
                                                    const float* __restrict__ Yf, int m, int ls, int64_t len,
                                                    const LanczosFlags* __restrict__ fl, const MultiCtl* ctl) {
  if (cta_gate(threadIdx.x == 0 && ctl->all_done)) return;
  extern __shared__ float ysh[];  // m x S x kMRLS
  for (int idx = threadIdx.x; idx < m * S * kMRLS; idx += kNT) {
    const int k = idx % kMRLS, ss = (idx / kMRLS) % S, j = idx / (kMRLS * S);
    ysh[idx] = k < ls ? Yf[(int64_t)ss * m * ls + (int64_t)k * m + j] : 0.f;
  }
  __syncthreads();
  const int s = threadIdx.x % S;
  if (lane_stopped(fl, s)) return;
  const int64_t LS = len * S;
  for (int64_t e = blockIdx.x * (int64_t)kNT + threadIdx.x; e < LS; e += (int64_t)gridDim.x * kNT) {
    KahanF acc[kMRLS];
#pragma unroll
    for (int k = 0; k < kMRLS; ++k) acc[k].init();
    int j = 0;
    for (; j + 4 <= m; j += 4) {
      float x[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) x[u] = V[(int64_t)(j + u) * LS + e];
      // the four terms of a group summed with plain FMAs, the group sums
      // compensated (half the operations of a compensated step per term)
      const float4* y0 = reinterpret_cast<const float4*>(ysh + ((j + 0) * S + s) * kMRLS);
      const float4* y1 = reinterpret_cast<const float4*>(ysh + ((j + 1) * S + s) * kMRLS);
      const float4* y2 = reinterpret_cast<const float4*>(ysh + ((j + 2) * S + s) * kMRLS);
      const float4* y3 = reinterpret_cast<const float4*>(ysh + ((j + 3) * S + s) * kMRLS);
#pragma unroll
      for (int q = 0; q < kMRLS / 4; ++q) {
        const float4 a = y0[q], b = y1[q], c = y2[q], d = y3[q];
        acc[4 * q].add(__fmaf_rn(d.x, x[3], __fmaf_rn(c.x, x[2], __fmaf_rn(b.x, x[1], __fmul_rn(a.x, x[0])))));
        acc[4 * q + 1].add(__fmaf_rn(d.y, x[3], __fmaf_rn(c.y, x[2], __fmaf_rn(b.y, x[1], __fmul_rn(a.y, x[0])))));
        acc[4 * q + 2].add(__fmaf_rn(d.z, x[3], __fmaf_rn(c.z, x[2], __fmaf_rn(b.z, x[1], __fmul_rn(a.z, x[0])))));
        acc[4 * q + 3].add(__fmaf_rn(d.w, x[3], __fmaf_rn(c.w, x[2], __fmaf_rn(b.w, x[1], __fmul_rn(a.w, x[0])))));
      }
    }
    for (; j < m; ++j) {
      const float x = V[(int64_t)j * LS + e];
      const float4* y4 = reinterpret_cast<const float4*>(ysh + (j * S + s) * kMRLS);
#pragma unroll
      for (int q = 0; q < kMRLS / 4; ++q) {
        const float4 y = y4[q];
        acc[4 * q].add_prod(y.x, x);
        acc[4 * q + 1].add_prod(y.y, x);
        acc[4 * q + 2].add_prod(y.z, x);
        acc[4 * q + 3].add_prod(y.w, x);
      }
    }
#pragma unroll
    for (int k = 0; k < kMRLS; ++k)
      if (k < ls) U[(int64_t)k * LS + e] = acc[k].get();
  }
}

// The apply with U of a thread's element in registers and every sample's X
// in shared memory (odd row stride: the lanes' samples hit distinct banks).
template <int S>
__global__ void __launch_bounds__(kNT) k_m_apply_r(const float* __restrict__ U, float* __restrict__ V,
                                                   const float* __restrict__ Xf, int ls, int lm, int64_t len,
                                                   const LanczosFlags* __restrict__ fl, const MultiCtl* ctl) {
  if (cta_gate(threadIdx.x == 0 && ctl->all_done)) return;
  extern __shared__ float xsh[];  // S x XST
  const int XN = ls * ls + ls, XST = XN | 1;
  for (int idx = threadIdx.x; idx < S * XN; idx += kNT) {
    const int ss = idx / XN, r = idx % XN;
    xsh[ss * XST + r] = Xf[(int64_t)ss * XN + r];
  }
  __syncthreads();
  const int s = threadIdx.x % S;
  if (lane_stopped(fl, s)) return;
  const float* xf = xsh + s * XST;
  const int64_t LS = len * S;
  for (int64_t e = blockIdx.x * (int64_t)kNT + threadIdx.x; e < LS; e += (int64_t)gridDim.x * kNT) {
    float u[kMRLS];
#pragma unroll
    for (int j = 0; j < kMRLS; ++j) u[j] = j < ls ? U[(int64_t)j * LS + e] : 0.f;
    KahanF last;
    last.init();
    last.add(V[(int64_t)(lm - 1) * LS + e]);
#pragma unroll
    for (int k = 0; k < kMRLS; ++k) {
      if (k >= ls) break;
      KahanF q;
      q.init();
#pragma unroll
      for (int j = 0; j <= k; ++j) q.add_prod(xf[k * ls + j], u[j]);
      const float qv = q.get();
      V[(int64_t)k * LS + e] = qv;
      last.add_prod(-xf[ls * ls + k], qv);
    }
    V[(int64_t)ls * LS + e] = last.get();
  }
}

// Each sample's Cholesky on one warp in double-float (chol_df_warp).
__global__ void __launch_bounds__(32) k_m_chol_df(const double* __restrict__ gram, int ls, int S, double* X,
                                                  float* Xf, double* cvec, LanczosFlags* fl, const MultiCtl* ctl) {
  const int s = blockIdx.x;
  if (ctl->all_done || lane_stopped(fl, s)) return;  // one warp: uniform
  double* Xs = X + (int64_t)s * ls * ls;
  double* cs = cvec + (int64_t)s * ls;
  float* xf = Xf + (int64_t)s * (ls * ls + ls);
  const bool bad = chol_df_warp(
      ls, [&](int idx) { return gram[(int64_t)idx * S + s]; },
      [&](int j, int i, double x) {
        Xs[j * ls + i] = x;
        xf[j * ls + i] = (float)x;
      },
      [&](int k, double c) {
        cs[k] = c;
        xf[ls * ls + k] = (float)c;
      });
  if (threadIdx.x == 0 && bad) fl[s].bad = 1;
}

// Gram matrices of U_s (packed upper triangle) and U_k,s·v_last,s for every
// sample: FP32 sums per tile, double-float across tiles.  Pair order as
// k_gram; c = pair*S + s.
template <int S>
__global__ void __launch_bounds__(kNT) k_m_gram(const float* __restrict__ U, const float* __restrict__ vl, int ls,
                                                int64_t len, int tile, double* __restrict__ part, int G,
                                                const MultiCtl* ctl) {
  if (ctl->all_done) return;
  extern __shared__ float tl[];  // (ls+1) x tile x S
  const int P = ls * (ls + 1) / 2 + ls;
  const int PS = P * S;
  const int TS = tile * S;
  const int64_t LS = len * S;
  int64_t cb, ce;
  chunk_of(len, G, cb, ce);
  for (int c0 = 0; c0 < PS; c0 += 16 * kNT) {
    DFAcc dacc[16];
    int kk[16], ll[16];
#pragma unroll
    for (int q = 0; q < 16; ++q) {
      dacc[q].init();
      const int c = c0 + threadIdx.x + q * kNT;
      kk[q] = 0;
      ll[q] = 0;
      if (c < PS) gram_pair(c / S, ls, kk[q], ll[q]);
    }
    for (int64_t t0 = cb; t0 < ce; t0 += tile) {
      const int cnt = (int)min((int64_t)tile, ce - t0);
      for (int idx = threadIdx.x; idx < (ls + 1) * TS; idx += kNT) {
        const int j = idx / TS, x = idx % TS;
        float val = 0.f;
        if (x < cnt * S) val = (j < ls) ? U[(int64_t)j * LS + t0 * S + x] : vl[t0 * S + x];
        tl[idx] = val;
      }
      __syncthreads();
#pragma unroll
      for (int q = 0; q < 16; ++q) {
        const int c = c0 + threadIdx.x + q * kNT;
        if (c >= PS) break;
        const int s = c % S;
        const float* a = tl + kk[q] * TS + s;
        const float* b = tl + ll[q] * TS + s;
        // the tile's products summed in FP32, the tile sums in double-float
        float p = 0.f;
        for (int x = 0; x < cnt; ++x) p = __fmaf_rn(a[x * S], b[x * S], p);
        df_add(dacc[q].hi, dacc[q].lo, p, 0.f);
      }
      __syncthreads();
    }
#pragma unroll
    for (int q = 0; q < 16; ++q) {
      const int c = c0 + threadIdx.x + q * kNT;
      if (c < PS) part[(int64_t)c * G + blockIdx.x] = dacc[q].get();
    }
  }
}

// Cholesky of each sample's Gram matrix, X = R⁻¹, c = Xᵀ g (as k_chol), plus
// FP32 copies for the apply kernel.
__global__ void k_m_chol(const double* __restrict__ gram, int ls, int S, double* X, float* Xf, double* cvec,
                         LanczosFlags* fl, const MultiCtl* ctl) {
  const int s = blockIdx.x;
  if (ctl->all_done || lane_stopped(fl, s) || threadIdx.x != 0) return;
  extern __shared__ double R[];  // ls x ls, column-major
  double* Xs = X + (int64_t)s * ls * ls;
  double* cs = cvec + (int64_t)s * ls;
  float* xf = Xf + (int64_t)s * (ls * ls + ls);
  auto Gm = [&](int k, int l) {  // k <= l
    int off = 0;
    for (int r = 0; r < k; ++r) off += ls - r;
    return gram[(int64_t)(off + (l - k)) * S + s];
  };
  for (int j = 0; j < ls; ++j) {
    for (int i = 0; i <= j; ++i) {
      double t = Gm(i, j);
      for (int k = 0; k < i; ++k) t -= R[j * ls + k] * R[i * ls + k];
      if (i == j) {
        if (!(t > 0.0)) {
          fl[s].bad = 1;
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
      for (int k = i + 1; k <= j; ++k) t -= R[k * ls + i] * Xs[j * ls + k];
      Xs[j * ls + i] = (i <= j) ? t / R[i * ls + i] : 0.0;
    }
  }
  const int gofs = ls * (ls + 1) / 2;
  for (int k = 0; k < ls; ++k) {
    double t = 0.0;
    for (int j = 0; j <= k; ++j) t += Xs[k * ls + j] * gram[(int64_t)(gofs + j) * S + s];
    cs[k] = t;
  }
  for (int idx = 0; idx < ls * ls; ++idx) xf[idx] = (float)Xs[idx];
  for (int k = 0; k < ls; ++k) xf[ls * ls + k] = (float)cs[k];
}

// V_k,s = Σ_{j<=k} X_s[j,k] U_j,s;  V_ls,s = V_{lm-1},s − Σ_k c_k,s V_k,s
// (FP32 products, Kahan sums, as the mixed form of k_restart_apply).
template <int S>
__global__ void __launch_bounds__(kNT) k_m_apply(const float* __restrict__ U, float* __restrict__ V,
                                                 const float* __restrict__ Xf, int ls, int lm, int64_t len,
                                                 const LanczosFlags* __restrict__ fl, const MultiCtl* ctl) {
  if (ctl->all_done) return;
  const int s = threadIdx.x % S;
  if (lane_stopped(fl, s)) return;
  const float* __restrict__ xf = Xf + (int64_t)s * (ls * ls + ls);
  const int64_t LS = len * S;
  for (int64_t e = blockIdx.x * (int64_t)kNT + threadIdx.x; e < LS; e += (int64_t)gridDim.x * kNT) {
    KahanF last;
    last.init();
    last.add(V[(int64_t)(lm - 1) * LS + e]);
    for (int k = 0; k < ls; ++k) {
      KahanF q;
      q.init();
      for (int j = 0; j <= k; ++j) q.add(__fmul_rn(__ldg(xf + k * ls + j), U[(int64_t)j * LS + e]));
      const float qv = q.get();
      V[(int64_t)k * LS + e] = qv;
      last.add(__fmul_rn(-__ldg(xf + ls * ls + k), qv));
    }
    V[(int64_t)ls * LS + e] = last.get();
  }
}

// R_e = Σ_{k<elit} Y[k,e] V_k,s (sample s), FP64, padded layout.
__global__ void __launch_bounds__(kNT) k_m_ritz(const float* __restrict__ V, int64_t len, int S, int s,
                                                const double* __restrict__ Y, int elit, int nev,
                                                double* __restrict__ R) {
  const int64_t LS = len * S;
  for (int64_t i = blockIdx.x * (int64_t)kNT + threadIdx.x; i < len; i += (int64_t)gridDim.x * kNT) {
    for (int e = 0; e < nev; ++e) {
      double t = 0.0;
      for (int k = 0; k < elit; ++k) t = fma(Y[(int64_t)e * elit + k], (double)V[(int64_t)k * LS + i * S + s], t);
      R[(int64_t)e * len + i] = t;
    }
  }
}

size_t jacobi_smem(int n) { return jacobi_smem_bytes(n); }

int gram_tile(int ls, int S) {
  int t = (int)(48 * 1024 / ((size_t)(ls + 1) * S * sizeof(float)));
  return t > 32 ? 32 : (t < 1 ? 1 : t);
}

#define SMGPU_S_DISPATCH(S, CALL)            \
  switch (S) {                               \
    case 4: { constexpr int SS = 4; CALL; } break;   \
    case 8: { constexpr int SS = 8; CALL; } break;   \
    case 16: { constexpr int SS = 16; CALL; } break; \
    default: break;                          \
  }
}  // namespace

// ------------------------------------------------------------------ launchers
void launch_m_start(int S, const DevTables& t, uint64_t seed, double* w, cudaStream_t st) {
  k_m_start<<<grid_for(t.len_pad), kNT, 0, st>>>(t, S, seed, w);
}
void launch_m_to_padded(int S, const DevTables& t, const double* src, double* w, cudaStream_t st) {
  k_m_to_padded<double><<<grid_for(t.len_pad), kNT, 0, st>>>(t, S, src, w);
}
void launch_m_to_padded_f(int S, const DevTables& t, const double* src, float* v, cudaStream_t st) {
  k_m_to_padded<float><<<grid_for(t.len_pad), kNT, 0, st>>>(t, S, src, v);
}
void launch_m_from_padded(int S, const DevTables& t, const double* w, double* dst, cudaStream_t st) {
  k_m_from_padded<<<grid_for(t.len_pad), kNT, 0, st>>>(t, S, w, dst);
}

void launch_m_init(const MultiDev& M, const double* w, float* V0, cudaStream_t st) {
  SMGPU_S_DISPATCH(M.S, (k_m_selfdot<SS><<<M.G, kNT, 0, st>>>(w, M.len, M.part, M.G)));
  k_m_reduce<<<(M.S * 32 + kNT - 1) / kNT, kNT, 0, st>>>(M.part, M.G, M.S, M.nrm1, M.ctl, 0);
  SMGPU_S_DISPATCH(M.S, (k_m_scale_init<SS><<<grid_for(M.len * M.S), kNT, 0, st>>>(w, V0, M.nrm1, M.len)));
}

void launch_m_alpha(const MultiDev& M, int it0, cudaStream_t st) {
  k_m_alpha<<<M.S, kNT, 0, st>>>(M.alpha_part + (int64_t)it0 * M.S * M.nalpha, M.nalpha, M.T, M.lm, it0, M.fl,
                                 M.ctl);
}

void launch_m_sturm(const MultiDev& M, int k, int lock, cudaStream_t st) {
  int threads = ((M.num_ev * kLPE + 31) / 32) * 32;
  if (threads > 1024) threads = 1024;
  if (threads < 32) threads = 32;
  const size_t shm = sizeof(double) * (3 * (size_t)M.lm + M.num_ev);
  k_m_sturm<<<M.S, threads, shm, st>>>(M.T, M.lm, k, lock, M.num_ev, M.en, M.nh, M.tol, M.mdim, M.fl, M.ctl, M.S);
}

static int reduce_grid(int count) { return (count * 32 + kNT - 1) / kNT; }

void launch_m_orth(const MultiDev& M, float* V, float* wh, float* wl, int it0, cudaStream_t st) {
  const int m = it0 + 1, S = M.S, G = M.G;
  const size_t hsh = 2 * sizeof(float) * (size_t)m * S;  // FP32 splits of the h_j
  SMGPU_S_DISPATCH(S, (k_m_dot_df<SS><<<G, kNT, 0, st>>>(V, M.len, it0, wh, wl, M.T, M.lm, M.part, G, M.fl, M.ctl, 1)));
  k_m_reduce<<<reduce_grid((m + 1) * S), kNT, 0, st>>>(M.part, G, (m + 1) * S, M.h1, M.ctl, 1);
  SMGPU_S_DISPATCH(S, (k_m_axpy_df<SS><<<G, kNT, hsh, st>>>(V, M.len, m, wh, wl, M.h1, M.part, G, M.fl, M.ctl,
                                                            nullptr)));
  k_m_reduce<<<reduce_grid(S), kNT, 0, st>>>(M.part, G, S, M.nrm1, M.ctl, 1);
  k_m_decide<<<1, 32, 0, st>>>(M.h1, M.nrm1, m, M.sec, M.fl, M.ctl, S);
  SMGPU_S_DISPATCH(S, (k_m_dot_df<SS><<<G, kNT, 0, st>>>(V, M.len, it0, wh, wl, M.T, M.lm, M.part, G, M.fl, M.ctl, 0)));
  k_m_reduce<<<reduce_grid(m * S), kNT, 0, st>>>(M.part, G, m * S, M.h2, M.ctl, 2);
  SMGPU_S_DISPATCH(S, (k_m_axpy_df<SS><<<G, kNT, hsh, st>>>(V, M.len, m, wh, wl, M.h2, M.part, G, M.fl, M.ctl,
                                                            M.sec)));
  k_m_reduce<<<reduce_grid(S), kNT, 0, st>>>(M.part, G, S, M.nrm2, M.ctl, 2);
  k_m_beta<<<1, 32, 0, st>>>(M.T, M.lm, it0, M.nrm1, M.nrm2, M.sec, M.invb, M.beta2, M.fl, M.ctl, S);
  SMGPU_S_DISPATCH(S, (k_m_scale_df<SS><<<grid_for(M.len * S / 4), kNT, 0, st>>>(
                          wh, wl, V + (int64_t)(it0 + 1) * M.len * S, M.invb, M.len, M.ctl)));
}

void launch_m_cycle_end(const MultiDev& M, cudaStream_t st) { k_m_cycle_end<<<1, 32, 0, st>>>(M.fl, M.ctl, M.S); }

void launch_m_restart(const MultiDev& M, float* V, float* U, cudaStream_t st) {
  const int S = M.S, lm = M.lm, ls = M.ls, m = lm - 1;
  const int64_t LS = M.len * S;
  k_m_jacobi<<<S, 256, jacobi_smem(m), st>>>(M.T, lm, m, M.jacA, M.jacZ, M.evals, M.fl, M.ctl, 1);
  k_m_restart_small<<<S, 256, 0, st>>>(M.T, lm, ls, M.evals, M.jacA, M.Yf, M.fl, M.ctl);
  const size_t ysh = sizeof(float) * (size_t)m * 8 * S;
  const int use_smem = ysh <= 48 * 1024 ? 1 : 0;
  const size_t yshr = sizeof(float) * (size_t)m * S * kMRLS;
  if (ls <= kMRLS && yshr <= 48 * 1024) {
    SMGPU_S_DISPATCH(S, (k_m_rotate_r<SS><<<grid_for(LS), kNT, yshr, st>>>(V, U, M.Yf, m, ls, M.len, M.fl, M.ctl)));
  } else {
    SMGPU_S_DISPATCH(S, (k_m_rotate<SS><<<grid_for(LS), kNT, use_smem ? ysh : 0, st>>>(V, U, M.Yf, m, ls, M.len, M.fl,
                                                                                    M.ctl, use_smem)));
  }
  const int tile = gram_tile(ls, S);
  const size_t gsh = sizeof(float) * (size_t)(ls + 1) * tile * S;
  SMGPU_S_DISPATCH(S, (k_m_gram<SS><<<M.G, kNT, gsh, st>>>(U, V + (int64_t)(lm - 1) * LS, ls, M.len, tile, M.part,
                                                           M.G, M.ctl)));
  const int PS = (ls * (ls + 1) / 2 + ls) * S;
  k_m_reduce<<<reduce_grid(PS), kNT, 0, st>>>(M.part, M.G, PS, M.gram, M.ctl, 1);
  if (ls <= 32) k_m_chol_df<<<S, 32, 0, st>>>(M.gram, ls, S, M.X, M.Xf, M.cvec, M.fl, M.ctl);
  else k_m_chol<<<S, 32, sizeof(double) * ls * ls, st>>>(M.gram, ls, S, M.X, M.Xf, M.cvec, M.fl, M.ctl);
  const size_t xsh = sizeof(float) * (size_t)S * ((ls * ls + ls) | 1);
  if (ls <= kMRLS && xsh <= 48 * 1024) {
    SMGPU_S_DISPATCH(S, (k_m_apply_r<SS><<<grid_for(LS), kNT, xsh, st>>>(U, V, M.Xf, ls, lm, M.len, M.fl, M.ctl)));
  } else {
    SMGPU_S_DISPATCH(S, (k_m_apply<SS><<<grid_for(LS), kNT, 0, st>>>(U, V, M.Xf, ls, lm, M.len, M.fl, M.ctl)));
  }
}

void launch_m_jacobi_one(const MultiDev& M, int s, int n, cudaStream_t st) {
  // one CTA on the slices of sample s
  const int64_t o = (int64_t)s * M.lm * M.lm;
  k_m_jacobi<<<1, 256, jacobi_smem(n), st>>>(M.T + o, M.lm, n, M.jacA + o, M.jacZ + o, M.evals + (int64_t)s * M.lm,
                                            M.fl, M.ctl, 0);
}

void launch_m_ritz(const MultiDev& M, const float* V, int s, int elit, int nev, double* R, cudaStream_t st) {
  k_m_ritz<<<grid_for(M.len), kNT, 0, st>>>(V, M.len, M.S, s, M.jacA + (int64_t)s * M.lm * M.lm, elit, nev, R);
}

}  // namespace smgpu
