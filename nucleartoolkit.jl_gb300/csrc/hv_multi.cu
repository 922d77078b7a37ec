// Multi-sample H·V on sm_103a: S interaction samples that share one basis
// (identical jump tables, S coefficient sets), FP32-mixed.  The counterpart
// of bl_operate_H! (src/ShellModel/lanczos_methods.jl:439-565) with one
// Hamiltonian per column instead of one shared Hamiltonian, and of the
// per-sample operate_H! calls of prepEC's sample loop
// (src/ShellModel/eigenvector_continuation.jl:140-177).
//
// Vectors and coefficients are interleaved sample-innermost (v[i*S + s],
// V[idx*S + s]), so one gather fetches S/4 aligned 16-byte pieces that hold
// every sample's value.  One output row (proton SD) per CTA; Q = S/4 threads
// per output column, each owning four samples, so a warp covers 32/Q
// consecutive columns and every pp gather is a contiguous run.  The pn term
// follows hv_tile_kernel: per link, the column's neutron entries are cached
// in registers (KM of them) and reused for every proton entry of the row;
// the neutron sign is folded into the signed-table index.  Epilogue per
// sample as in hv_tile_kernel: α partials in FP64 and the three-term
// correction −β_s v_prev.
//
// The launch shape (threads per CTA, minimum resident CTAs per SM, register
// cache length) is picked per problem by the autotuner in multi.cu from
// hv_multi_candidates().
#include "device.cuh"

namespace smgpu {

namespace {
struct AccKahanM {
  float s, c;
  __device__ __forceinline__ void init() { s = 0.f; c = 0.f; }
  __device__ __forceinline__ void add(float x) {
    float y = __fsub_rn(x, c);
    float t = __fadd_rn(s, y);
    c = __fsub_rn(__fsub_rn(t, s), y);
    s = t;
  }
  __device__ __forceinline__ double result() const { return (double)s - (double)c; }
};
}  // namespace

namespace {
template <int S>
struct MultiHvArgs {
  DevTables t;
  TileTables tt;  // one row per task
  MultiCoef c;
  const float* v;
  double* w;
  MultiEpilogue epi;
};

__device__ __forceinline__ void ld4(const float* __restrict__ p, float (&o)[4]) {
  const float4 f = *reinterpret_cast<const float4*>(p);
  o[0] = f.x;
  o[1] = f.y;
  o[2] = f.z;
  o[3] = f.w;
}
// Loads and stores of data touched once per H·V (v_prev, the output) with
// the evict-first hint: the interleaved vector that every gather reads
// (16 samples: 126 MB, about the L2) then keeps more of the L2.
__device__ __forceinline__ void ld4_stream(const float* __restrict__ p, float (&o)[4]) {
  const float4 f = __ldcs(reinterpret_cast<const float4*>(p));
  o[0] = f.x;
  o[1] = f.y;
  o[2] = f.z;
  o[3] = f.w;
}

template <int S, int NT, int MINB, int KM, bool DF>
__global__ void __launch_bounds__(NT, MINB) hv_multi_kernel(const MultiHvArgs<S> a) {
  if (a.epi.all_done != nullptr && cta_gate(threadIdx.x == 0 && *a.epi.all_done)) return;
  if (a.epi.count != nullptr && blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(a.epi.count, 1);
  constexpr int Q = S / 4;      // threads per column
  constexpr int CP = NT / Q;    // columns per pass
  const DevTables& t = a.t;
  const int task = blockIdx.x;
  const int b = a.tt.task_b[task];
  const int p = a.tt.task_p0[task];
  const int nn = t.nn[b];
  const int stride = t.stride[b];
  const int64_t blk = t.off_pad[b];
  const int g = t.pstart[b] + p, nst = t.nstart[b];
  const int lb = a.tt.link_begin[b];
  const int nl = a.tt.link_begin[b + 1] - lb;
  const int64_t rl0 = a.tt.rl_base[b] + (int64_t)p * (nl + 1);
  const int64_t rowoff = blk + (int64_t)p * stride;
  const int q = threadIdx.x % Q;
  const int s0 = 4 * q;
  const float* __restrict__ v = a.v + s0;
  double apart[4] = {0.0, 0.0, 0.0, 0.0};
  float aH[4] = {0.f, 0.f, 0.f, 0.f}, aL[4] = {0.f, 0.f, 0.f, 0.f};  // DF: α partials

  for (int n0 = 0; n0 < nn; n0 += CP) {
    const int n = n0 + (int)(threadIdx.x / Q);
    const bool act = n < nn;
    AccKahanM acc[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) acc[u].init();
    float x[4], cf[4];
    if (act) {
      const int gn = nst + n;
      for (int k = t.nn_ptr[gn]; k < t.nn_ptr[gn + 1]; ++k) {
        ld4(a.c.nn_val + (int64_t)k * S + s0, cf);
        ld4(v + (rowoff + t.nn_col[k]) * S, x);
#pragma unroll
        for (int u = 0; u < 4; ++u) acc[u].add(cf[u] * x[u]);
      }
      for (int k = t.pp_ptr[g]; k < t.pp_ptr[g + 1]; ++k) {
        ld4(a.c.pp_val + (int64_t)k * S + s0, cf);
        ld4(v + (blk + (int64_t)t.pp_col[k] * stride + n) * S, x);
#pragma unroll
        for (int u = 0; u < 4; ++u) acc[u].add(cf[u] * x[u]);
      }
    }
    for (int j = 0; j < nl; ++j) {
      const int L = lb + j;
      const int eb = a.tt.rl[rl0 + j], ee = a.tt.rl[rl0 + j + 1];
      if (eb == ee) continue;
      const int4 la = t.link_a[L];
      const int nB = la.y;
      const float* __restrict__ vt = a.c.vtab + t.link_v[L] * S + s0;
      const float* __restrict__ vs = v + t.off_pad[la.x] * S;
      const int sstride = t.stride[la.x];
      int64_t jb = 0;
      int K = 0;
      if (act) {
        const int64_t* np_ = a.tt.npn_ptr + t.link_n[L];
        jb = np_[n];
        K = (int)(np_[n + 1] - jb);
      }
      int Kw = K;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) Kw = max(Kw, __shfl_xor_sync(0xffffffffu, Kw, o));
      uint32_t ent[KM];
#pragma unroll
      for (int k = 0; k < KM; ++k) ent[k] = (k < K) ? a.tt.npn_ent[jb + k] : 0u;
      float part[4] = {0.f, 0.f, 0.f, 0.f};
      for (int e = eb; e < ee; ++e) {
        const uint32_t meta = t.ppn_meta[e];
        const float* __restrict__ row = vs + (int64_t)t.ppn_src[e] * sstride * S;
        const float* __restrict__ vr = vt + (int64_t)((meta >> 1) & 0x7fffu) * nB * S;
        float pe[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
        for (int k = 0; k < KM; ++k) {
          if (k >= Kw) break;
          if (k < K) {
            ld4(vr + (int)(ent[k] & 0x3fffu) * S, cf);
            ld4(row + (int)(ent[k] >> 14) * S, x);
#pragma unroll
            for (int u = 0; u < 4; ++u) pe[u] = fmaf(cf[u], x[u], pe[u]);
          }
        }
        if (Kw > KM)  // lists longer than the register cache
          for (int k = KM; k < K; ++k) {
            const uint32_t en = a.tt.npn_ent[jb + k];
            ld4(vr + (int)(en & 0x3fffu) * S, cf);
            ld4(row + (int)(en >> 14) * S, x);
#pragma unroll
            for (int u = 0; u < 4; ++u) pe[u] = fmaf(cf[u], x[u], pe[u]);
          }
        if (meta & 1u) {
#pragma unroll
          for (int u = 0; u < 4; ++u) part[u] -= pe[u];
        } else {
#pragma unroll
          for (int u = 0; u < 4; ++u) part[u] += pe[u];
        }
      }
#pragma unroll
      for (int u = 0; u < 4; ++u) acc[u].add(part[u]);
    }
    if (DF && act) {
      // epilogue in double-float on the FP32 pipe: w = wh + wl
      const int64_t o = (rowoff + n) * S;
      const int gn = nst + n;
      ld4(v + o, x);
      float xp[4] = {0.f, 0.f, 0.f, 0.f};
      if (a.epi.vprev != nullptr) ld4_stream(a.epi.vprev + s0 + o, xp);
      float hh[4], hl[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        fast_two_sum(acc[u].s, -acc[u].c, hh[u], hl[u]);
        const float2 ep = a.c.ep2[(int64_t)g * S + s0 + u], en = a.c.en2[(int64_t)gn * S + s0 + u];
        float dh = ep.x, dl = ep.y;
        df_add(dh, dl, en.x, en.y);
        df_fma(hh[u], hl[u], x[u], dh, dl);
        {  // α partial x·hv in double-float
          const float pp = __fmul_rn(x[u], hh[u]);
          const float pe = __fmaf_rn(x[u], hh[u], -pp);
          float t, e;
          two_sum(aH[u], pp, t, e);
          aH[u] = t;
          aL[u] = __fadd_rn(aL[u], __fadd_rn(e, __fmaf_rn(x[u], hl[u], pe)));
        }
        if (a.epi.vprev != nullptr) {
          const float2 b = a.epi.beta2[s0 + u];
          df_fma(hh[u], hl[u], xp[u], -b.x, -b.y);
        }
      }
      __stcs(reinterpret_cast<float4*>(a.epi.wh + o + s0), make_float4(hh[0], hh[1], hh[2], hh[3]));
      __stcs(reinterpret_cast<float4*>(a.epi.wl + o + s0), make_float4(hl[0], hl[1], hl[2], hl[3]));
    } else if (!DF && act) {
      const int64_t o = (rowoff + n) * S;
      const int gn = nst + n;
      ld4(v + o, x);
      float xp[4] = {0.f, 0.f, 0.f, 0.f};
      if (a.epi.vprev != nullptr) ld4_stream(a.epi.vprev + s0 + o, xp);
      double hv[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const double xd = (double)x[u];
        hv[u] = fma(a.c.ep[(int64_t)g * S + s0 + u] + a.c.en[(int64_t)gn * S + s0 + u], xd, acc[u].result());
        apart[u] = fma(xd, hv[u], apart[u]);
        if (a.epi.vprev != nullptr)
          hv[u] = fma(-a.epi.beta_base[(int64_t)(s0 + u) * a.epi.beta_stride], (double)xp[u], hv[u]);
      }
      double* wo = a.w + o + s0;
      __stcs(reinterpret_cast<double2*>(wo), make_double2(hv[0], hv[1]));
      __stcs(reinterpret_cast<double2*>(wo + 2), make_double2(hv[2], hv[3]));
    }
  }
  if constexpr (DF) {
#pragma unroll
    for (int u = 0; u < 4; ++u) apart[u] = (double)aH[u] + (double)aL[u];
  }
  if (a.epi.alpha_part != nullptr) {
    // sum over the threads of each sample group, fixed order
    __shared__ double red[NT / 32][S];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      double y = apart[u];
#pragma unroll
      for (int o = Q; o < 32; o <<= 1) y += __shfl_xor_sync(0xffffffffu, y, o);
      apart[u] = y;
    }
    const int lane = threadIdx.x & 31;
    if (lane < Q) {
#pragma unroll
      for (int u = 0; u < 4; ++u) red[threadIdx.x >> 5][4 * lane + u] = apart[u];
    }
    __syncthreads();
    if (threadIdx.x < S) {
      double sum = 0.0;
      for (int k = 0; k < NT / 32; ++k) sum += red[k][threadIdx.x];
      a.epi.alpha_part[(int64_t)threadIdx.x * gridDim.x + task] = sum;
    }
  }
}

// Launch shapes: threads per CTA, minimum resident CTAs per SM (caps the
// registers per thread), neutron entries cached in registers.
constexpr MultiHvConfig kMultiCand[] = {
    {256, 2, 16}, {256, 3, 8}, {256, 4, 8}, {128, 4, 16}, {128, 6, 8}, {128, 8, 8}, {512, 2, 8},
};
constexpr int kNMultiCand = (int)(sizeof(kMultiCand) / sizeof(kMultiCand[0]));

template <int S, int NT, int MINB, int KM>
static void launch_one(const DevTables& t, const TileTables& tt1, int ntasks, const MultiCoef& c, const float* v,
                       double* w, const MultiEpilogue& epi, cudaStream_t st) {
  const MultiHvArgs<S> a{t, tt1, c, v, w, epi};
  if (epi.wh != nullptr) hv_multi_kernel<S, NT, MINB, KM, true><<<ntasks, NT, 0, st>>>(a);
  else hv_multi_kernel<S, NT, MINB, KM, false><<<ntasks, NT, 0, st>>>(a);
}

template <int S>
static void launch_multi_s(int cand, const DevTables& t, const TileTables& tt1, int ntasks, const MultiCoef& c,
                           const float* v, double* w, const MultiEpilogue& epi, cudaStream_t st) {
  switch (cand) {
    case 0: launch_one<S, 256, 2, 16>(t, tt1, ntasks, c, v, w, epi, st); break;
    case 1: launch_one<S, 256, 3, 8>(t, tt1, ntasks, c, v, w, epi, st); break;
    case 2: launch_one<S, 256, 4, 8>(t, tt1, ntasks, c, v, w, epi, st); break;
    case 3: launch_one<S, 128, 4, 16>(t, tt1, ntasks, c, v, w, epi, st); break;
    case 4: launch_one<S, 128, 6, 8>(t, tt1, ntasks, c, v, w, epi, st); break;
    case 5: launch_one<S, 128, 8, 8>(t, tt1, ntasks, c, v, w, epi, st); break;
    default: launch_one<S, 512, 2, 8>(t, tt1, ntasks, c, v, w, epi, st); break;
  }
}

}  // namespace

const MultiHvConfig* hv_multi_candidates(int* count) {
  *count = kNMultiCand;
  return kMultiCand;
}

bool hv_multi_supported(int S) { return S == 4 || S == 8 || S == 16; }

void launch_hv_multi(int S, int cand, const DevTables& t, const TileTables& tt1, int ntasks, const MultiCoef& c,
                     const float* v, double* w, const MultiEpilogue& epi, cudaStream_t st) {
  if (cand < 0 || cand >= kNMultiCand) cand = 0;
  switch (S) {
    case 4: launch_multi_s<4>(cand, t, tt1, ntasks, c, v, w, epi, st); break;
    case 8: launch_multi_s<8>(cand, t, tt1, ntasks, c, v, w, epi, st); break;
    case 16: launch_multi_s<16>(cand, t, tt1, ntasks, c, v, w, epi, st); break;
    default: break;
  }
}

}  // namespace smgpu
