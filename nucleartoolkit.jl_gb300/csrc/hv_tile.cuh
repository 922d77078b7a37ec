// The row-tile body of the H·v kernel, shared by the single-problem kernel
// (hv.cu) and the batched kernel (hv_batch.cu).  See hv.cu for the algorithm.
#pragma once
#include "device.cuh"

namespace smgpu {

struct AccF64 {
  double s;
  __device__ __forceinline__ void init() { s = 0.0; }
  __device__ __forceinline__ void add(double x) { s += x; }
  __device__ __forceinline__ double result() const { return s; }
};

// Kahan-compensated FP32 accumulator (explicit round-to-nearest intrinsics so
// the compiler cannot re-associate or contract the compensation away).
struct AccKahan {
  float s, c;
  __device__ __forceinline__ void init() { s = 0.f; c = 0.f; }
  __device__ __forceinline__ void add(float x) {
    float y = __fsub_rn(x, c);
    float t = __fadd_rn(s, y);
    c = __fsub_rn(__fsub_rn(t, s), y);
    s = t;
  }
  // (widened with integer instructions: conversions on this GPU share the
  // scarce FP64 pipe)
  __device__ __forceinline__ double result() const { return widen(s) - widen(c); }
};

template <class TV, class TC>
struct HvArgs {
  DevTables t;
  TileTables tt;
  CoefTables<TC> c;
  const double* ep;
  const double* en;
  const TV* v;
  double* w;
  const LanczosFlags* fl;  // gate (may be null)
  const TV* vprev;         // three-term correction (may be null)
  const double* beta;      // β of the previous iteration
  double* alpha_part;      // per-CTA partial of v·Hv (may be null)
  // double-float output (the DF kernels): w = wh + wl, one-body diagonals as
  // (hi, lo) pairs
  float* wh;
  float* wl;
  const float2* ep2;
  const float2* en2;
};

constexpr int KMAX = 16;

// The rows p0 .. p0+R-1 of block b (one CTA): w = H v on those rows, with
// the tables of `a` (its v/w/vprev fields are not read; the vectors are the
// explicit arguments).  vprev: three-term correction w -= beta*vprev (null:
// none); alpha_out: where the CTA's partial of v·Hv goes (null: none).
// DF = true (FP32 v, Kahan accumulation): the epilogue runs in double-float
// and writes w as the pair (a.wh, a.wl); the α partial is stored as a
// double-float (hi, lo) float pair in the FP64 slot.
template <class TV, class TC, class Acc, int NT, int R, bool DF = false>
__device__ __forceinline__ void hv_tile_rows(const HvArgs<TV, TC>& a, const TV* __restrict__ v, double* w,
                                             const TV* vprev, const int b, const int p0, const double beta,
                                             double* alpha_out) {
  const DevTables& t = a.t;
  const int np = t.np[b];
  const int nr = min(R, np - p0);
  const int nn = t.nn[b];
  const int stride = t.stride[b];
  const int64_t blk = t.off_pad[b];
  const int pst = t.pstart[b], nst = t.nstart[b];
  const int lb = a.tt.link_begin[b];
  const int nl = a.tt.link_begin[b + 1] - lb;
  const int64_t rlb = a.tt.rl_base[b] + (int64_t)p0 * (nl + 1);
  double apart = 0.0;
  float ah = 0.f, al = 0.f;  // DF: α partial
  float bh = 0.f, bl = 0.f;  // DF: β
  if constexpr (DF) df_from_double(beta, bh, bl);

  for (int n0 = 0; n0 < nn; n0 += NT) {
    const int n = n0 + threadIdx.x;
    const bool act = n < nn;
    Acc acc[R];
#pragma unroll
    for (int r = 0; r < R; ++r) acc[r].init();

    // nn: same proton row, other neutron columns (the column list is shared by the R rows)
    if (act) {
      const int gn = nst + n;
      const int kb = t.nn_ptr[gn], ke = t.nn_ptr[gn + 1];
      for (int k = kb; k < ke; ++k) {
        const int c = t.nn_col[k];
        const TC cv = a.c.nn_val[k];
#pragma unroll
        for (int r = 0; r < R; ++r)
          if (r < nr) acc[r].add(cv * (TC)v[blk + (int64_t)(p0 + r) * stride + c]);
      }
    }
    // pp: other proton rows of the block, same neutron column (coalesced)
#pragma unroll
    for (int r = 0; r < R; ++r) {
      if (r >= nr) break;
      const int g = pst + p0 + r;
      const int kb = t.pp_ptr[g], ke = t.pp_ptr[g + 1];
      if (act)
        for (int k = kb; k < ke; ++k) acc[r].add(a.c.pp_val[k] * (TC)v[blk + (int64_t)t.pp_col[k] * stride + n]);
    }
    // pn, link by link
    for (int j = 0; j < nl; ++j) {
      const int L = lb + j;
      const int4 la = t.link_a[L];
      const int nB = la.y;
      const TC* __restrict__ vt = a.c.vtab + t.link_v[L];
      const TV* __restrict__ vs = v + t.off_pad[la.x];
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
      // the thread's neutron entries (n' << 14 | signed table column), packed
      uint32_t ent[KMAX];
#pragma unroll
      for (int k = 0; k < KMAX; ++k) ent[k] = (k < K) ? a.tt.npn_ent[jb + k] : 0u;
#pragma unroll
      for (int r = 0; r < R; ++r) {
        if (r >= nr) break;
        const int eb = a.tt.rl[rlb + (int64_t)r * (nl + 1) + j];
        const int ee = a.tt.rl[rlb + (int64_t)r * (nl + 1) + j + 1];
        TC part = (TC)0;
        int e = eb;
        // two proton entries in flight: twice the independent gathers per thread
        for (; e + 1 < ee; e += 2) {
          const TV* __restrict__ row0 = vs + (int64_t)t.ppn_src[e] * sstride;
          const TV* __restrict__ row1 = vs + (int64_t)t.ppn_src[e + 1] * sstride;
          const uint32_t m0 = t.ppn_meta[e], m1 = t.ppn_meta[e + 1];
          const TC* __restrict__ vr0 = vt + (int)((m0 >> 1) & 0x7fffu) * nB;
          const TC* __restrict__ vr1 = vt + (int)((m1 >> 1) & 0x7fffu) * nB;
          TC pe0 = (TC)0, pe1 = (TC)0;
#pragma unroll
          for (int k = 0; k < KMAX; ++k) {
            if (k >= Kw) break;
            if (k < K) {
              const int nf = (int)(ent[k] >> 14), vc = (int)(ent[k] & 0x3fffu);
              pe0 += vr0[vc] * (TC)row0[nf];
              pe1 += vr1[vc] * (TC)row1[nf];
            }
          }
          if (Kw > KMAX)  // lists longer than the register cache
            for (int k = KMAX; k < K; ++k) {
              const uint32_t en = a.tt.npn_ent[jb + k];
              pe0 += vr0[en & 0x3fffu] * (TC)row0[en >> 14];
              pe1 += vr1[en & 0x3fffu] * (TC)row1[en >> 14];
            }
          part += (m0 & 1u) ? -pe0 : pe0;
          part += (m1 & 1u) ? -pe1 : pe1;
        }
        if (e < ee) {
          const TV* __restrict__ row = vs + (int64_t)t.ppn_src[e] * sstride;
          const uint32_t meta = t.ppn_meta[e];
          const TC* __restrict__ vr = vt + (int)((meta >> 1) & 0x7fffu) * nB;
          TC pe = (TC)0;
#pragma unroll
          for (int k = 0; k < KMAX; ++k) {
            if (k >= Kw) break;
            if (k < K) pe += vr[ent[k] & 0x3fffu] * (TC)row[ent[k] >> 14];
          }
          if (Kw > KMAX)
            for (int k = KMAX; k < K; ++k) {
              const uint32_t en = a.tt.npn_ent[jb + k];
              pe += vr[en & 0x3fffu] * (TC)row[en >> 14];
            }
          part += (meta & 1u) ? -pe : pe;
        }
        acc[r].add(part);
      }
    }
    // one-body term, Lanczos epilogue, store
    if constexpr (DF) {
      if (act) {
        const float2 en2 = a.en2[nst + n];
#pragma unroll
        for (int r = 0; r < R; ++r) {
          if (r >= nr) break;
          const int64_t o = blk + (int64_t)(p0 + r) * stride + n;
          const float x = (float)v[o];
          float hh, hl;
          fast_two_sum(acc[r].s, -acc[r].c, hh, hl);  // the Kahan pair as a double-float value
          const float2 ep2 = a.ep2[pst + p0 + r];
          float dh = ep2.x, dl = ep2.y;
          df_add(dh, dl, en2.x, en2.y);
          df_fma(hh, hl, x, dh, dl);
          // α partial: x·hv
          {
            const float p = __fmul_rn(x, hh);
            const float pe = __fmaf_rn(x, hh, -p);
            float s, e;
            two_sum(ah, p, s, e);
            ah = s;
            al = __fadd_rn(al, __fadd_rn(e, __fmaf_rn(x, hl, pe)));
          }
          if (vprev != nullptr) df_fma(hh, hl, (float)vprev[o], -bh, -bl);
          a.wh[o] = hh;
          a.wl[o] = hl;
        }
      }
    } else if (act) {
      const double enn = a.en[nst + n];
#pragma unroll
      for (int r = 0; r < R; ++r) {
        if (r >= nr) break;
        const int64_t o = blk + (int64_t)(p0 + r) * stride + n;
        const double x = widen(v[o]);
        double hv = fma(a.ep[pst + p0 + r] + enn, x, acc[r].result());
        apart = fma(x, hv, apart);
        if (vprev != nullptr) hv = fma(-beta, widen(vprev[o]), hv);
        w[o] = hv;
      }
    }
  }
  if (alpha_out != nullptr) {
    __shared__ double red[NT / 32];
    if constexpr (DF) {
      // double-float all the way; the partial is stored as a (hi, lo) pair
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        const float oh = __shfl_down_sync(0xffffffffu, ah, o);
        const float ol = __shfl_down_sync(0xffffffffu, al, o);
        df_add(ah, al, oh, ol);
      }
      float2* r2 = reinterpret_cast<float2*>(red);
      if ((threadIdx.x & 31) == 0) r2[threadIdx.x >> 5] = make_float2(ah, al);
      __syncthreads();
      if (threadIdx.x == 0) {
        float h = r2[0].x, l = r2[0].y;
        for (int k = 1; k < NT / 32; ++k) df_add(h, l, r2[k].x, r2[k].y);
        *reinterpret_cast<float2*>(alpha_out) = make_float2(h, l);
      }
      return;
    } else {
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) apart += __shfl_down_sync(0xffffffffu, apart, o);
    }
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = apart;
    __syncthreads();
    if (threadIdx.x == 0) {
      double s = 0.0;
      for (int k = 0; k < NT / 32; ++k) s += red[k];
      *alpha_out = s;
    }
  }
}

}  // namespace smgpu
