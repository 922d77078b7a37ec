// H·v for the M-scheme shell-model Hamiltonian on sm_103a.
//
// Replaces operate_H! (src/ShellModel/lanczos_methods.jl:153-248).  The
// reference walks (block pair, V entry) lists and scatters into twf from one
// thread per block.  Here the output is tiled by rows of a (Mp,Mn) block — a
// row is one proton Slater determinant p with all its neutron partners n —
// and every CTA owns R consecutive rows of one block, pulls every
// contribution to them and writes each output element exactly once:
//
//   w[b,p,n] = (e_p + e_n) v[b,p,n]                         one-body
//            + Σ_{p'} Hpp[p,p'] v[b,p',n]                    pp (coalesced rows)
//            + Σ_{n'} Hnn[n,n'] v[b,p,n']                    nn
//            + Σ_links Σ_{(p',a†c,±)} ± Σ_{(n',b†d,±)} V[ac][bd] v[s,p',n']   pn
//
// The pn term is factorised per link (output block b <- source block s): the
// proton pull entries of each row (source row p', operator index, sign) are
// combined with the neutron pull list of the link.  A thread owns one column
// n; its neutron list for the link (at most 16 entries for the pf shell) is
// loaded once into registers and reused for all proton entries of the R rows.
// The per-ΔM coefficient table is stored twice (V and −V) so the neutron sign
// is folded into the table index.  No atomics; no scratch.
//
// Lanczos epilogue (optional): per-CTA partial sums of α = v·Hv (FP64) and
// the three-term correction w = Hv − β v_prev, so the re-orthogonalisation
// passes start from the Lanczos residual.
//
// Precision forms
//   FP64 plain : v, coefficients, accumulation FP64.
//   mixed      : v and coefficients FP32; FP32 partial sums per (row, link) and
//                per pp/nn entry, combined with Kahan compensation; the
//                one-body term, the epilogue and the output in FP64.
#include "device.cuh"
#include "lanczos.cuh"

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
  __device__ __forceinline__ double result() const { return (double)s - (double)c; }
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
};

constexpr int KMAX = 16;

template <class TV, class TC, class Acc, int NT, int R, int MINB>
__global__ void __launch_bounds__(NT, MINB) hv_tile_kernel(const HvArgs<TV, TC> a) {
  if (a.fl != nullptr && (a.fl->done || a.fl->exhausted)) return;
  const DevTables& t = a.t;
  const int task = blockIdx.x;
  const int b = a.tt.task_b[task];
  const int p0 = a.tt.task_p0[task];
  const int np = t.np[b];
  const int nr = min(R, np - p0);
  const int nn = t.nn[b];
  const int stride = t.stride[b];
  const int64_t blk = t.off_pad[b];
  const int pst = t.pstart[b], nst = t.nstart[b];
  const int lb = a.tt.link_begin[b];
  const int nl = a.tt.link_begin[b + 1] - lb;
  const int64_t rlb = a.tt.rl_base[b] + (int64_t)p0 * (nl + 1);
  const TV* __restrict__ v = a.v;
  const double beta = (a.vprev != nullptr) ? *a.beta : 0.0;
  double apart = 0.0;

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
    if (act) {
      const double enn = a.en[nst + n];
#pragma unroll
      for (int r = 0; r < R; ++r) {
        if (r >= nr) break;
        const int64_t o = blk + (int64_t)(p0 + r) * stride + n;
        const double x = (double)v[o];
        double hv = acc[r].result() + (a.ep[pst + p0 + r] + enn) * x;
        apart = fma(x, hv, apart);
        if (a.vprev != nullptr) hv = fma(-beta, (double)a.vprev[o], hv);
        a.w[o] = hv;
      }
    }
  }
  if (a.alpha_part != nullptr) {
    __shared__ double red[NT / 32];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) apart += __shfl_down_sync(0xffffffffu, apart, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = apart;
    __syncthreads();
    if (threadIdx.x == 0) {
      double s = 0.0;
      for (int k = 0; k < NT / 32; ++k) s += red[k];
      a.alpha_part[task] = s;
    }
  }
}

// ---------------------------------------------------------------- dispatch
template <class TV, class TC, class Acc>
static void launch_cfg(const HvConfig& cfg, const HvArgs<TV, TC>& a, cudaStream_t st) {
  const int grid = cfg.ntasks;
#define SMGPU_HV_CASE(NT_, R_, MB_)                                           \
  if (cfg.nt == NT_ && cfg.rows == R_ && cfg.minb == MB_) {                   \
    hv_tile_kernel<TV, TC, Acc, NT_, R_, MB_><<<grid, NT_, 0, st>>>(a);       \
    return;                                                                   \
  }
  SMGPU_HV_CASE(128, 1, 1)
  SMGPU_HV_CASE(128, 2, 1)
  SMGPU_HV_CASE(128, 4, 1)
  SMGPU_HV_CASE(128, 8, 1)
  SMGPU_HV_CASE(128, 1, 8)
  SMGPU_HV_CASE(128, 2, 6)
  SMGPU_HV_CASE(128, 4, 6)
  SMGPU_HV_CASE(192, 2, 4)
  SMGPU_HV_CASE(256, 1, 1)
  SMGPU_HV_CASE(256, 2, 1)
  SMGPU_HV_CASE(256, 4, 1)
  SMGPU_HV_CASE(256, 2, 3)
  SMGPU_HV_CASE(256, 4, 3)
#undef SMGPU_HV_CASE
}

const HvConfig* hv_candidates(int* count) {
  // {threads, rows per CTA, -, min CTAs per SM (register cap)}
  static const HvConfig c[] = {{128, 1, 0, 1}, {128, 2, 0, 1}, {128, 4, 0, 1}, {128, 8, 0, 1}, {128, 1, 0, 8},
                               {128, 2, 0, 6}, {128, 4, 0, 6}, {192, 2, 0, 4}, {256, 1, 0, 1}, {256, 2, 0, 1},
                               {256, 4, 0, 1}, {256, 2, 0, 3}, {256, 4, 0, 3}};
  *count = (int)(sizeof(c) / sizeof(c[0]));
  return c;
}

void launch_hv_fp64(const DevTables& t, const TileTables& tt, const HvConfig& cfg, const double* ep,
                    const double* en, const CoefTables<double>& c, const double* v, double* w,
                    const HvEpilogue<double>& epi, cudaStream_t st) {
  HvArgs<double, double> a{t, tt, c, ep, en, v, w, epi.fl, epi.vprev, epi.beta, epi.alpha_part};
  launch_cfg<double, double, AccF64>(cfg, a, st);
}

void launch_hv_mixed(const DevTables& t, const TileTables& tt, const HvConfig& cfg, const double* ep,
                     const double* en, const CoefTables<float>& c, const float* v, double* w,
                     const HvEpilogue<float>& epi, cudaStream_t st) {
  HvArgs<float, float> a{t, tt, c, ep, en, v, w, epi.fl, epi.vprev, epi.beta, epi.alpha_part};
  launch_cfg<float, float, AccKahan>(cfg, a, st);
}

}  // namespace smgpu
