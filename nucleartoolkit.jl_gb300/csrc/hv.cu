// H·v for the M-scheme shell-model Hamiltonian on sm_103a.
//
// Replaces operate_H! (src/ShellModel/lanczos_methods.jl:153-248).  The
// reference walks (block pair, V entry) lists and scatters into twf from one
// thread per block.  Here every output row of a (Mp,Mn) block — one proton
// Slater determinant p with all its neutron partners n — is owned by one CTA,
// which pulls every contribution to that row and writes it exactly once:
//
//   w[b,p,n] = (e_p + e_n) v[b,p,n]                         one-body
//            + Σ_{p'} Hpp[p,p'] v[b,p',n]                    pp (coalesced rows)
//            + Σ_{n'} Hnn[n,n'] v[b,p,n']                    nn
//            + Σ_{(s,p',a,c,±)} ± Σ_{(n',b,d,±)} V[ac][bd] v[s,p',n']   pn
//
// The pn term is factorised: each proton pull entry (source block s, source
// row p', operator a†c, sign) is combined with the neutron pull list of the
// (b <- s) link, whose coefficients come from the small per-ΔM table V[ac][bd].
// There are no atomics and every output element is written once.
//
// The vector lives in a padded layout: block b occupies np[b] rows of
// stride[b] = round_up(nn[b], 4) elements starting at off_pad[b]; padding is 0.
//
// Precision forms
//   FP64 plain : v, coefficients, accumulation FP64.
//   mixed      : v and coefficients FP32, FP32 partial sums combined with
//                Kahan compensation; the one-body term and the output FP64.
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
  __device__ __forceinline__ double result() const { return (double)s - (double)c; }
};

template <class TV, class TC, class Acc, int NT>
__global__ void __launch_bounds__(NT) hv_pull_kernel(DevTables t, const double* __restrict__ ep,
                                                     const double* __restrict__ en, CoefTables<TC> c,
                                                     const TV* __restrict__ v, double* __restrict__ w,
                                                     const int* __restrict__ done) {
  if (done != nullptr && *done) return;
  const int g = blockIdx.x;  // global proton row
  const int b = t.prow_block[g];
  const int p = g - t.pstart[b];
  const int nn = t.nn[b];
  const int stride = t.stride[b];
  const int64_t blk = t.off_pad[b];
  const int64_t rowoff = blk + (int64_t)p * stride;
  const int ppb = t.pp_ptr[g], ppe = t.pp_ptr[g + 1];
  const int pnb = t.ppn_ptr[g], pne = t.ppn_ptr[g + 1];
  const double epg = ep[g];
  const int nst = t.nstart[b];

  for (int n = threadIdx.x; n < nn; n += NT) {
    Acc acc;
    acc.init();
    // pp: other proton rows of the same block, same neutron column (coalesced)
    for (int k = ppb; k < ppe; ++k) acc.add(c.pp_val[k] * (TC)v[blk + (int64_t)t.pp_col[k] * stride + n]);
    // nn: same proton row, other neutron columns
    const int gn = nst + n;
    const int nnb = t.nn_ptr[gn], nne = t.nn_ptr[gn + 1];
    for (int k = nnb; k < nne; ++k) acc.add(c.nn_val[k] * (TC)v[rowoff + t.nn_col[k]]);
    // pn
    int cur = -1;
    int64_t sblk = 0;
    int sstride = 0, nB = 0;
    const TC* vt = nullptr;
    int64_t jb = 0, je = 0;
    for (int k = pnb; k < pne; ++k) {
      const uint32_t meta = t.ppn_meta[k];
      const int L = (int)(meta >> 16);
      if (L != cur) {
        cur = L;
        const int4 la = t.link_a[L];
        nB = la.y;
        sblk = t.off_pad[la.x];
        sstride = t.stride[la.x];
        vt = c.vtab + t.link_v[L];
        const int64_t* np_ = t.npn_ptr + t.link_n[L];
        jb = np_[n];
        je = np_[n + 1];
      }
      const TV* row = v + sblk + (int64_t)t.ppn_src[k] * sstride;
      const TC* vrow = vt + (int)((meta >> 1) & 0x7fffu) * nB;
      TC part = (TC)0;
      for (int64_t j = jb; j < je; ++j) {
        const uint32_t e = t.npn_ent[j];
        const TC term = vrow[(e >> 1) & 0x1fffu] * (TC)row[e >> 14];
        part += (e & 1u) ? -term : term;
      }
      acc.add((meta & 1u) ? -part : part);
    }
    const double diag = (epg + en[gn]) * (double)v[rowoff + n];
    w[rowoff + n] = acc.result() + diag;
  }
}

void launch_hv_fp64(const DevTables& t, const double* ep, const double* en, const CoefTables<double>& c,
                    const double* v, double* w, int nrows, const int* done, cudaStream_t st) {
  constexpr int NT = 128;
  hv_pull_kernel<double, double, AccF64, NT><<<nrows, NT, 0, st>>>(t, ep, en, c, v, w, done);
}

void launch_hv_mixed(const DevTables& t, const double* ep, const double* en, const CoefTables<float>& c,
                     const float* v, double* w, int nrows, const int* done, cudaStream_t st) {
  constexpr int NT = 128;
  hv_pull_kernel<float, float, AccKahan, NT><<<nrows, NT, 0, st>>>(t, ep, en, c, v, w, done);
}

}  // namespace smgpu
