// One-body M1 / E2 operators on the GPU: O·v in the pull form of obtr.h and
// the matrix of overlaps <l_a| O |r_b> (op_obtr_diag / op_obtr_nondiag and
// the dot products of eval_moment / transit_main, src/ShellModel/transit.jl:
// 247-284, 447-499, 561-765).  FP64 throughout; vectors in the reference's
// basis order (block by block, proton-major inside a block).
#include <cmath>
#include <string>

#include "lanczos_dev.cuh"
#include "obtr.h"
#include "pairdots.cuh"
#include "problem.h"

namespace smgpu {
namespace {

struct ObtrDev {
  int nb_l;
  const int64_t* tdims_l;  // nb_l + 1
  const int* nn_l;
  const int* pstart_l;
  const int* nstart_l;
  const int64_t* tdims_r;
  const int* nn_r;
  const int* psrc;
  const int* nsrc;
  const int* p_ptr;
  const int* p_col;
  const double* p_val;
  const int* n_ptr;
  const int* n_col;
  const double* n_val;
};

constexpr int kApplyNT = 256;

// w[k] = O v[k] for the right vectors k = blockIdx.y; one thread per element
// of the left basis, neutron index fastest (coalesced rows).
__global__ void __launch_bounds__(kApplyNT) k_obtr_apply(ObtrDev o, const double* __restrict__ v, int64_t mdim_r,
                                                         double* __restrict__ w, int64_t mdim_l) {
  const int64_t i = (int64_t)blockIdx.x * kApplyNT + threadIdx.x;
  if (i >= mdim_l) return;
  const double* vk = v + (int64_t)blockIdx.y * mdim_r;
  const int b = dev::find_block(o.tdims_l, o.nb_l, i);
  const int nn = o.nn_l[b];
  const int64_t loc = i - o.tdims_l[b];
  const int p = (int)(loc / nn), n = (int)(loc - (int64_t)p * nn);
  double acc = 0.0;
  const int bp = o.psrc[b];
  if (bp >= 0) {
    const double* src = vk + o.tdims_r[bp] + n;  // same neutron list: nn_r[bp] == nn
    const int row = o.pstart_l[b] + p;
    for (int e = o.p_ptr[row]; e < o.p_ptr[row + 1]; ++e) acc = fma(o.p_val[e], src[(int64_t)o.p_col[e] * nn], acc);
  }
  const int bn = o.nsrc[b];
  if (bn >= 0) {
    const double* src = vk + o.tdims_r[bn] + (int64_t)p * o.nn_r[bn];  // same proton list
    const int row = o.nstart_l[b] + n;
    for (int e = o.n_ptr[row]; e < o.n_ptr[row + 1]; ++e) acc = fma(o.n_val[e], src[o.n_col[e]], acc);
  }
  w[(int64_t)blockIdx.y * mdim_l + i] = acc;
}

constexpr int kDotNT = 256;

// partial[(a*nw + b)*G + g] = Σ over chunk g of x[a]·y[b]   (blockIdx.y = a*nw + b)
__global__ void __launch_bounds__(kDotNT) k_pair_dots(const double* __restrict__ x, int nx, const double* __restrict__ y,
                                                      int ny, int64_t len, double* __restrict__ partial) {
  __shared__ double red[kDotNT / 32];
  const int pair = blockIdx.y, a = pair / ny, b = pair - a * ny;
  int64_t s, e;
  dev::chunk_of(len, gridDim.x, s, e);
  const double* xa = x + (int64_t)a * len;
  const double* yb = y + (int64_t)b * len;
  double acc = 0.0;
  for (int64_t i = s + threadIdx.x; i < e; i += kDotNT) acc = fma(xa[i], yb[i], acc);
  acc = dev::block_sum_all<kDotNT>(acc, red);
  if (threadIdx.x == 0) partial[(int64_t)pair * gridDim.x + blockIdx.x] = acc;
  (void)nx;
}

// out[pair] = Σ_g partial[pair*G + g] in a fixed order, one warp per pair.
__global__ void __launch_bounds__(kDotNT) k_pair_reduce(const double* __restrict__ partial, int G, int npairs,
                                                        double* __restrict__ out) {
  const int lane = threadIdx.x & 31;
  const int pair = blockIdx.x * (kDotNT / 32) + (threadIdx.x >> 5);
  if (pair >= npairs) return;
  double x = 0.0;
  for (int g = lane; g < G; g += 32) x += partial[(int64_t)pair * G + g];
  x = dev::warp_sum(x);
  if (lane == 0) out[pair] = x;
}

}  // namespace

int pair_dot_chunks(int64_t len) {
  int64_t G = (len + kDotNT * 16 - 1) / (kDotNT * 16);
  return (int)(G < 1 ? 1 : (G > 128 ? 128 : G));
}

void launch_pair_dots(const double* x, int nx, const double* y, int ny, int64_t len, double* partial, double* out,
                      cudaStream_t st) {
  const int G = pair_dot_chunks(len);
  k_pair_dots<<<dim3(G, nx * ny), kDotNT, 0, st>>>(x, nx, y, ny, len, partial);
  SMGPU_CUDA_TRY(cudaGetLastError());
  const int npairs = nx * ny;
  k_pair_reduce<<<(npairs + kDotNT / 32 - 1) / (kDotNT / 32), kDotNT, 0, st>>>(partial, G, npairs, out);
  SMGPU_CUDA_TRY(cudaGetLastError());
}

}  // namespace smgpu

namespace {
int obtr_fail(smgpu_problem* h, int code, const std::string& msg) {
  if (h) h->err = msg;
  return code;
}
bool same_orbits(const std::vector<Orbit>& a, const std::vector<Orbit>& b) {
  if (a.size() != b.size()) return false;
  for (size_t k = 0; k < a.size(); ++k)
    if (a[k].n != b[k].n || a[k].l != b[k].l || a[k].j2 != b[k].j2 || a[k].tz != b[k].tz) return false;
  return true;
}
}  // namespace

extern "C" {

double smgpu_wigner3j(int tj1, int tj2, int tj3, int tm1, int tm2, int tm3) {
  return smgpu::wigner3j(tj1, tj2, tj3, tm1, tm2, tm3);
}

double smgpu_wigner6j(int tj1, int tj2, int tj3, int tj4, int tj5, int tj6) {
  return smgpu::wigner6j(tj1, tj2, tj3, tj4, tj5, tj6);
}

int smgpu_obtr(smgpu_problem* hl, smgpu_problem* hr, int op, int symmetric, const double* gfactors,
               const double* effcharge, const double* vl, int nl, const double* vr, int nr, double* out) {
  if (!hl || !hr || !vl || !vr || !out || nl < 1 || nr < 1) return obtr_fail(hl, SMGPU_ERR_ARG, "bad obtr arguments");
  if (op != OBTR_M1 && op != OBTR_E2) return obtr_fail(hl, SMGPU_ERR_ARG, "op must be SMGPU_OBTR_M1 or SMGPU_OBTR_E2");
  if (hl->vp != hr->vp || hl->vn != hr->vn || hl->I.cp != hr->I.cp || hl->I.cn != hr->I.cn ||
      !same_orbits(hl->I.porb, hr->I.porb) || !same_orbits(hl->I.norb, hr->I.norb))
    return obtr_fail(hl, SMGPU_ERR_ARG, "the two handles must describe one nucleus on one model space");
  if ((int64_t)nl * nr > 65535) return obtr_fail(hl, SMGPU_ERR_LIMIT, "nl * nr must not exceed 65535");
  const double gdef[4] = {1.0, 0.0, 5.586, -3.826}, edef[2] = {1.5, 0.5};
  const double* gf = gfactors ? gfactors : gdef;
  const double* ec = effcharge ? effcharge : edef;
  DeviceArena tmp;
  try {
    const int A = hl->I.cp + hl->I.cn + hl->vp + hl->vn;
    ObtrTables ot;
    build_obtr(hl->I, hl->T, hr->T, hl->mtot2, hr->mtot2, A, op, symmetric != 0, gf, ec, ot);
    const Tables& L = hl->T;
    const Tables& R = hr->T;
    cudaStream_t st = hl->st;
    ObtrDev o{};
    o.nb_l = L.nb;
    o.tdims_l = tmp.upload(L.tdims);
    o.nn_l = tmp.upload(L.nn);
    o.pstart_l = tmp.upload(L.pstart);
    o.nstart_l = tmp.upload(L.nstart);
    o.tdims_r = tmp.upload(R.tdims);
    o.nn_r = tmp.upload(R.nn);
    o.psrc = tmp.upload(ot.psrc);
    o.nsrc = tmp.upload(ot.nsrc);
    o.p_ptr = tmp.upload(ot.p_ptr);
    o.p_col = tmp.upload(ot.p_col);
    o.p_val = tmp.upload(ot.p_val);
    o.n_ptr = tmp.upload(ot.n_ptr);
    o.n_col = tmp.upload(ot.n_col);
    o.n_val = tmp.upload(ot.n_val);
    SMGPU_CUDA_TRY(cudaDeviceSynchronize());  // uploads complete before work on the handle's stream
    const int64_t ml = L.mdim, mr = R.mdim;
    constexpr int kChunk = 8;  // right vectors per pass
    const int nrc = nr < kChunk ? nr : kChunk;
    double* d_vl = tmp.alloc<double>((size_t)nl * ml);
    double* d_vr = tmp.alloc<double>((size_t)nrc * mr);
    double* d_w = tmp.alloc<double>((size_t)nrc * ml);
    double* d_part = tmp.alloc<double>((size_t)nl * nrc * pair_dot_chunks(ml));
    double* d_out = tmp.alloc<double>((size_t)nl * nrc);
    std::vector<double> h_out((size_t)nl * nrc);
    SMGPU_CUDA_TRY(cudaMemcpyAsync(d_vl, vl, sizeof(double) * nl * ml, cudaMemcpyHostToDevice, st));
    for (int b0 = 0; b0 < nr; b0 += nrc) {
      const int nb = (nr - b0) < nrc ? (nr - b0) : nrc;
      SMGPU_CUDA_TRY(cudaMemcpyAsync(d_vr, vr + (size_t)b0 * mr, sizeof(double) * nb * mr, cudaMemcpyHostToDevice, st));
      k_obtr_apply<<<dim3((unsigned)((ml + kApplyNT - 1) / kApplyNT), nb), kApplyNT, 0, st>>>(o, d_vr, mr, d_w, ml);
      SMGPU_CUDA_TRY(cudaGetLastError());
      launch_pair_dots(d_vl, nl, d_w, nb, ml, d_part, d_out, st);
      const int npairs = nl * nb;
      SMGPU_CUDA_TRY(cudaMemcpyAsync(h_out.data(), d_out, sizeof(double) * npairs, cudaMemcpyDeviceToHost, st));
      SMGPU_CUDA_TRY(cudaStreamSynchronize(st));
      for (int a = 0; a < nl; ++a)
        for (int b = 0; b < nb; ++b) out[(size_t)a * nr + b0 + b] = h_out[(size_t)a * nb + b];
    }
  } catch (const SetupError& e) {
    tmp.free_all();
    return obtr_fail(hl, e.code, e.msg);
  } catch (const CudaError& e) {
    tmp.free_all();
    return obtr_fail(hl, SMGPU_ERR_CUDA, std::string("CUDA error ") + cudaGetErrorString(e.err) + " at " + e.what);
  } catch (const std::bad_alloc&) {
    tmp.free_all();
    return obtr_fail(hl, SMGPU_ERR_NOMEM, "host allocation failed");
  }
  tmp.free_all();
  return SMGPU_OK;
}

}  // extern "C"
