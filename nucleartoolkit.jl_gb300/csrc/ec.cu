// Transition densities of eigenvector continuation (prepEC mode "TD",
// src/ShellModel/eigenvector_continuation.jl:212-310 with calcOBTD, prepTBTD
// and calcTBTD, :1035-1380).
//
// The reference accumulates, for every pair of sample vectors (i <= j), the
// one-body densities Σ_M w_i[M] w_j[M] occ_o(M) per orbit and, per snt TBME
// line, the two-body densities of the line's m-scheme operators (its
// hermitian partner included).  Both are the derivatives of <w_i|H|w_j> with
// respect to the SPE of the orbit and the value of the line: H is linear in
// them, so the TD of unit u (an orbit or a line) is <w_i|H_u|w_j> with H_u
// the Hamiltonian of the interaction whose only non-zero entry is u = 1 (no
// mass scaling).  Here each H_u is set up on the sample basis like any
// interaction (device enumeration of its tables) and applied with the FP64
// H·v kernel to all sample vectors; the overlaps come from the pair-dot
// kernels.  Nothing of the TD computation runs on the host but the set-up.
#include <string>
#include <vector>

#include "../../include/smgpu.h"
#include "lanczos.cuh"
#include "pairdots.cuh"
#include "problem.h"

using namespace smgpu;

namespace {

Interaction unit_interaction(const Interaction& I, int u) {
  Interaction J;
  J.lp = I.lp;
  J.ln = I.ln;
  J.cp = I.cp;
  J.cn = I.cn;
  J.porb = I.porb;
  J.norb = I.norb;
  J.spe_p.assign(I.lp, 0.0);
  J.spe_n.assign(I.ln, 0.0);
  J.nlines = I.nlines;
  if (u < I.lp) {
    J.spe_p[u] = 1.0;
  } else if (u < I.lp + I.ln) {
    J.spe_n[u - I.lp] = 1.0;
  } else {
    const int line = u - I.lp - I.ln + 1;
    for (int k = 0; k < 3; ++k)
      for (const auto& t : I.tb[k])
        if (t.line == line) {
          Interaction::TB x = t;
          x.v = 1.0;
          J.tb[k].push_back(x);
        }
  }
  return J;
}

int ec_fail(smgpu_problem* h, int code, const std::string& msg) {
  if (h) h->err = msg;
  return code;
}

}  // namespace

extern "C" {

int smgpu_ec_td_length(const smgpu_problem* h, int* ltd) {
  if (!h || !ltd) return SMGPU_ERR_ARG;
  *ltd = h->I.lp + h->I.ln + h->I.nlines;
  return SMGPU_OK;
}

int smgpu_ec_td(smgpu_problem* h, const double* vecs, int nvec, double* nmat_out, double* td_out) {
  if (!h || !vecs || nvec < 1 || !nmat_out || !td_out) return ec_fail(h, SMGPU_ERR_ARG, "bad ec_td arguments");
  if ((int64_t)nvec * nvec > 65535) return ec_fail(h, SMGPU_ERR_LIMIT, "at most 255 sample vectors");
  if (h->I.nlines > 0) {
    bool have_lines = false;
    for (int k = 0; k < 3; ++k)
      for (const auto& t : h->I.tb[k]) have_lines |= t.line > 0;
    if (!have_lines) return ec_fail(h, SMGPU_ERR_ARG, "the handle's interaction carries no snt line numbers");
  }
  const int ltd = h->I.lp + h->I.ln + h->I.nlines;
  const int64_t mdim = h->T.mdim, len = h->T.len_pad;
  const int npair = nvec * (nvec + 1) / 2;
  DeviceArena tmp;
  try {
    cudaStream_t st = h->st;
    double* d_w = tmp.alloc<double>((size_t)nvec * mdim);
    double* d_pad = tmp.alloc<double>((size_t)nvec * len);
    double* d_hv = tmp.alloc<double>((size_t)len);
    double* d_out = tmp.alloc<double>((size_t)nvec * mdim);
    double* d_part = tmp.alloc<double>((size_t)nvec * nvec * pair_dot_chunks(mdim));
    double* d_dot = tmp.alloc<double>((size_t)nvec * nvec);
    std::vector<double> m((size_t)nvec * nvec);
    SMGPU_CUDA_TRY(cudaMemcpyAsync(d_w, vecs, sizeof(double) * nvec * mdim, cudaMemcpyHostToDevice, st));
    SMGPU_CUDA_TRY(cudaMemsetAsync(d_pad, 0, sizeof(double) * nvec * len, st));
    for (int j = 0; j < nvec; ++j) launch_to_padded<double>(h->dt, d_w + (size_t)j * mdim, d_pad + (size_t)j * len, st);
    // overlap matrix (Nmat)
    launch_pair_dots(d_w, nvec, d_w, nvec, mdim, d_part, d_dot, st);
    SMGPU_CUDA_TRY(cudaMemcpyAsync(nmat_out, d_dot, sizeof(double) * nvec * nvec, cudaMemcpyDeviceToHost, st));
    SMGPU_CUDA_TRY(cudaStreamSynchronize(st));
    for (int u = 0; u < ltd; ++u) {
      smgpu_problem q;
      q.precision = SMGPU_FP64;
      q.vp = h->vp;
      q.vn = h->vn;
      q.mtot2 = h->mtot2;
      q.I = unit_interaction(h->I, u);
      build_tables(q.I, h->vp, h->vn, h->mtot2, q.T);
      if (q.T.mdim != mdim || q.T.pbits != h->T.pbits || q.T.nbits != h->T.nbits || q.T.stride != h->T.stride)
        throw SetupError{SMGPU_ERR_DEVICE, "unit interaction basis differs from the sample basis"};
      q.upload(false);
      for (int j = 0; j < nvec; ++j) {
        SMGPU_CUDA_TRY(cudaMemsetAsync(d_hv, 0, sizeof(double) * len, st));
        q.hv((const double*)(d_pad + (size_t)j * len), d_hv, HvEpilogue<double>{}, st);
        launch_from_padded(q.dt, d_hv, d_out + (size_t)j * mdim, st);
      }
      launch_pair_dots(d_w, nvec, d_out, nvec, mdim, d_part, d_dot, st);
      SMGPU_CUDA_TRY(cudaMemcpyAsync(m.data(), d_dot, sizeof(double) * nvec * nvec, cudaMemcpyDeviceToHost, st));
      SMGPU_CUDA_TRY(cudaStreamSynchronize(st));
      // pairs i <= j in idx_from_ij order (shellmodel_main.jl:1297-1299)
      int p = 0;
      for (int i = 0; i < nvec; ++i)
        for (int j = i; j < nvec; ++j, ++p) td_out[(size_t)p * ltd + u] = m[(size_t)i * nvec + j];
    }
    (void)npair;
  } catch (const SetupError& e) {
    tmp.free_all();
    return ec_fail(h, e.code, e.msg);
  } catch (const CudaError& e) {
    tmp.free_all();
    return ec_fail(h, SMGPU_ERR_CUDA, std::string("CUDA error ") + cudaGetErrorString(e.err) + " at " + e.what);
  } catch (const std::bad_alloc&) {
    tmp.free_all();
    return ec_fail(h, SMGPU_ERR_NOMEM, "host allocation failed");
  }
  tmp.free_all();
  return SMGPU_OK;
}

}  // extern "C"
