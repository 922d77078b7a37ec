// extern "C" entry points for interaction samples that share one basis
// (smgpu_multi_*, declared in include/smgpu.h).
//
// The reference solves such samples one after another: prepEC
// (src/ShellModel/eigenvector_continuation.jl:140-177) re-reads each snt,
// rebuilds the jump tables on the fixed basis and runs TRL.  Here the jump
// tables are built once (every sample must give the same sparsity pattern),
// the S samples' coefficients are interleaved sample-innermost, and all
// samples iterate together: one multi-sample H·V per Lanczos iteration, the
// per-sample recurrences and restarts of multi_lanczos.cu, one CUDA graph per
// restart cycle as in the single-problem driver.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <tuple>
#include <vector>

#include "../../include/smgpu.h"
#include "device.cuh"
#include "lanczos.cuh"
#include "multi.cuh"
#include "problem.h"
#include "setup.h"

struct smgpu_multi {
  int nsamples = 0;
  int S = 0;               // lanes the kernels run with (4, 8 or 16)
  smgpu_problem base;      // basis, structure tables and streams (sample 0)
  DeviceArena coef;        // interleaved coefficients of all samples
  MultiCoef mc{};
  TileTables tt1{};        // one proton row per CTA
  int ntasks1 = 0;
  int cand = 0;            // H·V launch shape (index into hv_multi_candidates)
  double tune_ms[16] = {0};

  void hv(const float* v, double* w, const MultiEpilogue& epi, cudaStream_t st) {
    launch_hv_multi(S, cand, base.dt, tt1, ntasks1, mc, v, w, epi, st);
  }
  void autotune();
  std::string err;
  double times[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  DeviceArena solver;

  ~smgpu_multi() {
    solver.free_all();
    coef.free_all();
  }
};

namespace {
thread_local std::string g_multi_create_error;

double now_s() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

int fail(smgpu_multi* h, int code, const std::string& msg) {
  if (h) h->err = msg;
  else g_multi_create_error = msg;
  return code;
}

template <class F>
int guarded(smgpu_multi* h, F&& f) {
  try {
    return f();
  } catch (const SetupError& e) {
    return fail(h, e.code, e.msg);
  } catch (const CudaError& e) {
    return fail(h, SMGPU_ERR_CUDA,
                std::string("CUDA error ") + cudaGetErrorString(e.err) + " at " + e.what + " (" + e.file + ":" +
                    std::to_string(e.line) + ")");
  } catch (const std::bad_alloc&) {
    return fail(h, SMGPU_ERR_NOMEM, "host allocation failed");
  } catch (const std::exception& e) {
    return fail(h, SMGPU_ERR_ARG, e.what());
  }
}

bool same_links(const std::vector<Tables::Link>& a, const std::vector<Tables::Link>& b) {
  if (a.size() != b.size()) return false;
  for (size_t k = 0; k < a.size(); ++k)
    if (a[k].b != b[k].b || a[k].s != b[k].s || a[k].dm != b[k].dm || a[k].nA != b[k].nA || a[k].nB != b[k].nB ||
        a[k].vtab_off != b[k].vtab_off || a[k].nptr_off != b[k].nptr_off)
      return false;
  return true;
}

// Same basis and the same non-zero pattern of every table the kernels read.
bool same_structure(const Tables& a, const Tables& b) {
  return a.mdim == b.mdim && a.nb == b.nb && a.np == b.np && a.nn == b.nn && a.pbits == b.pbits &&
         a.nbits == b.nbits && a.pp_ptr == b.pp_ptr && a.pp_col == b.pp_col && a.nn_ptr == b.nn_ptr &&
         a.nn_col == b.nn_col && a.link_begin == b.link_begin && same_links(a.links, b.links) &&
         a.ppn_ptr == b.ppn_ptr && a.ppn_src == b.ppn_src && a.ppn_meta == b.ppn_meta && a.npn_ptr == b.npn_ptr &&
         a.npn_ent == b.npn_ent && a.vtab_off_dm == b.vtab_off_dm;
}

// [k*S + s] = sample s's value k; idle lanes repeat sample 0.
template <class TO, class TI>
std::vector<TO> interleave(const std::vector<std::vector<TI>>& per, int S) {
  const size_t n = per[0].size();
  std::vector<TO> out(n * (size_t)S);
  for (int s = 0; s < S; ++s) {
    const std::vector<TI>& src = per[(size_t)s < per.size() ? s : 0];
    for (size_t k = 0; k < n; ++k) out[k * S + s] = (TO)src[k];
  }
  return out;
}

int lanes_for(int nsamples) { return nsamples <= 4 ? 4 : (nsamples <= 8 ? 8 : 16); }

long long graph_kernel_nodes(cudaGraph_t g) {
  size_t nn = 0;
  SMGPU_CUDA_TRY(cudaGraphGetNodes(g, nullptr, &nn));
  std::vector<cudaGraphNode_t> nodes(nn);
  SMGPU_CUDA_TRY(cudaGraphGetNodes(g, nodes.data(), &nn));
  long long nk = 0;
  for (auto nd : nodes) {
    cudaGraphNodeType ty;
    SMGPU_CUDA_TRY(cudaGraphNodeGetType(nd, &ty));
    if (ty == cudaGraphNodeTypeKernel) ++nk;
  }
  return nk;
}

// ---- autotuner cache: (lanes, m-states and valence particles of both
// species, total M) -> launch shape, for the life of the process
typedef std::tuple<int, int, int, int, int, int> MultiKey;
std::mutex g_mtune_mu;
std::map<MultiKey, int> g_mtune;
}  // namespace

// Time every launch shape (3 launches each, the first a warm-up) on a seeded
// device vector and keep the fastest.  SMGPU_AUTOTUNE=0 keeps the default.
void smgpu_multi::autotune() {
  const Tables& T = base.T;
  const MultiKey key{S, T.Lp, T.Ln, base.vp, base.vn, base.mtot2};
  // SMGPU_MULTI_CAND=k selects candidate k of hv_multi_candidates outright
  // (for tests that run every shape)
  if (const char* c = std::getenv("SMGPU_MULTI_CAND")) {
    int nc = 0;
    hv_multi_candidates(&nc);
    const int k = std::atoi(c);
    if (k < 0 || k >= nc) throw SetupError{SMGPU_ERR_ARG, "SMGPU_MULTI_CAND out of range"};
    cand = k;
    return;
  }
  {
    std::lock_guard<std::mutex> lk(g_mtune_mu);
    auto it = g_mtune.find(key);
    if (it != g_mtune.end()) {
      cand = it->second;
      return;
    }
  }
  const char* off = std::getenv("SMGPU_AUTOTUNE");
  if (off && std::string(off) == "0") return;
  const int64_t LS = T.len_pad * S;
  DeviceArena tmp;
  cudaEvent_t a = nullptr, b = nullptr;
  try {
    double* d_start = tmp.alloc<double>(LS);
    float* d_v = tmp.alloc<float>(LS);
    double* d_w = tmp.alloc<double>(LS);
    launch_m_start(S, base.dt, 1234ull, d_start, base.st);
    launch_convert(d_start, d_v, LS, base.st);
    SMGPU_CUDA_TRY(cudaEventCreate(&a));
    SMGPU_CUDA_TRY(cudaEventCreate(&b));
    int nc = 0;
    hv_multi_candidates(&nc);
    int best = 0;
    float best_ms = 1e30f;
    for (int c = 0; c < nc; ++c) {
      cand = c;
      float total = 0.f;
      bool dropped = false;
      for (int rep = 0; rep < 3; ++rep) {
        SMGPU_CUDA_TRY(cudaEventRecord(a, base.st));
        hv(d_v, d_w, MultiEpilogue{}, base.st);
        SMGPU_CUDA_TRY(cudaEventRecord(b, base.st));
        SMGPU_CUDA_TRY(cudaEventSynchronize(b));
        float ms = 0.f;
        SMGPU_CUDA_TRY(cudaEventElapsedTime(&ms, a, b));
        if (rep > 0) total += ms;
        // a warm-up launch over twice the best mean so far: dropped untimed
        if (rep == 0 && best_ms < 1e29f && ms > 2.f * (best_ms / 2)) {
          if (c < 16) tune_ms[c] = ms;
          dropped = true;
          break;
        }
      }
      SMGPU_CUDA_TRY(cudaGetLastError());
      if (dropped) continue;
      if (c < 16) tune_ms[c] = total / 2;
      if (total < best_ms) {
        best_ms = total;
        best = c;
      }
    }
    cand = best;
    std::lock_guard<std::mutex> lk(g_mtune_mu);
    g_mtune[key] = cand;
  } catch (...) {
    if (a) cudaEventDestroy(a);
    if (b) cudaEventDestroy(b);
    tmp.free_all();
    throw;
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  tmp.free_all();
}

namespace {
// ------------------------------------------------------------------ solver
struct MultiSolve {

  smgpu_multi* H;
  MultiDev M{};
  float* V = nullptr;
  float* U = nullptr;
  double* w = nullptr;
  int* hv_count = nullptr;
  long long launches_first = 0, launches_rest = 0;

  int64_t LS() const { return M.len * M.S; }

  void alloc(int lm, int ls, int num_ev, double tol) {
    DeviceArena& A = H->solver;
    A.free_all();
    smgpu_problem& B = H->base;
    const int S = H->S;
    M.S = S;
    M.G = 2 * B.sms;
    M.lm = lm;
    M.ls = ls;
    M.num_ev = num_ev;
    M.nh = 3;
    M.len = B.T.len_pad;
    M.mdim = B.T.mdim;
    M.tol = tol;
    M.nalpha = H->ntasks1;
    const int P = ls * (ls + 1) / 2 + ls;
    const size_t LSz = (size_t)M.len * S;
    V = A.alloc<float>((size_t)lm * LSz);
    U = A.alloc<float>((size_t)ls * LSz);
    w = A.alloc<double>(LSz);
    M.T = A.alloc<double>((size_t)S * lm * lm);
    M.en = A.alloc<double>((size_t)S * M.nh * num_ev);
    M.alpha_part = A.alloc<double>((size_t)lm * S * M.nalpha);
    M.part = A.alloc<double>((size_t)std::max(lm + 2, P) * S * M.G);
    M.h1 = A.alloc<double>((size_t)(lm + 2) * S);
    M.h2 = A.alloc<double>((size_t)(lm + 2) * S);
    M.nrm1 = A.alloc<double>(S);
    M.nrm2 = A.alloc<double>(S);
    M.invb = A.alloc<double>(S);
    M.sec = A.alloc<int>(S);
    M.jacA = A.alloc<double>((size_t)S * lm * lm);
    M.jacZ = A.alloc<double>((size_t)S * lm * lm);
    M.evals = A.alloc<double>((size_t)S * lm);
    M.Yf = A.alloc<float>((size_t)S * (lm - 1) * ls);
    M.wsplit = A.alloc<float>(2 * LSz);
    M.beta2 = A.alloc<float2>(S);
    M.gram = A.alloc<double>((size_t)P * S);
    M.X = A.alloc<double>((size_t)S * ls * ls);
    M.Xf = A.alloc<float>((size_t)S * (ls * ls + ls));
    M.cvec = A.alloc<double>((size_t)S * ls);
    M.fl = A.alloc<LanczosFlags>(S);
    M.ctl = A.alloc<MultiCtl>(1);
    hv_count = A.alloc<int>(1);
    cudaStream_t st = B.st;
    SMGPU_CUDA_TRY(cudaMemsetAsync(V, 0, sizeof(float) * (size_t)lm * LSz, st));
    SMGPU_CUDA_TRY(cudaMemsetAsync(U, 0, sizeof(float) * (size_t)ls * LSz, st));
    SMGPU_CUDA_TRY(cudaMemsetAsync(w, 0, sizeof(double) * LSz, st));
    SMGPU_CUDA_TRY(cudaMemsetAsync(M.wsplit, 0, sizeof(float) * 2 * LSz, st));
    SMGPU_CUDA_TRY(cudaMemsetAsync(M.beta2, 0, sizeof(float2) * S, st));
    SMGPU_CUDA_TRY(cudaMemsetAsync(M.T, 0, sizeof(double) * (size_t)S * lm * lm, st));
    SMGPU_CUDA_TRY(cudaMemsetAsync(M.sec, 0, sizeof(int) * S, st));
    SMGPU_CUDA_TRY(cudaMemsetAsync(hv_count, 0, sizeof(int), st));
    // idle lanes start converged
    std::vector<LanczosFlags> fl(S);
    std::memset(fl.data(), 0, sizeof(LanczosFlags) * S);
    for (int s = H->nsamples; s < S; ++s) fl[s].done = 1;
    MultiCtl ctl{0, S - H->nsamples, 0, 0};
    SMGPU_CUDA_TRY(cudaMemcpyAsync(M.fl, fl.data(), sizeof(LanczosFlags) * S, cudaMemcpyHostToDevice, st));
    SMGPU_CUDA_TRY(cudaMemcpyAsync(M.ctl, &ctl, sizeof(MultiCtl), cudaMemcpyHostToDevice, st));
    std::vector<double> en0((size_t)S * M.nh * num_ev, 1.0e4);
    SMGPU_CUDA_TRY(cudaMemcpyAsync(M.en, en0.data(), sizeof(double) * en0.size(), cudaMemcpyHostToDevice, st));
    SMGPU_CUDA_TRY(cudaStreamSynchronize(st));  // host staging buffers go out of scope
  }

  // One lockstep iteration, `it` 1-based.
  void iteration(int it, int lock, cudaEvent_t ev_fork) {
    smgpu_problem& B = H->base;
    cudaStream_t s = B.st, s2 = B.st2;
    const int it0 = it - 1;
    MultiEpilogue epi{};
    epi.all_done = &M.ctl->all_done;
    epi.alpha_part = M.alpha_part + (size_t)it0 * M.S * M.nalpha;
    epi.count = hv_count;
    if (it0 > lock) {
      epi.vprev = V + (size_t)(it0 - 1) * LS();
      epi.beta_base = M.T + (size_t)(it0 - 1) * M.lm + it0;
      epi.beta_stride = M.lm * M.lm;
    }
    // the residual of the iterations is a double-float pair (wsplit)
    epi.wh = M.wsplit;
    epi.wl = M.wsplit + LS();
    epi.beta2 = M.beta2;
    H->hv(V + (size_t)it0 * LS(), nullptr, epi, s);
    launch_m_alpha(M, it0, s);
    SMGPU_CUDA_TRY(cudaEventRecord(ev_fork, s));
    SMGPU_CUDA_TRY(cudaStreamWaitEvent(s2, ev_fork, 0));
    launch_m_sturm(M, it, lock, s2);
    launch_m_orth(M, V, M.wsplit, M.wsplit + LS(), it0, s);
  }

  cudaGraphExec_t capture_cycle(int kstart, int lock, long long* nkernels) {
    smgpu_problem& B = H->base;
    cudaStream_t s = B.st, s2 = B.st2;
    cudaEvent_t e_fork, e_join;
    SMGPU_CUDA_TRY(cudaEventCreateWithFlags(&e_fork, cudaEventDisableTiming));
    SMGPU_CUDA_TRY(cudaEventCreateWithFlags(&e_join, cudaEventDisableTiming));
    cudaGraph_t g;
    SMGPU_CUDA_TRY(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    for (int it = kstart; it <= M.lm - 1; ++it) iteration(it, lock, e_fork);
    SMGPU_CUDA_TRY(cudaEventRecord(e_join, s2));
    SMGPU_CUDA_TRY(cudaStreamWaitEvent(s, e_join, 0));
    launch_m_cycle_end(M, s);
    launch_m_restart(M, V, U, s);
    SMGPU_CUDA_TRY(cudaStreamEndCapture(s, &g));
    *nkernels = graph_kernel_nodes(g);
    cudaGraphExec_t ex;
    SMGPU_CUDA_TRY(cudaGraphInstantiate(&ex, g, 0));
    cudaGraphDestroy(g);
    cudaEventDestroy(e_fork);
    cudaEventDestroy(e_join);
    return ex;
  }

  int run(int num_ev, int lm, int ls, double tol, int max_restarts, const double* v1, double* evals_out,
          double* evecs_out, int* stats_out) {
    smgpu_problem& B = H->base;
    cudaStream_t st = B.st;
    const int S = H->S, ns = H->nsamples;
    const int64_t mdim = B.T.mdim;
    const int nev = (int)std::min<int64_t>(num_ev, mdim);
    const double tw0 = now_s();
    alloc(lm, ls, num_ev, tol);
    double* v1dev = nullptr;
    if (v1) {
      v1dev = H->solver.alloc<double>((size_t)S * mdim);
      for (int s = 0; s < S; ++s)
        SMGPU_CUDA_TRY(cudaMemcpyAsync(v1dev + (size_t)s * mdim, v1 + (size_t)(s < ns ? s : 0) * mdim,
                                       sizeof(double) * mdim, cudaMemcpyHostToDevice, st));
    }
    const double tc0 = now_s();
    cudaGraphExec_t g_first = capture_cycle(1, 0, &launches_first);
    cudaGraphExec_t g_rest = capture_cycle(ls + 1, ls, &launches_rest);
    H->times[3] = now_s() - tc0;
    cudaEvent_t e0, e1, e2;
    SMGPU_CUDA_TRY(cudaEventCreate(&e0));
    SMGPU_CUDA_TRY(cudaEventCreate(&e1));
    SMGPU_CUDA_TRY(cudaEventCreate(&e2));
    SMGPU_CUDA_TRY(cudaEventRecord(e0, st));
    if (v1dev) launch_m_to_padded(S, B.dt, v1dev, w, st);
    else launch_m_start(S, B.dt, 1234ull, w, st);
    launch_m_init(M, w, V, st);
    long long launches = 4;
    int n_restart = 0, status = SMGPU_OK;
    MultiCtl ctl{};
    SMGPU_CUDA_TRY(cudaGraphLaunch(g_first, st));
    launches += launches_first;
    while (true) {
      SMGPU_CUDA_TRY(cudaMemcpyAsync(&ctl, M.ctl, sizeof(MultiCtl), cudaMemcpyDeviceToHost, st));
      SMGPU_CUDA_TRY(cudaStreamSynchronize(st));
      if (ctl.all_done) break;
      ++n_restart;
      if (n_restart > max_restarts) {
        status = SMGPU_ERR_NOCONV;
        break;
      }
      SMGPU_CUDA_TRY(cudaGraphLaunch(g_rest, st));
      launches += launches_rest;
    }
    std::vector<double> en((size_t)S * M.nh * num_ev);
    std::vector<LanczosFlags> fl(S);
    int n_hv = 0;
    SMGPU_CUDA_TRY(cudaMemcpyAsync(en.data(), M.en, sizeof(double) * en.size(), cudaMemcpyDeviceToHost, st));
    SMGPU_CUDA_TRY(cudaMemcpyAsync(fl.data(), M.fl, sizeof(LanczosFlags) * S, cudaMemcpyDeviceToHost, st));
    SMGPU_CUDA_TRY(cudaMemcpyAsync(&n_hv, hv_count, sizeof(int), cudaMemcpyDeviceToHost, st));
    SMGPU_CUDA_TRY(cudaEventRecord(e1, st));
    SMGPU_CUDA_TRY(cudaStreamSynchronize(st));
    cudaGraphExecDestroy(g_first);
    cudaGraphExecDestroy(g_rest);
    for (int s = 0; s < ns; ++s)
      for (int j = 0; j < nev; ++j) evals_out[(size_t)s * nev + j] = en[(size_t)s * M.nh * num_ev + j];
    for (int s = 0; s < ns; ++s)
      if (fl[s].bad) return fail(H, SMGPU_ERR_DEVICE, "restart Gram matrix was not positive definite");
    if (evecs_out) {
      std::memset(evecs_out, 0, sizeof(double) * (size_t)ns * nev * mdim);
      double* R = H->solver.alloc<double>((size_t)nev * M.len);
      double* tmp = H->solver.alloc<double>(mdim);
      LanczosDev L{};
      L.G = M.G;
      L.len = M.len;
      L.partials = M.part;
      L.h = M.h1;
      for (int s = 0; s < ns; ++s) {
        if (!fl[s].done || fl[s].elit <= 0) continue;
        const int elit = fl[s].elit;
        launch_m_jacobi_one(M, s, elit, st);
        launch_m_ritz(M, V, s, elit, nev, R, st);
        launches += 2;
        for (int e = 0; e < nev; ++e) {
          double* r = R + (size_t)e * M.len;
          launch_multidot<double>(L, r, 1, r, false, st);
          launch_reduce(L, 1, RED_INVNORM, L.h + e, st);
          launch_scale_store<double>(L, r, r, L.h + e, st);
          launch_from_padded(B.dt, r, tmp, st);
          launches += 4;
          SMGPU_CUDA_TRY(cudaMemcpyAsync(evecs_out + ((size_t)s * nev + e) * mdim, tmp, sizeof(double) * mdim,
                                         cudaMemcpyDeviceToHost, st));
        }
      }
    }
    SMGPU_CUDA_TRY(cudaEventRecord(e2, st));
    SMGPU_CUDA_TRY(cudaStreamSynchronize(st));
    SMGPU_CUDA_TRY(cudaGetLastError());
    float ms1 = 0.f, ms2 = 0.f;
    SMGPU_CUDA_TRY(cudaEventElapsedTime(&ms1, e0, e1));
    SMGPU_CUDA_TRY(cudaEventElapsedTime(&ms2, e1, e2));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaEventDestroy(e2);
    bool all = true;
    for (int s = 0; s < ns; ++s) all = all && fl[s].done;
    if (stats_out) {
      stats_out[0] = n_hv;
      stats_out[1] = n_restart;
      stats_out[2] = all ? 1 : 0;
      stats_out[3] = nev;
      stats_out[4] = (int)launches;
      stats_out[5] = S;
      stats_out[6] = 0;
      stats_out[7] = 0;
      for (int s = 0; s < ns; ++s) {
        stats_out[8 + 4 * s] = fl[s].done ? fl[s].elit : 0;
        stats_out[8 + 4 * s + 1] = fl[s].done ? 1 : 0;
        stats_out[8 + 4 * s + 2] = fl[s].n_second;
        stats_out[8 + 4 * s + 3] = 0;
      }
    }
    H->times[1] = ms1 * 1e-3;
    H->times[4] = ms2 * 1e-3;
    H->times[5] = now_s() - tw0;
    return status;
  }
};

}  // namespace

// =========================================================================
extern "C" {

int smgpu_multi_create_from_snt(const char* const* snt_paths, int nsamples, const char* nucleus,
                                smgpu_multi** out) {
  if (!snt_paths || !nucleus || !out || nsamples < 1) return fail(nullptr, SMGPU_ERR_ARG, "bad arguments");
  *out = nullptr;
  if (nsamples > 16) return fail(nullptr, SMGPU_ERR_LIMIT, "at most 16 samples per handle");
  for (int s = 0; s < nsamples; ++s)
    if (!snt_paths[s]) return fail(nullptr, SMGPU_ERR_ARG, "null snt path");
  return guarded(nullptr, [&]() {
    int A = 0, Z = 0;
    parse_nucleus(nucleus, A, Z);
    int ndev = 0;
    cudaError_t ce = cudaGetDeviceCount(&ndev);
    if (ce != cudaSuccess || ndev == 0)
      throw SetupError{SMGPU_ERR_CUDA, "no CUDA device available: the GPU library has no CPU path"};
    const double t0 = now_s();
    smgpu_multi* h = new smgpu_multi();
    try {
      h->nsamples = nsamples;
      h->S = lanes_for(nsamples);
      smgpu_problem& B = h->base;
      B.precision = SMGPU_MIXED;
      const int mtot2 = (A % 2 == 0) ? 0 : 1;  // shellmodel_main.jl:110
      std::vector<std::vector<float>> pp(nsamples), nn(nsamples), vt(nsamples);
      std::vector<std::vector<double>> ep(nsamples), en(nsamples);
      int vp0 = 0, vn0 = 0;
      for (int s = 0; s < nsamples; ++s) {
        Interaction I = read_snt(snt_paths[s], A);
        const int vp = Z - I.cp, vn = (A - Z) - I.cn;
        if (vp < 0 || vn < 0) throw SetupError{SMGPU_ERR_NUCLEUS, "nucleus lies below the snt core"};
        if (s == 0) {
          vp0 = vp;
          vn0 = vn;
          build_tables(I, vp, vn, mtot2, B.T);
          if (B.T.mdim == 0) throw SetupError{SMGPU_ERR_EMPTY, "M-scheme dimension is zero"};
        } else if (vp != vp0 || vn != vn0) {
          throw SetupError{SMGPU_ERR_LIMIT, "interaction samples have different cores"};
        }
        Tables Ts;
        const Tables* T = &B.T;
        if (s > 0) {
          build_tables(I, vp, vn, mtot2, Ts);
          if (!same_structure(B.T, Ts))
            throw SetupError{SMGPU_ERR_LIMIT, "interaction sample " + std::to_string(s) +
                                                  " does not share the non-zero pattern of sample 0"};
          T = &Ts;
        }
        pp[s] = to_f32(T->pp_val);
        nn[s] = to_f32(T->nn_val);
        vt[s] = to_f32(signed_vtab(*T));
        ep[s] = T->ep;
        en[s] = T->en;
      }
      B.vp = vp0;
      B.vn = vn0;
      B.mtot2 = mtot2;
      B.upload();
      B.ensure_tasks(1);
      h->tt1 = B.tt;
      h->tt1.task_b = B.task_arrays[1].first;
      h->tt1.task_p0 = B.task_arrays[1].second;
      h->ntasks1 = B.task_count[1];
      const int S = h->S;
      h->mc.pp_val = h->coef.upload(interleave<float>(pp, S));
      h->mc.nn_val = h->coef.upload(interleave<float>(nn, S));
      h->mc.vtab = h->coef.upload(interleave<float>(vt, S));
      h->mc.ep = h->coef.upload(interleave<double>(ep, S));
      h->mc.en = h->coef.upload(interleave<double>(en, S));
      h->mc.ep2 = h->coef.upload(to_df(interleave<double>(ep, S)));
      h->mc.en2 = h->coef.upload(to_df(interleave<double>(en, S)));
      h->autotune();
      SMGPU_CUDA_TRY(cudaStreamSynchronize(B.st));
      h->times[0] = now_s() - t0;
    } catch (...) {
      delete h;
      throw;
    }
    *out = h;
    return SMGPU_OK;
  });
}

int smgpu_multi_destroy(smgpu_multi* h) {
  delete h;
  return SMGPU_OK;
}

const char* smgpu_multi_last_error(const smgpu_multi* h) { return h ? h->err.c_str() : g_multi_create_error.c_str(); }

int smgpu_multi_dims(const smgpu_multi* h, long long* mdim, int* nsamples, int* lanes) {
  if (!h) return SMGPU_ERR_ARG;
  if (mdim) *mdim = h->base.T.mdim;
  if (nsamples) *nsamples = h->nsamples;
  if (lanes) *lanes = h->S;
  return SMGPU_OK;
}

int smgpu_multi_matvec(smgpu_multi* h, const double* v, double* w, int accumulate) {
  if (!h || !v || !w) return fail(h, SMGPU_ERR_ARG, "bad matvec arguments");
  return guarded(h, [&]() {
    smgpu_problem& B = h->base;
    const int S = h->S, ns = h->nsamples;
    const int64_t mdim = B.T.mdim, LS = B.T.len_pad * S;
    DeviceArena tmp;
    try {
      const double t0 = now_s();
      double* d_in = tmp.alloc<double>((size_t)S * mdim);
      double* d_out = tmp.alloc<double>((size_t)S * mdim);
      float* d_v = tmp.alloc<float>(LS);
      double* d_w = tmp.alloc<double>(LS);
      SMGPU_CUDA_TRY(cudaMemsetAsync(d_in, 0, sizeof(double) * (size_t)S * mdim, B.st));
      SMGPU_CUDA_TRY(cudaMemsetAsync(d_w, 0, sizeof(double) * LS, B.st));
      SMGPU_CUDA_TRY(cudaMemcpyAsync(d_in, v, sizeof(double) * (size_t)ns * mdim, cudaMemcpyHostToDevice, B.st));
      launch_m_to_padded_f(S, B.dt, d_in, d_v, B.st);
      h->hv(d_v, d_w, MultiEpilogue{}, B.st);
      launch_m_from_padded(S, B.dt, d_w, d_out, B.st);
      std::vector<double> host((size_t)ns * mdim);
      SMGPU_CUDA_TRY(cudaMemcpyAsync(host.data(), d_out, sizeof(double) * host.size(), cudaMemcpyDeviceToHost, B.st));
      SMGPU_CUDA_TRY(cudaStreamSynchronize(B.st));
      SMGPU_CUDA_TRY(cudaGetLastError());
      if (accumulate)
        for (size_t i = 0; i < host.size(); ++i) w[i] += host[i];
      else
        std::memcpy(w, host.data(), sizeof(double) * host.size());
      h->times[2] = now_s() - t0;
    } catch (...) {
      tmp.free_all();
      throw;
    }
    tmp.free_all();
    return SMGPU_OK;
  });
}

int smgpu_multi_solve(smgpu_multi* h, int num_ev, int lm, int ls, double tol, int max_restarts, const double* v1,
                      double* evals_out, double* evecs_out, int* stats_out) {
  if (!h || !evals_out) return fail(h, SMGPU_ERR_ARG, "null argument");
  if (num_ev < 1 || lm < 3 || ls < 1 || ls > lm - 2 || ls > 60 || lm > 1000 || num_ev > lm - 1 || !(tol > 0.0))
    return fail(h, SMGPU_ERR_ARG, "need 1 <= num_ev < lm, 1 <= ls <= min(lm-2, 60), lm <= 1000, tol > 0");
  return guarded(h, [&]() {
    MultiSolve solve{h};
    return solve.run(num_ev, lm, ls, tol, max_restarts, v1, evals_out, evecs_out, stats_out);
  });
}

int smgpu_multi_stats(const smgpu_multi* h, long long* s) {
  if (!h || !s) return SMGPU_ERR_ARG;
  int nc = 0;
  const MultiHvConfig* c = hv_multi_candidates(&nc);
  const Tables& T = h->base.T;
  s[0] = T.updates;
  s[1] = h->S;
  s[2] = (long long)(h->base.tables.bytes + h->coef.bytes);
  s[3] = (long long)T.len_pad;
  s[4] = h->ntasks1;
  s[5] = c[h->cand].nt;
  s[6] = c[h->cand].minb;
  s[7] = c[h->cand].km;
  return SMGPU_OK;
}

int smgpu_multi_timings(const smgpu_multi* h, double* t) {
  if (!h || !t) return SMGPU_ERR_ARG;
  for (int k = 0; k < 8; ++k) t[k] = h->times[k];
  return SMGPU_OK;
}

int smgpu_multi_time_matvec(smgpu_multi* h, int reps, int flush_l2, double* ms_out) {
  if (!h || !ms_out || reps < 1) return fail(h, SMGPU_ERR_ARG, "bad time_matvec arguments");
  return guarded(h, [&]() {
    smgpu_problem& B = h->base;
    const int S = h->S;
    const int64_t LS = B.T.len_pad * S;
    DeviceArena tmp;
    cudaEvent_t a = nullptr, b = nullptr;
    try {
      double* d_start = tmp.alloc<double>(LS);
      float* d_v = tmp.alloc<float>(LS);
      double* d_w = tmp.alloc<double>(LS);
      char* flush = flush_l2 ? tmp.alloc<char>(256u << 20) : nullptr;
      launch_m_start(S, B.dt, 1234ull, d_start, B.st);
      launch_convert(d_start, d_v, LS, B.st);
      SMGPU_CUDA_TRY(cudaEventCreate(&a));
      SMGPU_CUDA_TRY(cudaEventCreate(&b));
      double total = 0.0;
      for (int r = 0; r < reps; ++r) {
        if (flush) SMGPU_CUDA_TRY(cudaMemsetAsync(flush, r & 0xff, 256u << 20, B.st));
        SMGPU_CUDA_TRY(cudaEventRecord(a, B.st));
        h->hv(d_v, d_w, MultiEpilogue{}, B.st);
        SMGPU_CUDA_TRY(cudaEventRecord(b, B.st));
        SMGPU_CUDA_TRY(cudaEventSynchronize(b));
        float ms = 0.f;
        SMGPU_CUDA_TRY(cudaEventElapsedTime(&ms, a, b));
        total += ms;
      }
      SMGPU_CUDA_TRY(cudaGetLastError());
      *ms_out = total / reps;
    } catch (...) {
      if (a) cudaEventDestroy(a);
      if (b) cudaEventDestroy(b);
      tmp.free_all();
      throw;
    }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    tmp.free_all();
    return SMGPU_OK;
  });
}

}  // extern "C"
