// extern "C" entry points of libsmgpu.so (declared in include/smgpu.h).
//
// A handle owns one problem: the host tables from setup.cpp, their device
// copies, and (during smgpu_solve) the Krylov basis.  The Lanczos iteration
// of one restart cycle — H·v with its α/three-term epilogue, the eigenvalue
// test, the re-orthogonalisation passes, β, the next basis vector and the
// thick restart — is captured once as a CUDA graph and replayed until the
// device-side convergence flag is set; the host reads that flag once per
// cycle.  The eigenvalue test of iteration k runs on a second stream,
// concurrently with the re-orthogonalisation of iteration k and the H·v of
// iteration k+1.
//
// H·v launch shape (threads per CTA, rows per CTA) is chosen per problem by a
// small autotuner that times the candidate shapes on the device; results are
// cached per shape class (precision, m-states and valence particles of both
// species, total M) for the life of the process, and in the file named by
// SMGPU_TUNE_CACHE when that variable is set.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
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
#include "setup.h"
#include "problem.h"

using namespace smgpu;

namespace {
thread_local std::string g_create_error;

double now_s() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}


// ---- autotuner cache: shape class -> (threads, rows, min CTAs per SM, staged)
typedef std::tuple<int, int, int, int, int, int> ShapeKey;  // precision, Lp, Ln, vp, vn, mtot2
std::mutex g_tune_mu;
std::map<ShapeKey, std::tuple<int, int, int, int>> g_tune;
bool g_tune_file_loaded = false;

void tune_file_load() {
  if (g_tune_file_loaded) return;
  g_tune_file_loaded = true;
  const char* path = std::getenv("SMGPU_TUNE_CACHE");
  if (!path) return;
  FILE* f = std::fopen(path, "r");
  if (!f) return;
  int a[10];
  while (std::fscanf(f, "%d %d %d %d %d %d %d %d %d %d", &a[0], &a[1], &a[2], &a[3], &a[4], &a[5], &a[6], &a[7],
                     &a[8], &a[9]) == 10)
    g_tune[ShapeKey{a[0], a[1], a[2], a[3], a[4], a[5]}] = std::make_tuple(a[6], a[7], a[8], a[9]);
  std::fclose(f);
}
void tune_file_store() {
  const char* path = std::getenv("SMGPU_TUNE_CACHE");
  if (!path) return;
  FILE* f = std::fopen(path, "w");
  if (!f) return;
  for (auto& kv : g_tune)
    std::fprintf(f, "%d %d %d %d %d %d %d %d %d %d\n", std::get<0>(kv.first), std::get<1>(kv.first),
                 std::get<2>(kv.first), std::get<3>(kv.first), std::get<4>(kv.first), std::get<5>(kv.first),
                 std::get<0>(kv.second), std::get<1>(kv.second), std::get<2>(kv.second), std::get<3>(kv.second));
  std::fclose(f);
}
}  // namespace

void smgpu_problem::autotune() {
  // both FP32-mixed forms run the same H·v kernels: one cache entry
  ShapeKey key{precision == SMGPU_FP64 ? SMGPU_FP64 : SMGPU_MIXED, T.Lp, T.Ln, vp, vn, mtot2};
  // SMGPU_HV_SHAPE="threads,rows,min_ctas,staged" selects one candidate
  // launch shape outright (for tests that run every shape); unknown or
  // non-fitting shapes are an error.
  if (const char* shape = std::getenv("SMGPU_HV_SHAPE")) {
    HvConfig want{0, 0, 0, 0, 0};
    if (std::sscanf(shape, "%d,%d,%d,%d", &want.nt, &want.rows, &want.minb, &want.staged) != 4)
      throw SetupError{SMGPU_ERR_ARG, "SMGPU_HV_SHAPE must be threads,rows,min_ctas,staged"};
    int n0 = 0, n1 = 0;
    const HvConfig* c0 = hv_candidates(&n0);
    const HvConfig* c1 = hv_staged_candidates(&n1);
    bool known = false;
    for (int k = 0; k < n0 && !known; ++k)
      known = !want.staged && c0[k].nt == want.nt && c0[k].rows == want.rows && c0[k].minb == want.minb;
    for (int k = 0; k < n1 && !known; ++k)
      known = want.staged && precision != SMGPU_FP64 && c1[k].nt == want.nt && c1[k].rows == want.rows &&
              c1[k].minb == want.minb && hv_staged_fits(c1[k], tt, nnmax_raw);
    if (!known) throw SetupError{SMGPU_ERR_ARG, "SMGPU_HV_SHAPE is not a candidate shape for this problem"};
    set_config(want.nt, want.rows, want.minb, want.staged);
    return;
  }
  // SMGPU_HV_FORM=tile|staged restricts the candidates to one H·v kernel form
  // (and bypasses the shape cache); unset, both forms compete.
  const char* form_env = std::getenv("SMGPU_HV_FORM");
  const std::string form = form_env ? form_env : "";
  const bool forced = form == "tile" || form == "staged";
  if (!forced) {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    tune_file_load();
    auto it = g_tune.find(key);
    if (it != g_tune.end()) {
      set_config(std::get<0>(it->second), std::get<1>(it->second), std::get<2>(it->second), std::get<3>(it->second));
      return;
    }
  }
  const char* off = std::getenv("SMGPU_AUTOTUNE");
  if (off && std::string(off) == "0") return;
  DeviceArena tmp;
  cudaEvent_t a = nullptr, b = nullptr;
  try {
    double* d_start = tmp.alloc<double>(T.len_pad);
    double* d_w = tmp.alloc<double>(T.len_pad);
    void* d_v = (precision == SMGPU_FP64) ? (void*)tmp.alloc<double>(T.len_pad) : (void*)tmp.alloc<float>(T.len_pad);
    launch_start_vector(dt, 1234ull, d_start, st);
    if (precision == SMGPU_FP64)
      SMGPU_CUDA_TRY(cudaMemcpyAsync(d_v, d_start, sizeof(double) * T.len_pad, cudaMemcpyDeviceToDevice, st));
    else
      launch_convert(d_start, (float*)d_v, T.len_pad, st);
    SMGPU_CUDA_TRY(cudaEventCreate(&a));
    SMGPU_CUDA_TRY(cudaEventCreate(&b));
    int nc0 = 0, ns = 0;
    const HvConfig* c0 = hv_candidates(&nc0);
    const HvConfig* cs = hv_staged_candidates(&ns);
    // staged shapes first: usually the fastest, so the row-tile shapes
    // behind them are mostly dropped after their first launch (below)
    std::vector<HvConfig> cand;
    if (precision != SMGPU_FP64 && form != "tile")
      for (int k = 0; k < ns; ++k)
        if (hv_staged_fits(cs[k], tt, nnmax_raw)) cand.push_back(cs[k]);
    if (form != "staged" || precision == SMGPU_FP64) cand.insert(cand.end(), c0, c0 + nc0);
    if (cand.empty()) cand.assign(c0, c0 + nc0);  // the staged form does not fit this problem
    const int nc = (int)cand.size();
    tune_shapes = cand;
    tune_ms.assign(nc, 0.0);
    int best = -1;
    float best_ms = 1e30f;
    for (int c = 0; c < nc; ++c) {
      set_config(cand[c].nt, cand[c].rows, cand[c].minb, cand[c].staged);
      float total = 0.f;
      bool dropped = false;
      for (int rep = 0; rep < 3; ++rep) {
        SMGPU_CUDA_TRY(cudaEventRecord(a, st));
        if (precision == SMGPU_FP64) hv((const double*)d_v, d_w, HvEpilogue<double>{}, st);
        else hv((const float*)d_v, d_w, HvEpilogue<float>{}, st);
        SMGPU_CUDA_TRY(cudaEventRecord(b, st));
        SMGPU_CUDA_TRY(cudaEventSynchronize(b));
        float ms = 0.f;
        SMGPU_CUDA_TRY(cudaEventElapsedTime(&ms, a, b));
        if (rep > 0) total += ms;  // first launch is the warm-up
        // a shape whose warm-up launch already takes more than twice the
        // best time so far cannot win: dropped without the timed launches
        if (rep == 0 && best >= 0 && ms > 2.f * (best_ms / 2)) {
          tune_ms[c] = ms;
          dropped = true;
          break;
        }
      }
      SMGPU_CUDA_TRY(cudaGetLastError());
      if (dropped) continue;
      tune_ms[c] = total / 2;
      if (total < best_ms) {
        best_ms = total;
        best = c;
      }
    }
    set_config(cand[best].nt, cand[best].rows, cand[best].minb, cand[best].staged);
    if (!forced) {
      std::lock_guard<std::mutex> lk(g_tune_mu);
      g_tune[key] = std::make_tuple(cfg.nt, cfg.rows, cfg.minb, cfg.staged);
      tune_file_store();
    }
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

int fail(smgpu_problem* h, int code, const std::string& msg) {
  if (h) h->err = msg;
  else g_create_error = msg;
  return code;
}

template <class F>
int guarded(smgpu_problem* h, F&& f) {
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

int create_common(const Interaction& I, int vp, int vn, int mtot2, int precision, smgpu_problem** out) {
  if (precision != SMGPU_FP64 && precision != SMGPU_MIXED && precision != SMGPU_MIXED_DF)
    throw SetupError{SMGPU_ERR_ARG, "unknown precision"};
  int ndev = 0;
  cudaError_t ce = cudaGetDeviceCount(&ndev);
  if (ce != cudaSuccess || ndev == 0)
    throw SetupError{SMGPU_ERR_CUDA, "no CUDA device available: the GPU library has no CPU path"};
  smgpu_problem* h = new smgpu_problem();
  try {
    h->precision = precision;
    h->I = I;
    h->vp = vp;
    h->vn = vn;
    h->mtot2 = mtot2;
    double t0 = now_s();
    build_tables(I, vp, vn, mtot2, h->T);
    if (h->T.mdim == 0) throw SetupError{SMGPU_ERR_EMPTY, "M-scheme dimension is zero"};
    const double t1 = now_s();
    h->upload();
    h->autotune();
    SMGPU_CUDA_TRY(cudaStreamSynchronize(h->st));
    h->times[0] = now_s() - t0;
    h->times[6] = t1 - t0;
    h->times[7] = now_s() - t1;
  } catch (...) {
    delete h;
    throw;
  }
  *out = h;
  return SMGPU_OK;
}

// J^2 as an FP64 operator on the basis of h (built on first use).
smgpu_problem* ensure_jj_op(smgpu_problem* h) {
  if (!h->jj_op) {
    smgpu_problem* q = new smgpu_problem();
    try {
      q->precision = SMGPU_FP64;
      q->vp = h->vp;
      q->vn = h->vn;
      q->mtot2 = h->mtot2;
      q->I = jj_interaction(h->I);
      build_tables(q->I, h->vp, h->vn, h->mtot2, q->T);
      if (q->T.mdim != h->T.mdim || q->T.pbits != h->T.pbits || q->T.nbits != h->T.nbits ||
          q->T.stride != h->T.stride)
        throw SetupError{SMGPU_ERR_DEVICE, "J^2 basis differs from the problem's basis"};
      q->upload(false);
    } catch (...) {
      delete q;
      throw;
    }
    h->jj_op = q;
  }
  return h->jj_op;
}

// ------------------------------------------------------------------ solver
template <class TX>
struct Solve {
  smgpu_problem* P;
  LanczosDev L{};
  TX* V = nullptr;
  TX* U = nullptr;
  double* w = nullptr;
  long long launches_first = 0, launches_rest = 0;
  // FP32 basis only: true runs the residual, re-orthogonalisation and the
  // restart's small dense algebra in double-float (SMGPU_MIXED_DF), false in
  // FP64 (SMGPU_MIXED)
  bool df = false;
  bool dfs() const { return sizeof(TX) == 4 && df; }
  // FP32 basis, FP64 arithmetic: the restart and Ritz eigenproblems by the
  // FP64 Jacobi started from an FP32 Jacobi's eigenbasis
  bool refj() const { return sizeof(TX) == 4 && !df; }

  void alloc(int lm, int ls, int num_ev, double tol) {
    DeviceArena& A = P->solver;
    A.free_all();
    L.G = 2 * P->sms;
    L.lm = lm;
    L.ls = ls;
    L.num_ev = num_ev;
    L.nh = 3;
    L.len = P->T.len_pad;
    L.mdim = P->T.mdim;
    L.tol = tol;
    L.nalpha = P->cfg.ntasks;
    const int P_gram = ls * (ls + 1) / 2 + ls;
    const int npart = std::max(lm + 2, P_gram) + 2;
    V = A.alloc<TX>((size_t)lm * L.len);
    U = A.alloc<TX>((size_t)ls * L.len);
    w = A.alloc<double>(L.len);
    L.T = A.alloc<double>((size_t)lm * lm);
    L.en = A.alloc<double>((size_t)L.nh * num_ev);
    L.alpha_part = A.alloc<double>((size_t)lm * L.nalpha);
    L.pdot = A.alloc<double>((size_t)(lm + 2) * L.G);
    L.pn1 = A.alloc<double>(L.G);
    L.pdot2 = A.alloc<double>((size_t)(lm + 2) * L.G);
    L.pn2 = A.alloc<double>(L.G);
    L.partials = A.alloc<double>((size_t)npart * L.G);
    L.h = A.alloc<double>(lm + 2);
    L.jacA = A.alloc<double>((size_t)lm * lm);
    L.jacZ = A.alloc<double>((size_t)lm * lm);
    L.evals = A.alloc<double>(lm);
    L.Yf = A.alloc<float>((size_t)lm * ls);
    L.wsplit = dfs() ? A.alloc<float>(2 * (size_t)L.len) : nullptr;
    L.gram = A.alloc<double>(P_gram);
    L.X = A.alloc<double>((size_t)ls * ls);
    L.cvec = A.alloc<double>(ls);
    L.sc = A.alloc<LanczosScalars>(1);
    L.fl = A.alloc<LanczosFlags>(1);
    L.alpha_df = dfs() ? 1 : 0;  // the double-float solve runs the double-float H·v epilogue
    L.fastnorm = fastnorm_threshold();
    SMGPU_CUDA_TRY(cudaMemsetAsync(V, 0, sizeof(TX) * (size_t)lm * L.len, P->st));
    SMGPU_CUDA_TRY(cudaMemsetAsync(w, 0, sizeof(double) * L.len, P->st));
    // the padding slots of the double-float residual are never written by H·v
    if (L.wsplit) SMGPU_CUDA_TRY(cudaMemsetAsync(L.wsplit, 0, sizeof(float) * 2 * L.len, P->st));
    SMGPU_CUDA_TRY(cudaMemsetAsync(L.T, 0, sizeof(double) * (size_t)lm * lm, P->st));
    SMGPU_CUDA_TRY(cudaMemsetAsync(L.sc, 0, sizeof(LanczosScalars), P->st));
    SMGPU_CUDA_TRY(cudaMemsetAsync(L.fl, 0, sizeof(LanczosFlags), P->st));
    std::vector<double> en0((size_t)L.nh * num_ev, 1.0e4);
    SMGPU_CUDA_TRY(cudaMemcpyAsync(L.en, en0.data(), sizeof(double) * en0.size(), cudaMemcpyHostToDevice, P->st));
  }

  // v1 -> V[0] normalised (start vector in w on entry)
  void init_start() {
    launch_multidot<double>(L, w, 1, w, false, P->st);
    launch_reduce(L, 1, RED_INVNORM, L.h, P->st);
    launch_scale_store<TX>(L, w, V, L.h, P->st);
  }

  // One Lanczos iteration, `it` 1-based (lanczos_methods.jl:34-62).
  void iteration(int it, int lock, cudaEvent_t ev_fork) {
    cudaStream_t s = P->st, s2 = P->st2;
    const int it0 = it - 1;
    TX* vk = V + (size_t)it0 * L.len;
    HvEpilogue<TX> epi{};
    epi.fl = L.fl;
    epi.alpha_part = L.alpha_part + (size_t)it0 * L.nalpha;
    if (it0 > lock) {
      // three-term correction; the first iteration after a restart couples to
      // every kept Ritz vector and is left to the Gram-Schmidt passes
      epi.vprev = V + (size_t)(it0 - 1) * L.len;
      epi.beta = L.T + (size_t)(it0 - 1) * L.lm + it0;
    }
    if constexpr (sizeof(TX) == 4) {
      // FP32 basis: the residual w is FP64, or a double-float pair (wsplit)
      if (df) P->hv_df(vk, L.wsplit, L.wsplit + L.len, epi, s);
      else P->hv(vk, w, epi, s);
    } else {
      P->hv(vk, w, epi, s);
    }
    SMGPU_CUDA_TRY(cudaEventRecord(ev_fork, s));
    SMGPU_CUDA_TRY(cudaStreamWaitEvent(s2, ev_fork, 0));
    launch_sturm(L, it, lock, s2);
    if (dfs()) {
      launch_orth_iteration_df(L, reinterpret_cast<float*>(V), L.wsplit, L.wsplit + L.len, it0, s);
    } else {
      launch_orth_iteration<TX>(L, V, w, it0, s);
    }
  }

  void restart(cudaStream_t s) {
    // ThickRestart (lanczos_methods.jl:260-307)
    launch_jacobi(L, L.lm - 1, true, dfs(), refj(), s);
    launch_restart_small(L, s);
    launch_restart_rotate<TX>(L, V, U, s);
    launch_gram<TX>(L, U, V + (size_t)(L.lm - 1) * L.len, dfs(), s);
    launch_gram_reduce(L, dfs(), s);
    launch_chol(L, dfs(), s);
    // the updated basis is stored in FP32: for an FP32 basis the update runs
    // in compensated FP32, as the rotation does
    launch_restart_apply<TX>(L, U, V, sizeof(TX) == 4, s);
  }

  cudaGraphExec_t capture_cycle(int kstart, int lock, long long* nkernels) {
    cudaStream_t s = P->st, s2 = P->st2;
    cudaEvent_t e_fork, e_join;
    SMGPU_CUDA_TRY(cudaEventCreateWithFlags(&e_fork, cudaEventDisableTiming));
    SMGPU_CUDA_TRY(cudaEventCreateWithFlags(&e_join, cudaEventDisableTiming));
    cudaGraph_t g;
    SMGPU_CUDA_TRY(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    for (int it = kstart; it <= L.lm - 1; ++it) iteration(it, lock, e_fork);
    SMGPU_CUDA_TRY(cudaEventRecord(e_join, s2));
    SMGPU_CUDA_TRY(cudaStreamWaitEvent(s, e_join, 0));
    restart(s);
    SMGPU_CUDA_TRY(cudaStreamEndCapture(s, &g));
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
    *nkernels = nk;
    cudaGraphExec_t ex;
    SMGPU_CUDA_TRY(cudaGraphInstantiate(&ex, g, 0));
    cudaGraphDestroy(g);
    cudaEventDestroy(e_fork);
    cudaEventDestroy(e_join);
    return ex;
  }

  // ---- J projection (doubleLanczos, lanczos_methods.jl:1-151): an inner
  // Lanczos on J^2 = J-J+ + M(M+1) (the basis has M = J) projects every new
  // Krylov vector onto J.  Vector work on the device, the small matrices of
  // the inner Lanczos on the host with their eigen-decompositions on the
  // device; control flow as the reference's Jlanczos / ThickRestart_J.
  smgpu_problem* Jop = nullptr;
  double eval_jj = -1.0;
  int lnJ = 0;
  double* Q = nullptr;    // lnJ x len inner Krylov vectors (FP64)
  double* jx = nullptr;   // combination / projected vector
  double* js = nullptr;   // device dot products (lm + 2)
  double* jn = nullptr;   // device norms (2)
  double* jT = nullptr;   // small matrix for the device eigensolver
  double* jA = nullptr;
  double* jZ = nullptr;
  double* jev = nullptr;
  std::vector<double> Jm;  // inner Lanczos matrix (host, lnJ x lnJ, column-major)

  void alloc_j(int ls) {
    DeviceArena& A = P->solver;
    lnJ = ls;
    Q = A.alloc<double>((size_t)lnJ * L.len);
    jx = A.alloc<double>(L.len);
    js = A.alloc<double>((size_t)L.lm + 2);
    jn = A.alloc<double>(2);
    jT = A.alloc<double>((size_t)lnJ * lnJ);
    jA = A.alloc<double>((size_t)lnJ * lnJ);
    jZ = A.alloc<double>((size_t)lnJ * lnJ);
    jev = A.alloc<double>(lnJ);
    SMGPU_CUDA_TRY(cudaMemsetAsync(Q, 0, sizeof(double) * (size_t)lnJ * L.len, P->st));
  }
  double host_scalar(const double* d) {
    double x = 0.0;
    SMGPU_CUDA_TRY(cudaMemcpyAsync(&x, d, sizeof(double), cudaMemcpyDeviceToHost, P->st));
    SMGPU_CUDA_TRY(cudaStreamSynchronize(P->st));
    return x;
  }
  // eigenvalues (ascending) and eigenvectors (column-major) of Jm[0:n,0:n]
  void small_eig(int n, std::vector<double>& vals, std::vector<double>* vecs) {
    std::vector<double> sub((size_t)n * n);
    for (int j = 0; j < n; ++j)
      for (int i = 0; i < n; ++i) sub[(size_t)j * n + i] = Jm[(size_t)j * lnJ + i];
    SMGPU_CUDA_TRY(cudaMemcpyAsync(jT, sub.data(), sizeof(double) * sub.size(), cudaMemcpyHostToDevice, P->st));
    launch_small_eig(jT, n, jA, jZ, jev, P->st);
    vals.resize(n);
    SMGPU_CUDA_TRY(cudaMemcpyAsync(vals.data(), jev, sizeof(double) * n, cudaMemcpyDeviceToHost, P->st));
    if (vecs) {
      vecs->resize((size_t)n * n);
      SMGPU_CUDA_TRY(cudaMemcpyAsync(vecs->data(), jA, sizeof(double) * n * n, cudaMemcpyDeviceToHost, P->st));
    }
    SMGPU_CUDA_TRY(cudaStreamSynchronize(P->st));
  }
  // y -= its components along the first m columns of X (two CGS passes)
  template <class TY>
  void cgs(const TY* X, int m, double* y) {
    for (int pass = 0; pass < 2 && m > 0; ++pass) {
      launch_multidot<TY>(L, X, m, y, false, P->st);
      launch_reduce(L, m, RED_STORE, js, P->st);
      launch_axpy_dev<TY>(X, L.len, m, js, y, L.len, P->st);
    }
  }
  // ||y||; y /= ||y|| into out
  template <class TO>
  double normalize(const double* y, TO* out) {
    launch_multidot<double>(L, y, 1, y, false, P->st);
    launch_reduce(L, 1, RED_STORE, jn, P->st);
    launch_reduce(L, 1, RED_INVNORM, jn + 1, P->st);
    launch_scale_store<TO>(L, y, out, jn + 1, P->st);
    return std::sqrt(host_scalar(jn));
  }
  // lanczos_methods.jl:132-151 with ls = 1 (the arrow element goes to row 2
  // and column k, as in the reference)
  void thick_restart_j(int lmj) {
    const int m = lmj - 1;
    std::vector<double> vals, vecs;
    small_eig(m, vals, &vecs);
    int k = 0;
    for (int i = 1; i < m; ++i)
      if (std::fabs(vals[i] - eval_jj) < std::fabs(vals[k] - eval_jj)) k = i;
    const double beta = Jm[(size_t)(lmj - 1) * lnJ + (lmj - 2)];
    std::fill(Jm.begin(), Jm.end(), 0.0);
    Jm[0] = vals[k];
    const double tmp = beta * vecs[(size_t)k * m + (m - 1)];
    Jm[(size_t)k * lnJ + 1] = tmp;
    Jm[(size_t)1 * lnJ + k] = tmp;
    SMGPU_CUDA_TRY(cudaMemcpyAsync(js, vecs.data() + (size_t)k * m, sizeof(double) * m, cudaMemcpyHostToDevice, P->st));
    launch_combine(Q, L.len, m, js, jx, L.len, P->st);
    normalize<double>(jx, Q);
    if (lmj - 1 != 1)
      SMGPU_CUDA_TRY(cudaMemcpyAsync(Q + L.len, Q + (size_t)(lmj - 1) * L.len, sizeof(double) * L.len,
                                     cudaMemcpyDeviceToDevice, P->st));
    if (lnJ > 2)
      SMGPU_CUDA_TRY(cudaMemsetAsync(Q + 2 * L.len, 0, sizeof(double) * (size_t)(lnJ - 2) * L.len, P->st));
  }
  // lanczos_methods.jl:93-131 Jlanczos on Q[0] (Q[0] returns the projection)
  void jlanczos() {
    const double Jtol = 1.e-7;
    Jm.assign((size_t)lnJ * lnJ, 0.0);
    auto JM = [&](int i, int j) -> double& { return Jm[(size_t)(j - 1) * lnJ + (i - 1)]; };
    int eljit = 1, k = 1, inow = k, rounds = 0;
    bool JTF = false;
    std::vector<double> vals;
    while (!JTF) {
      if (++rounds > 1000) throw SetupError{SMGPU_ERR_NOCONV, "J projection did not converge"};
      for (int it = k; it <= lnJ - 1; ++it) {
        inow = it;
        double* vk = Q + (size_t)(it - 1) * L.len;
        double* vkp1 = Q + (size_t)it * L.len;
        Jop->hv((const double*)vk, vkp1, HvEpilogue<double>{}, P->st);  // J^2 vk = (J-J+ + eval_jj) vk
        launch_multidot<double>(L, vk, 1, vkp1, false, P->st);
        launch_reduce(L, 1, RED_STORE, js, P->st);
        JM(it, it) = host_scalar(js);
        small_eig(it, vals, nullptr);
        if (std::fabs(vals[0] - eval_jj) < Jtol) {
          eljit = it;
          JTF = true;
          break;
        }
        cgs<double>(Q, it, vkp1);
        const double beta = normalize<double>(vkp1, vkp1);
        JM(it + 1, it) = beta;
        JM(it, it + 1) = beta;
        eljit = it;
      }
      if (!JTF) {
        thick_restart_j(eljit + 1);
        k = 2;
      }
    }
    if (inow > k) thick_restart_j(eljit + 1);
  }
  // Krylov vector `slot` := its J projection, re-orthogonalised against the
  // slots before it and normalised (lanczos_methods.jl:24-28,64-76).
  void project(int slot) {
    TX* v = V + (size_t)slot * L.len;
    if (lnJ > 1)
      SMGPU_CUDA_TRY(cudaMemsetAsync(Q + L.len, 0, sizeof(double) * (size_t)(lnJ - 1) * L.len, P->st));
    launch_widen<TX>(v, Q, L.len, P->st);
    jlanczos();
    SMGPU_CUDA_TRY(cudaMemcpyAsync(jx, Q, sizeof(double) * L.len, cudaMemcpyDeviceToDevice, P->st));
    cgs<TX>(V, slot, jx);
    normalize<TX>(jx, v);
  }

  int run_projected(int num_ev, int lm, int ls, double tol, int max_restarts, const double* v1,
                    double* evals_out, double* evecs_out, int* stats_out) {
    const int64_t mdim = P->T.mdim;
    const int nev = (int)std::min<int64_t>(num_ev, mdim);
    const double tw0 = now_s();
    alloc(lm, ls, num_ev, tol);
    alloc_j(ls);
    cudaStream_t s = P->st, s2 = P->st2;
    double* v1dev = nullptr;
    if (v1) {
      v1dev = P->solver.alloc<double>(mdim);
      SMGPU_CUDA_TRY(cudaMemcpyAsync(v1dev, v1, sizeof(double) * mdim, cudaMemcpyHostToDevice, s));
    }
    cudaEvent_t e0, e1, e2, e_fork;
    SMGPU_CUDA_TRY(cudaEventCreate(&e0));
    SMGPU_CUDA_TRY(cudaEventCreate(&e1));
    SMGPU_CUDA_TRY(cudaEventCreate(&e2));
    SMGPU_CUDA_TRY(cudaEventCreateWithFlags(&e_fork, cudaEventDisableTiming));
    SMGPU_CUDA_TRY(cudaEventRecord(e0, s));
    if (v1dev) launch_to_padded<double>(P->dt, v1dev, w, s);
    else launch_start_vector(P->dt, 1234ull, w, s);
    init_start();
    // the start vector is projected and normalised (lanczos_methods.jl:24-28)
    launch_widen<TX>(V, Q, L.len, s);
    jlanczos();
    normalize<TX>(Q, V);
    int n_restart = 0, status = SMGPU_OK, elit = 0, n_hv = 0;
    bool done = false;
    LanczosFlags fl{};
    int kstart = 1, lock = 0;
    while (true) {
      for (int it = kstart; it <= lm - 1; ++it) {
        iteration(it, lock, e_fork);
        ++n_hv;
        SMGPU_CUDA_TRY(cudaStreamSynchronize(s2));
        SMGPU_CUDA_TRY(cudaMemcpyAsync(&fl, L.fl, sizeof(LanczosFlags), cudaMemcpyDeviceToHost, s));
        SMGPU_CUDA_TRY(cudaStreamSynchronize(s));
        if (fl.done) {
          done = true;
          elit = fl.elit;
          break;
        }
        if (fl.exhausted) {
          done = true;
          elit = fl.exh_k;
          break;
        }
        const double tbeta = host_scalar(L.T + (size_t)(it - 1) * lm + it);
        if (tbeta < 1.e-7) {  // lanczos_methods.jl:65
          done = true;
          elit = it;
          break;
        }
        project(it);
      }
      if (done) break;
      ++n_restart;
      if (n_restart > max_restarts) {
        status = SMGPU_ERR_NOCONV;
        break;
      }
      restart(s);
      kstart = ls + 1;
      lock = ls;
    }
    SMGPU_CUDA_TRY(cudaMemcpyAsync(evals_out, L.en, sizeof(double) * nev, cudaMemcpyDeviceToHost, s));
    SMGPU_CUDA_TRY(cudaEventRecord(e1, s));
    SMGPU_CUDA_TRY(cudaStreamSynchronize(s));
    if (status == SMGPU_ERR_NOCONV) elit = 0;
    long long launches = 0;
    if (evecs_out && elit > 0) {
      double* R = P->solver.alloc<double>((size_t)nev * L.len);
      double* tmp = P->solver.alloc<double>(mdim);
      launch_jacobi(L, elit, false, dfs(), refj(), s);
      launch_ritz<TX>(L, V, elit, nev, R, s);
      for (int e = 0; e < nev; ++e) {
        double* r = R + (size_t)e * L.len;
        launch_multidot<double>(L, r, 1, r, false, s);
        launch_reduce(L, 1, RED_INVNORM, L.h + e, s);
        launch_scale_store<double>(L, r, r, L.h + e, s);
        launch_from_padded(P->dt, r, tmp, s);
        SMGPU_CUDA_TRY(cudaMemcpyAsync(evecs_out + (size_t)e * mdim, tmp, sizeof(double) * mdim,
                                       cudaMemcpyDeviceToHost, s));
      }
    }
    SMGPU_CUDA_TRY(cudaEventRecord(e2, s));
    SMGPU_CUDA_TRY(cudaStreamSynchronize(s));
    SMGPU_CUDA_TRY(cudaGetLastError());
    float ms1 = 0.f, ms2 = 0.f;
    SMGPU_CUDA_TRY(cudaEventElapsedTime(&ms1, e0, e1));
    SMGPU_CUDA_TRY(cudaEventElapsedTime(&ms2, e1, e2));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaEventDestroy(e2);
    cudaEventDestroy(e_fork);
    if (fl.bad) return fail(P, SMGPU_ERR_DEVICE, "restart Gram matrix was not positive definite");
    if (stats_out) {
      stats_out[0] = elit;
      stats_out[1] = n_hv;
      stats_out[2] = n_restart;
      stats_out[3] = done ? 1 : 0;
      stats_out[4] = nev;
      stats_out[5] = fl.n_second;
      stats_out[6] = (int)launches;
      stats_out[7] = 0;
    }
    P->times[1] = ms1 * 1e-3;
    P->times[4] = ms2 * 1e-3;
    P->times[5] = now_s() - tw0;
    return status;
  }

  int run(int num_ev, int lm, int ls, double tol, int max_restarts, const double* v1, double* evals_out,
          double* evecs_out, int* stats_out) {
    const int64_t mdim = P->T.mdim;
    const int nev = (int)std::min<int64_t>(num_ev, mdim);
    double tw0 = now_s();
    alloc(lm, ls, num_ev, tol);
    double* v1dev = nullptr;
    if (v1) {
      v1dev = P->solver.alloc<double>(mdim);
      SMGPU_CUDA_TRY(cudaMemcpyAsync(v1dev, v1, sizeof(double) * mdim, cudaMemcpyHostToDevice, P->st));
    }
    double tc0 = now_s();
    cudaGraphExec_t g_first = capture_cycle(1, 0, &launches_first);
    cudaGraphExec_t g_rest = capture_cycle(ls + 1, ls, &launches_rest);
    P->times[3] = now_s() - tc0;
    cudaEvent_t e0, e1, e2;
    SMGPU_CUDA_TRY(cudaEventCreate(&e0));
    SMGPU_CUDA_TRY(cudaEventCreate(&e1));
    SMGPU_CUDA_TRY(cudaEventCreate(&e2));
    SMGPU_CUDA_TRY(cudaEventRecord(e0, P->st));
    if (v1dev) launch_to_padded<double>(P->dt, v1dev, w, P->st);
    else launch_start_vector(P->dt, 1234ull, w, P->st);
    init_start();
    long long launches = 4;
    int n_restart = 0, status = SMGPU_OK;
    LanczosFlags fl{};
    SMGPU_CUDA_TRY(cudaGraphLaunch(g_first, P->st));
    launches += launches_first;
    while (true) {
      SMGPU_CUDA_TRY(cudaMemcpyAsync(&fl, L.fl, sizeof(LanczosFlags), cudaMemcpyDeviceToHost, P->st));
      SMGPU_CUDA_TRY(cudaStreamSynchronize(P->st));
      if (fl.done) break;
      if (fl.exhausted) {
        fl.done = 1;
        fl.elit = fl.exh_k;
        break;
      }
      ++n_restart;
      if (n_restart > max_restarts) {
        status = SMGPU_ERR_NOCONV;
        fl.elit = lm - 1;
        break;
      }
      SMGPU_CUDA_TRY(cudaGraphLaunch(g_rest, P->st));
      launches += launches_rest;
    }
    // eigenvalues: en[1] of the last eigenvalue test (main_sm returns en[1])
    SMGPU_CUDA_TRY(cudaMemcpyAsync(evals_out, L.en, sizeof(double) * nev, cudaMemcpyDeviceToHost, P->st));
    SMGPU_CUDA_TRY(cudaEventRecord(e1, P->st));
    SMGPU_CUDA_TRY(cudaStreamSynchronize(P->st));
    cudaGraphExecDestroy(g_first);
    cudaGraphExecDestroy(g_rest);
    if (fl.bad) return fail(P, SMGPU_ERR_DEVICE, "restart Gram matrix was not positive definite");
    int elit = fl.elit;
    if (status == SMGPU_ERR_NOCONV) elit = 0;
    if (evecs_out && elit > 0) {
      // Ritz vectors (shellmodel_main.jl:208-224)
      double* R = P->solver.alloc<double>((size_t)nev * L.len);
      double* tmp = P->solver.alloc<double>(mdim);
      launch_jacobi(L, elit, false, dfs(), refj(), P->st);
      launch_ritz<TX>(L, V, elit, nev, R, P->st);
      launches += 2;
      for (int e = 0; e < nev; ++e) {
        double* r = R + (size_t)e * L.len;
        launch_multidot<double>(L, r, 1, r, false, P->st);
        launch_reduce(L, 1, RED_INVNORM, L.h + e, P->st);
        launch_scale_store<double>(L, r, r, L.h + e, P->st);
        launch_from_padded(P->dt, r, tmp, P->st);
        launches += 4;
        SMGPU_CUDA_TRY(cudaMemcpyAsync(evecs_out + (size_t)e * mdim, tmp, sizeof(double) * mdim,
                                       cudaMemcpyDeviceToHost, P->st));
      }
    }
    SMGPU_CUDA_TRY(cudaEventRecord(e2, P->st));
    SMGPU_CUDA_TRY(cudaStreamSynchronize(P->st));
    SMGPU_CUDA_TRY(cudaGetLastError());
    float ms1 = 0.f, ms2 = 0.f;
    SMGPU_CUDA_TRY(cudaEventElapsedTime(&ms1, e0, e1));
    SMGPU_CUDA_TRY(cudaEventElapsedTime(&ms2, e1, e2));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaEventDestroy(e2);
    if (stats_out) {
      int n_hv = 0;
      // iterations executed: first cycle 1..lm-1, later cycles ls+1..lm-1
      if (fl.done) {
        n_hv = (n_restart == 0) ? elit : (lm - 1) + (n_restart - 1) * (lm - 1 - ls) + (elit - ls);
      } else {
        n_hv = (lm - 1) + (n_restart - 1) * (lm - 1 - ls);
      }
      stats_out[0] = elit;
      stats_out[1] = n_hv;
      stats_out[2] = n_restart;
      stats_out[3] = fl.done ? 1 : 0;
      stats_out[4] = nev;
      stats_out[5] = fl.n_second;
      stats_out[6] = (int)launches;
      stats_out[7] = 0;
    }
    P->times[1] = ms1 * 1e-3;
    P->times[4] = ms2 * 1e-3;
    P->times[5] = now_s() - tw0;
    return status;
  }
};

// ------------------------------------------------------------------ block
// Block thick-restart Lanczos TRBL (lanczos_methods.jl:312-423) with q
// vectors per block, FP64: bl_operate_H! as q H·v launches, bl_ReORTH
// (:425-436), bl_QR! (shellmodel_main.jl:1049-1066), add_bl_T! (:1201-1205),
// bl_ThickRestart (lanczos_methods.jl:647-716) and the block Ritz vectors
// (shellmodel_main.jl:208-224).  Vector work (H·v, dot products, updates,
// combinations) on the device; the block T matrix is kept on the host and
// diagonalised on the device every iteration; control flow on the host.
struct BlockSolve {
  smgpu_problem* P;
  int q = 2;
  LanczosDev L{};
  double* V = nullptr;   // nblk*q vectors of len
  double* U = nullptr;   // ls_sub*q vectors
  double* w = nullptr;
  double* js = nullptr;  // device scalars
  double* dT = nullptr;  // small matrix for the eigensolver
  double* dA = nullptr;
  double* dZ = nullptr;
  double* dev = nullptr;
  std::vector<double> T;  // lm x lm, column-major (host)
  int lm = 0;

  double* vec(int slot) { return V + (size_t)slot * L.len; }
  double host(const double* d) {
    double x = 0.0;
    SMGPU_CUDA_TRY(cudaMemcpyAsync(&x, d, sizeof(double), cudaMemcpyDeviceToHost, P->st));
    SMGPU_CUDA_TRY(cudaStreamSynchronize(P->st));
    return x;
  }
  double& Tm(int i, int j) { return T[(size_t)(j - 1) * lm + (i - 1)]; }  // 1-based
  // eigenvalues (ascending) and, if vecs, eigenvectors of T[1:n,1:n]
  void eig(int n, std::vector<double>& vals, std::vector<double>* vecs) {
    std::vector<double> sub((size_t)n * n);
    for (int j = 1; j <= n; ++j)
      for (int i = 1; i <= n; ++i) sub[(size_t)(j - 1) * n + (i - 1)] = Tm(i, j);
    SMGPU_CUDA_TRY(cudaMemcpyAsync(dT, sub.data(), sizeof(double) * sub.size(), cudaMemcpyHostToDevice, P->st));
    launch_small_eig(dT, n, dA, dZ, dev, P->st);
    vals.resize(n);
    SMGPU_CUDA_TRY(cudaMemcpyAsync(vals.data(), dev, sizeof(double) * n, cudaMemcpyDeviceToHost, P->st));
    if (vecs) {
      vecs->resize((size_t)n * n);
      SMGPU_CUDA_TRY(cudaMemcpyAsync(vecs->data(), dA, sizeof(double) * n * n, cudaMemcpyDeviceToHost, P->st));
    }
    SMGPU_CUDA_TRY(cudaStreamSynchronize(P->st));
  }
  // js[0..m) = X_j . y for the m vectors at X
  void dots(const double* X, int m, const double* y) {
    launch_multidot<double>(L, X, m, y, false, P->st);
    launch_reduce(L, m, RED_STORE, js, P->st);
  }
  // y -= sum_j js[j] X_j
  void sub(const double* X, int m, double* y) { launch_axpy_dev<double>(X, L.len, m, js, y, L.len, P->st); }
  // bl_QR! on the q vectors at slot0 (modified Gram-Schmidt); R (q x q, R[j*q+k]) on the host
  void qr(int slot0, std::vector<double>& R) {
    R.assign((size_t)q * q, 0.0);
    for (int j = 0; j < q; ++j) {
      double* qj = vec(slot0 + j);
      launch_multidot<double>(L, qj, 1, qj, false, P->st);
      launch_reduce(L, 1, RED_STORE, js + q, P->st);
      launch_reduce(L, 1, RED_INVNORM, js + q + 1, P->st);
      launch_scale_store<double>(L, qj, qj, js + q + 1, P->st);
      R[(size_t)j * q + j] = std::sqrt(host(js + q));
      for (int k = j + 1; k < q; ++k) {
        dots(qj, 1, vec(slot0 + k));
        R[(size_t)j * q + k] = host(js);
        sub(qj, 1, vec(slot0 + k));
      }
    }
  }

  int run(int q_, int num_ev, int lm_, int ls, double tol, int max_restarts, const double* v1, double* evals_out,
          double* evecs_out, int* stats_out) {
    q = q_;
    lm = lm_;
    const int64_t mdim = P->T.mdim;
    const int nev = (int)std::min<int64_t>(num_ev, mdim);
    const int ls_sub = ls / q, itmax = lm / q - 1, nblk = lm / q;
    const double tw0 = now_s();
    DeviceArena& A = P->solver;
    A.free_all();
    L.G = 2 * P->sms;
    L.len = P->T.len_pad;
    L.partials = A.alloc<double>((size_t)(q + 3) * L.G);
    V = A.alloc<double>((size_t)nblk * q * L.len);
    U = A.alloc<double>((size_t)std::max(1, ls_sub * q) * L.len);
    w = A.alloc<double>(L.len);
    js = A.alloc<double>((size_t)std::max(q * q, lm) + 8);
    dT = A.alloc<double>((size_t)lm * lm);
    dA = A.alloc<double>((size_t)lm * lm);
    dZ = A.alloc<double>((size_t)lm * lm);
    dev = A.alloc<double>(lm);
    cudaStream_t st = P->st;
    SMGPU_CUDA_TRY(cudaMemsetAsync(V, 0, sizeof(double) * (size_t)nblk * q * L.len, st));
    T.assign((size_t)lm * lm, 0.0);
    std::vector<std::vector<double>> en(3, std::vector<double>(num_ev, 1.0e4));
    cudaEvent_t e0, e1, e2;
    SMGPU_CUDA_TRY(cudaEventCreate(&e0));
    SMGPU_CUDA_TRY(cudaEventCreate(&e1));
    SMGPU_CUDA_TRY(cudaEventCreate(&e2));
    double* v1dev = nullptr;
    if (v1) {
      v1dev = A.alloc<double>((size_t)q * mdim);
      SMGPU_CUDA_TRY(cudaMemcpyAsync(v1dev, v1, sizeof(double) * q * mdim, cudaMemcpyHostToDevice, st));
    }
    SMGPU_CUDA_TRY(cudaEventRecord(e0, st));
    // start block: initialize_bl_wav (shellmodel_main.jl:950-965) + bl_QR!
    for (int i = 0; i < q; ++i) {
      if (v1dev) launch_to_padded<double>(P->dt, v1dev + (size_t)i * mdim, vec(i), st);
      else launch_start_vector(P->dt, 1234ull + (uint64_t)i, vec(i), st);
      for (int k = i - 1; k >= 0; --k) {
        dots(vec(k), 1, vec(i));
        sub(vec(k), 1, vec(i));
      }
      launch_multidot<double>(L, vec(i), 1, vec(i), false, st);
      launch_reduce(L, 1, RED_INVNORM, js + q + 1, st);
      launch_scale_store<double>(L, vec(i), vec(i), js + q + 1, st);
    }
    std::vector<double> Beta;
    qr(0, Beta);
    bool TF = false;
    int elit = 1, inow = 1, itmin = 1, n_restart = 0, n_hv = 0, status = SMGPU_OK;
    std::vector<double> vals, vecs, Rm((size_t)q * q);
    while (!TF) {
      for (int it = itmin; it <= itmax; ++it) {
        inow = it;
        const int v0 = (it - 1) * q, h0 = it * q;
        for (int i = 0; i < q; ++i) P->hv((const double*)vec(v0 + i), vec(h0 + i), HvEpilogue<double>{}, st);
        n_hv += q;
        for (int i = 0; i < q; ++i) {  // js[i*q + j] = V_i . HV_j
          launch_multidot<double>(L, vec(h0), q, vec(v0 + i), false, st);
          launch_reduce(L, q, RED_STORE, js + (size_t)i * q, st);
        }
        SMGPU_CUDA_TRY(cudaMemcpyAsync(Rm.data(), js, sizeof(double) * q * q, cudaMemcpyDeviceToHost, st));
        SMGPU_CUDA_TRY(cudaStreamSynchronize(st));
        bool sym = true;  // Rm[i*q+j] = V_i . HV_j
        for (int i = 0; i < q; ++i)
          for (int j = 0; j < q; ++j)
            if (Rm[(size_t)i * q + j] != Rm[(size_t)j * q + i]) sym = false;
        if (!sym)
          for (int i = 0; i < q; ++i)
            for (int j = i; j < q; ++j) Rm[(size_t)i * q + j] = Rm[(size_t)j * q + i];
        for (int i = 0; i < q; ++i)
          for (int j = 0; j < q; ++j) Tm(q * it - q + 1 + i, q * it - q + 1 + j) = Rm[(size_t)i * q + j];
        // diagonalize_T!(it*q) (lanczos_methods.jl:250-258)
        const int kk = it * q;
        eig(kk, vals, nullptr);
        for (int h = 2; h >= 1; --h) en[h] = en[h - 1];
        for (int i = 0; i < std::min(num_ev, kk); ++i) en[0][i] = vals[i];
        bool ok = true;
        for (int i = 0; i < num_ev; ++i)
          if (!(en[1][i] - en[0][i] < tol)) ok = false;
        if (ok) TF = true;
        // HV -= R V, bl_ReORTH, bl_QR!, add_bl_T!
        SMGPU_CUDA_TRY(cudaMemcpyAsync(js, Rm.data(), sizeof(double) * q * q, cudaMemcpyHostToDevice, st));
        for (int i = 0; i < q; ++i)
          launch_axpy_dev<double>(vec(v0), L.len, q, js + (size_t)i * q, vec(h0 + i), L.len, st);
        for (int l = it - 1; l >= 1; --l)
          for (int i = 0; i < q; ++i) {
            dots(vec((l - 1) * q), q, vec(h0 + i));
            sub(vec((l - 1) * q), q, vec(h0 + i));
          }
        qr(h0, Beta);
        for (int i = 0; i < q; ++i)
          for (int j = 0; j < q; ++j) {
            Tm(q * it + 1 + i, q * it - q + 1 + j) = Beta[(size_t)i * q + j];
            Tm(q * it - q + 1 + j, q * it + 1 + i) = Beta[(size_t)i * q + j];
          }
        if (TF) {
          elit = it;
          break;
        }
      }
      if (TF) break;
      ++n_restart;
      if (n_restart > max_restarts) {
        status = SMGPU_ERR_NOCONV;
        break;
      }
      // bl_ThickRestart (lanczos_methods.jl:647-716)
      const int lmq = q * inow, lsq = q * ls_sub;
      eig(lmq, vals, &vecs);
      auto VV = [&](int row, int col) { return vecs[(size_t)(col - 1) * lmq + (row - 1)]; };
      std::fill(T.begin(), T.end(), 0.0);
      for (int k = 1; k <= lsq; ++k) Tm(k, k) = vals[k - 1];
      for (int a = 1; a <= q; ++a)
        for (int k = 1; k <= lsq; ++k) {
          double r = 0.0;
          for (int b = 1; b <= q; ++b) r += Beta[(size_t)(a - 1) * q + (b - 1)] * VV(lmq - q + b, k);
          Tm(lsq + a, k) = r;
          Tm(k, lsq + a) = r;
        }
      for (int k = 1; k <= lsq; ++k) {
        SMGPU_CUDA_TRY(cudaMemcpyAsync(js, vecs.data() + (size_t)(k - 1) * lmq, sizeof(double) * lmq,
                                       cudaMemcpyHostToDevice, st));
        launch_combine(V, L.len, lmq, js, U + (size_t)(k - 1) * L.len, L.len, st);
      }
      SMGPU_CUDA_TRY(cudaMemcpyAsync(V, U, sizeof(double) * (size_t)lsq * L.len, cudaMemcpyDeviceToDevice, st));
      SMGPU_CUDA_TRY(cudaMemcpyAsync(vec(ls_sub * q), vec(inow * q), sizeof(double) * (size_t)q * L.len,
                                     cudaMemcpyDeviceToDevice, st));
      if (nblk > ls_sub + 1)
        SMGPU_CUDA_TRY(cudaMemsetAsync(vec((ls_sub + 1) * q), 0,
                                       sizeof(double) * (size_t)(nblk - ls_sub - 1) * q * L.len, st));
      for (int i = 2; i <= ls_sub + 1; ++i) {
        for (int j = i - 1; j >= 1; --j)
          for (int a = 0; a < q; ++a) {
            dots(vec((j - 1) * q), q, vec((i - 1) * q + a));
            sub(vec((j - 1) * q), q, vec((i - 1) * q + a));
          }
        qr((i - 1) * q, Beta);
      }
      itmin = ls_sub + 1;
    }
    for (int i = 0; i < nev; ++i) evals_out[i] = en[0][i];
    SMGPU_CUDA_TRY(cudaEventRecord(e1, st));
    if (evecs_out && TF) {
      const int m = elit * q;
      eig(m, vals, &vecs);
      double* R = A.alloc<double>(L.len);
      double* tmp = A.alloc<double>(mdim);
      for (int e = 0; e < nev; ++e) {
        SMGPU_CUDA_TRY(cudaMemcpyAsync(js, vecs.data() + (size_t)e * m, sizeof(double) * m, cudaMemcpyHostToDevice,
                                       st));
        launch_combine(V, L.len, m, js, R, L.len, st);
        launch_multidot<double>(L, R, 1, R, false, st);
        launch_reduce(L, 1, RED_INVNORM, js + q + 1, st);
        launch_scale_store<double>(L, R, R, js + q + 1, st);
        launch_from_padded(P->dt, R, tmp, st);
        SMGPU_CUDA_TRY(cudaMemcpyAsync(evecs_out + (size_t)e * mdim, tmp, sizeof(double) * mdim,
                                       cudaMemcpyDeviceToHost, st));
        SMGPU_CUDA_TRY(cudaStreamSynchronize(st));
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
    if (stats_out) {
      stats_out[0] = elit;
      stats_out[1] = n_hv;
      stats_out[2] = n_restart;
      stats_out[3] = TF ? 1 : 0;
      stats_out[4] = nev;
      stats_out[5] = 0;
      stats_out[6] = 0;
      stats_out[7] = q;
    }
    P->times[1] = ms1 * 1e-3;
    P->times[4] = ms2 * 1e-3;
    P->times[5] = now_s() - tw0;
    return status;
  }
};

}  // namespace

// =========================================================================
extern "C" {

int smgpu_problem_create_from_snt(const char* snt_path, const char* nucleus, int precision, smgpu_problem** out) {
  if (!snt_path || !nucleus || !out) return fail(nullptr, SMGPU_ERR_ARG, "null argument");
  *out = nullptr;
  return guarded(nullptr, [&]() {
    int A = 0, Z = 0;
    parse_nucleus(nucleus, A, Z);
    Interaction I = read_snt(snt_path, A);
    int vp = Z - I.cp, vn = (A - Z) - I.cn;
    if (vp < 0 || vn < 0) throw SetupError{SMGPU_ERR_NUCLEUS, "nucleus lies below the snt core"};
    int mtot2 = (A % 2 == 0) ? 0 : 1;  // shellmodel_main.jl:110
    return create_common(I, vp, vn, mtot2, precision, out);
  });
}

int smgpu_problem_create_from_snt_J(const char* snt_path, const char* nucleus, int twoJ, int precision,
                                    smgpu_problem** out) {
  if (!snt_path || !nucleus || !out || twoJ < 0) return fail(nullptr, SMGPU_ERR_ARG, "null argument or negative 2J");
  *out = nullptr;
  return guarded(nullptr, [&]() {
    int A = 0, Z = 0;
    parse_nucleus(nucleus, A, Z);
    if (A % 2 != twoJ % 2) throw SetupError{SMGPU_ERR_NUCLEUS, "invalid target J for this nucleus"};  // :116
    Interaction I = read_snt(snt_path, A);
    int vp = Z - I.cp, vn = (A - Z) - I.cn;
    if (vp < 0 || vn < 0) throw SetupError{SMGPU_ERR_NUCLEUS, "nucleus lies below the snt core"};
    return create_common(I, vp, vn, twoJ, precision, out);  // Mtot = tJ (:113)
  });
}

int smgpu_problem_create(const smgpu_problem_desc* d, int precision, smgpu_problem** out) {
  if (!d || !out || !d->orbits || !d->spe || (d->ntbme > 0 && (!d->tbme_labels || !d->tbme)))
    return fail(nullptr, SMGPU_ERR_ARG, "null argument");
  *out = nullptr;
  return guarded(nullptr, [&]() {
    Interaction I;
    I.lp = d->lp;
    I.ln = d->ln;
    if (I.lp <= 0 || I.ln <= 0) throw SetupError{SMGPU_ERR_ARG, "bad orbit counts"};
    for (int k = 0; k < I.lp + I.ln; ++k) {
      Orbit o{d->orbits[4 * k], d->orbits[4 * k + 1], d->orbits[4 * k + 2], d->orbits[4 * k + 3]};
      if (k < I.lp) { I.porb.push_back(o); I.spe_p.push_back(d->spe[k]); }
      else { I.norb.push_back(o); I.spe_n.push_back(d->spe[k]); }
    }
    for (int k = 0; k < d->ntbme; ++k) {
      const int* l = d->tbme_labels + 5 * k;
      int a = l[0], b = l[1], c = l[2], dd = l[3];
      int lim = I.lp + I.ln;
      if (a < 1 || b < 1 || c < 1 || dd < 1 || a > lim || b > lim || c > lim || dd > lim)
        throw SetupError{SMGPU_ERR_ARG, "TBME orbit index out of range"};
      int kind;
      if (a <= I.lp && b <= I.lp) kind = 0;
      else if (a > I.lp && b > I.lp) kind = 1;
      else if (a <= I.lp && b > I.lp) kind = 2;
      else throw SetupError{SMGPU_ERR_ARG, "TBME with the proton index after the neutron index"};
      if (d->hermitian_partners) {
        bool same = (a == b) ? (c == dd && c == a) : (c != dd && a == c && b == dd);
        if (!same) I.tb[kind].push_back({c, dd, a, b, l[4], d->tbme[k], k + 1});
      }
      I.tb[kind].push_back({a, b, c, dd, l[4], d->tbme[k], k + 1});
    }
    I.nlines = d->ntbme;
    return create_common(I, d->vp, d->vn, d->mtot2, precision, out);
  });
}

int smgpu_problem_destroy(smgpu_problem* h) {
  delete h;
  return SMGPU_OK;
}

const char* smgpu_last_error(const smgpu_problem* h) { return h ? h->err.c_str() : g_create_error.c_str(); }

int smgpu_dims(const smgpu_problem* h, long long* mdim, int* nblocks, long long* tdims_out) {
  if (!h) return SMGPU_ERR_ARG;
  if (mdim) *mdim = h->T.mdim;
  if (nblocks) *nblocks = h->T.nb;
  if (tdims_out)
    for (int b = 0; b <= h->T.nb; ++b) tdims_out[b] = h->T.tdims[b];
  return SMGPU_OK;
}

int smgpu_blocks(const smgpu_problem* h, int* np, int* nn, int* mp2, int* mn2) {
  if (!h) return SMGPU_ERR_ARG;
  for (int b = 0; b < h->T.nb; ++b) {
    if (np) np[b] = h->T.np[b];
    if (nn) nn[b] = h->T.nn[b];
    if (mp2) mp2[b] = h->T.mp2[b];
    if (mn2) mn2[b] = h->T.mn2[b];
  }
  return SMGPU_OK;
}

int smgpu_export_basis(const smgpu_problem* h, unsigned long long* pbits, unsigned long long* nbits) {
  if (!h) return SMGPU_ERR_ARG;
  if (pbits) std::memcpy(pbits, h->T.pbits.data(), sizeof(uint64_t) * h->T.pbits.size());
  if (nbits) std::memcpy(nbits, h->T.nbits.data(), sizeof(uint64_t) * h->T.nbits.size());
  return SMGPU_OK;
}

int smgpu_export_jumps(const smgpu_problem* h, int which, long long* count, long long* ints, double* coef) {
  if (!h || !count) return SMGPU_ERR_ARG;
  const Tables& T = h->T;
  long long c = 0;
  if (which == 0 || which == 1) {
    // forward links only (source block >= output block) = the reference's lists
    for (int b = 0; b < T.nb; ++b)
      for (int li = T.link_begin[b]; li < T.link_begin[b + 1]; ++li) {
        const auto& L = T.links[li];
        if (L.s < L.b) continue;
        if (which == 0) {
          for (int g = T.pstart[b]; g < T.pstart[b + 1]; ++g)
            for (int k = T.ppn_ptr[g]; k < T.ppn_ptr[g + 1]; ++k) {
              uint32_t meta = T.ppn_meta[k];
              if ((int)(meta >> 16) != li) continue;
              if (ints) {
                int ia = (meta >> 1) & 0x7fff;
                long long* e = ints + 7 * c;
                e[0] = b + 1; e[1] = L.s + 1;
                e[2] = (long long)T.Aops_dm[L.dm][2 * ia]; e[3] = (long long)T.Aops_dm[L.dm][2 * ia + 1];
                e[4] = g - T.pstart[b] + 1; e[5] = (long long)T.ppn_src[k] + 1;
                e[6] = (meta & 1) ? 0 : 1;  // reference phase flag: true for an even count
              }
              ++c;
            }
        } else {
          for (int n = 0; n < T.nn[b]; ++n)
            for (int64_t j = T.npn_ptr[L.nptr_off + n]; j < T.npn_ptr[L.nptr_off + n + 1]; ++j) {
              uint32_t e32 = T.npn_ent[j];
              if (ints) {
                int ib = (e32 >> 1) & 0x1fff;
                long long* e = ints + 7 * c;
                e[0] = b + 1; e[1] = L.s + 1;
                e[2] = (long long)T.Bops_dm[L.dm][2 * ib]; e[3] = (long long)T.Bops_dm[L.dm][2 * ib + 1];
                e[4] = n + 1; e[5] = (long long)(e32 >> 14) + 1;
                e[6] = (e32 & 1) ? 0 : 1;
              }
              ++c;
            }
        }
      }
  } else if (which == 2 || which == 3) {
    const auto& ptr = which == 2 ? T.pp_ptr : T.nn_ptr;
    const auto& col = which == 2 ? T.pp_col : T.nn_col;
    const auto& val = which == 2 ? T.pp_val : T.nn_val;
    const auto& start = which == 2 ? T.pstart : T.nstart;
    for (int b = 0; b < T.nb; ++b)
      for (int g = start[b]; g < start[b + 1]; ++g) {
        int i = g - start[b];
        for (int k = ptr[g]; k < ptr[g + 1]; ++k) {
          if (col[k] < i) continue;
          if (ints) {
            long long* e = ints + 3 * c;
            e[0] = b + 1; e[1] = i + 1; e[2] = col[k] + 1;
            coef[c] = (col[k] == i) ? 0.5 * val[k] : val[k];
          }
          ++c;
        }
      }
  } else {
    return SMGPU_ERR_ARG;
  }
  *count = c;
  return SMGPU_OK;
}

int smgpu_matvec(smgpu_problem* h, const double* v, double* w, int ncols, int accumulate) {
  if (!h || !v || !w || ncols < 1) return fail(h, SMGPU_ERR_ARG, "bad matvec arguments");
  return guarded(h, [&]() {
    const int64_t mdim = h->T.mdim, len = h->T.len_pad;
    DeviceArena tmp;
    try {
      double* d_in = tmp.alloc<double>(mdim);
      double* d_out = tmp.alloc<double>(mdim);
      double* d_w = tmp.alloc<double>(len);
      SMGPU_CUDA_TRY(cudaMemsetAsync(d_w, 0, sizeof(double) * len, h->st));
      std::vector<double> host(mdim);
      void* d_v = (h->precision == SMGPU_FP64) ? (void*)tmp.alloc<double>(len) : (void*)tmp.alloc<float>(len);
      double t0 = now_s();
      for (int c = 0; c < ncols; ++c) {
        SMGPU_CUDA_TRY(cudaMemcpyAsync(d_in, v + (size_t)c * mdim, sizeof(double) * mdim, cudaMemcpyHostToDevice, h->st));
        if (h->precision == SMGPU_FP64) {
          launch_to_padded<double>(h->dt, d_in, (double*)d_v, h->st);
          h->hv((const double*)d_v, d_w, HvEpilogue<double>{}, h->st);
        } else {
          launch_to_padded<float>(h->dt, d_in, (float*)d_v, h->st);
          h->hv((const float*)d_v, d_w, HvEpilogue<float>{}, h->st);
        }
        launch_from_padded(h->dt, d_w, d_out, h->st);
        SMGPU_CUDA_TRY(cudaMemcpyAsync(host.data(), d_out, sizeof(double) * mdim, cudaMemcpyDeviceToHost, h->st));
        SMGPU_CUDA_TRY(cudaStreamSynchronize(h->st));
        double* wc = w + (size_t)c * mdim;
        if (accumulate)
          for (int64_t i = 0; i < mdim; ++i) wc[i] += host[i];
        else
          std::memcpy(wc, host.data(), sizeof(double) * mdim);
      }
      SMGPU_CUDA_TRY(cudaGetLastError());
      h->times[2] = now_s() - t0;
    } catch (...) {
      tmp.free_all();
      throw;
    }
    tmp.free_all();
    return SMGPU_OK;
  });
}

int smgpu_solve(smgpu_problem* h, int num_ev, int lm, int ls, double tol, int max_restarts, const double* v1,
                double* evals_out, double* evecs_out, int* stats_out) {
  if (!h || !evals_out) return fail(h, SMGPU_ERR_ARG, "null argument");
  if (num_ev < 1 || lm < 3 || ls < 1 || ls > lm - 2 || ls > 60 || lm > 1000 || num_ev > lm - 1 || !(tol > 0.0))
    return fail(h, SMGPU_ERR_ARG, "need 1 <= num_ev < lm, 1 <= ls <= min(lm-2, 60), lm <= 1000, tol > 0");
  return guarded(h, [&]() {
    if (h->precision == SMGPU_FP64) {
      Solve<double> s{h};
      return s.run(num_ev, lm, ls, tol, max_restarts, v1, evals_out, evecs_out, stats_out);
    }
    Solve<float> s{h};
    s.df = h->precision == SMGPU_MIXED_DF;
    return s.run(num_ev, lm, ls, tol, max_restarts, v1, evals_out, evecs_out, stats_out);
  });
}

int smgpu_solve_J(smgpu_problem* h, int twoJ, int num_ev, int lm, int ls, double tol, int max_restarts,
                  const double* v1, double* evals_out, double* evecs_out, int* stats_out) {
  if (!h || !evals_out) return fail(h, SMGPU_ERR_ARG, "null argument");
  if (num_ev < 1 || lm < 3 || ls < 2 || ls > lm - 2 || ls > 60 || lm > 1000 || num_ev > lm - 1 || !(tol > 0.0))
    return fail(h, SMGPU_ERR_ARG, "need 1 <= num_ev < lm, 2 <= ls <= min(lm-2, 60), lm <= 1000, tol > 0");
  if (twoJ != h->mtot2)
    return fail(h, SMGPU_ERR_ARG, "the handle's basis has 2M = " + std::to_string(h->mtot2) +
                                      "; create it with smgpu_problem_create_from_snt_J for 2J = " +
                                      std::to_string(twoJ));
  return guarded(h, [&]() {
    const double eval_jj = 0.5 * twoJ * (0.5 * twoJ + 1.0);  // shellmodel_main.jl:114
    // FP64 in both forms: FP32 Krylov vectors carry rounding components of
    // every J at 1e-7, from which the Lanczos process recovers lower-lying
    // states of other J faster than the projection removes them.
    h->ensure_fp64();
    Solve<double> s{h};
    s.Jop = ensure_jj_op(h);
    s.eval_jj = eval_jj;
    return s.run_projected(num_ev, lm, ls, tol, max_restarts, v1, evals_out, evecs_out, stats_out);
  });
}

int smgpu_solve_block(smgpu_problem* h, int q, int num_ev, int lm, int ls, double tol, int max_restarts,
                      const double* v1, double* evals_out, double* evecs_out, int* stats_out) {
  if (!h || !evals_out) return fail(h, SMGPU_ERR_ARG, "null argument");
  if (q < 1 || q > 8 || num_ev < 1 || lm < 2 * q || ls < q || ls / q + 1 > lm / q - 1 || lm > 1000 ||
      !(tol > 0.0))
    return fail(h, SMGPU_ERR_ARG, "need 1 <= q <= 8, ls >= q, ls/q + 2 <= lm/q, lm <= 1000, tol > 0");
  return guarded(h, [&]() {
    h->ensure_fp64();
    BlockSolve s{h};
    return s.run(q, num_ev, lm, ls, tol, max_restarts, v1, evals_out, evecs_out, stats_out);
  });
}

int smgpu_time_matvec(smgpu_problem* h, int reps, int flush_l2, double* ms_out) {
  if (!h || !ms_out || reps < 1) return fail(h, SMGPU_ERR_ARG, "bad time_matvec arguments");
  return guarded(h, [&]() {
    DeviceArena tmp;
    cudaEvent_t a = nullptr, b = nullptr;
    try {
      const int64_t len = h->T.len_pad;
      double* d_start = tmp.alloc<double>(len);
      double* d_w = tmp.alloc<double>(len);
      void* d_v = (h->precision == SMGPU_FP64) ? (void*)tmp.alloc<double>(len) : (void*)tmp.alloc<float>(len);
      char* flush = flush_l2 ? tmp.alloc<char>(256u << 20) : nullptr;
      launch_start_vector(h->dt, 1234ull, d_start, h->st);
      if (h->precision == SMGPU_FP64)
        SMGPU_CUDA_TRY(cudaMemcpyAsync(d_v, d_start, sizeof(double) * len, cudaMemcpyDeviceToDevice, h->st));
      else
        launch_convert(d_start, (float*)d_v, len, h->st);
      SMGPU_CUDA_TRY(cudaEventCreate(&a));
      SMGPU_CUDA_TRY(cudaEventCreate(&b));
      double total = 0.0;
      for (int r = 0; r < reps; ++r) {
        if (flush) SMGPU_CUDA_TRY(cudaMemsetAsync(flush, r & 0xff, 256u << 20, h->st));
        SMGPU_CUDA_TRY(cudaEventRecord(a, h->st));
        if (h->precision == SMGPU_FP64) h->hv((const double*)d_v, d_w, HvEpilogue<double>{}, h->st);
        else h->hv((const float*)d_v, d_w, HvEpilogue<float>{}, h->st);
        SMGPU_CUDA_TRY(cudaEventRecord(b, h->st));
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

int smgpu_jj(smgpu_problem* h, const double* vecs, int nvec, double* jj_out) {
  if (!h || !vecs || !jj_out || nvec < 1) return fail(h, SMGPU_ERR_ARG, "bad jj arguments");
  return guarded(h, [&]() {
    smgpu_problem* q = ensure_jj_op(h);
    const int64_t mdim = h->T.mdim, len = q->T.len_pad;
    DeviceArena tmp;
    try {
      double* d_in = tmp.alloc<double>(mdim);
      double* d_out = tmp.alloc<double>(mdim);
      double* d_v = tmp.alloc<double>(len);
      double* d_w = tmp.alloc<double>(len);
      std::vector<double> w(mdim);
      for (int k = 0; k < nvec; ++k) {
        const double* v = vecs + (size_t)k * mdim;
        SMGPU_CUDA_TRY(cudaMemcpyAsync(d_in, v, sizeof(double) * mdim, cudaMemcpyHostToDevice, h->st));
        SMGPU_CUDA_TRY(cudaMemsetAsync(d_w, 0, sizeof(double) * len, h->st));
        launch_to_padded<double>(q->dt, d_in, d_v, h->st);
        q->hv((const double*)d_v, d_w, HvEpilogue<double>{}, h->st);
        launch_from_padded(q->dt, d_w, d_out, h->st);
        SMGPU_CUDA_TRY(cudaMemcpyAsync(w.data(), d_out, sizeof(double) * mdim, cudaMemcpyDeviceToHost, h->st));
        SMGPU_CUDA_TRY(cudaStreamSynchronize(h->st));
        double vw = 0.0, vv = 0.0;
        for (int64_t i = 0; i < mdim; ++i) {
          vw += v[i] * w[i];
          vv += v[i] * v[i];
        }
        jj_out[k] = vv > 0.0 ? vw / vv : 0.0;
      }
      SMGPU_CUDA_TRY(cudaGetLastError());
    } catch (...) {
      tmp.free_all();
      throw;
    }
    tmp.free_all();
    return SMGPU_OK;
  });
}

int smgpu_tune_report(const smgpu_problem* h, int max, int* shapes, double* ms, int* count) {
  if (!h || !count || max < 0 || (max > 0 && (!shapes || !ms))) return SMGPU_ERR_ARG;
  const int n = (int)h->tune_shapes.size();
  *count = n;
  for (int k = 0; k < n && k < max; ++k) {
    const HvConfig& c = h->tune_shapes[k];
    shapes[4 * k + 0] = c.nt;
    shapes[4 * k + 1] = c.rows;
    shapes[4 * k + 2] = c.minb;
    shapes[4 * k + 3] = c.staged;
    ms[k] = h->tune_ms[k];
  }
  return SMGPU_OK;
}

int smgpu_timings(const smgpu_problem* h, double* t) {
  if (!h || !t) return SMGPU_ERR_ARG;
  for (int k = 0; k < 8; ++k) t[k] = h->times[k];
  return SMGPU_OK;
}

int smgpu_stats(const smgpu_problem* h, long long* s) {
  if (!h || !s) return SMGPU_ERR_ARG;
  const Tables& T = h->T;
  s[0] = T.updates;
  s[1] = (long long)T.ppn_src.size();
  s[2] = (long long)T.npn_ent.size();
  s[3] = (long long)T.pp_col.size();
  s[4] = (long long)T.nn_col.size();
  s[5] = (long long)h->tables.bytes;
  s[6] = (long long)T.len_pad;
  s[7] = (long long)T.links.size();
  s[8] = h->cfg.nt;
  s[9] = h->cfg.rows;
  s[10] = h->cfg.minb;
  s[11] = h->cfg.staged;
  return SMGPU_OK;
}

}  // extern "C"

// ===========================================================================
// Allocation-free H·v (smgpu_matvec_noalloc).
//
// For callers that cannot let a library allocate device memory while they
// run: hosts whose device memory belongs to their own pool allocator (a Julia
// CuArray pool, PyTorch's caching allocator).  Such a pool usually holds most
// of the device's memory, so a library's cudaMalloc in the middle of a step
// can fail or force the pool to release its cache, and a cudaFree
// synchronizes the whole device, stalling the host's queued work.  The only
// scratch this H·v needs — the per-CTA partial sums of <v|H|v> — lives in the
// file-scope array below, so the call allocates nothing.  Every GPU that
// loads the library holds this array (512 KB) until the process exits.
//
// Ordering: the kernels run on the handle's own stream, which does not
// synchronize with the caller's streams or the legacy default stream, so the
// caller must have finished all device work that writes v (or still reads
// w) before the call; the call returns after w and *vhv are written.
namespace {
constexpr int kNoAllocMaxPartials = 1 << 16;  // CTAs of one H·v launch; 65,536 doubles = 512 KB
static __device__ __align__(256) double g_noalloc_partials[kNoAllocMaxPartials];

constexpr int kMaxDevices = 64;
std::mutex g_noalloc_mu;
double* g_noalloc_addr[kMaxDevices] = {nullptr};

// Device address of g_noalloc_partials on the current device.  Host code only
// holds a host-side stand-in for the symbol, so the address is looked up once
// per device (with that device current, on the first call there) and cached
// for the life of the process: a cudaDeviceReset between calls would leave
// the cached address stale and is not supported.
double* noalloc_scratch() {
  int dev = -1;
  SMGPU_CUDA_TRY(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices) throw SetupError{SMGPU_ERR_ARG, "device ordinal out of range"};
  std::lock_guard<std::mutex> lk(g_noalloc_mu);
  if (g_noalloc_addr[dev] == nullptr) {
    void* p = nullptr;
    SMGPU_CUDA_TRY(cudaGetSymbolAddress(&p, g_noalloc_partials));
    g_noalloc_addr[dev] = static_cast<double*>(p);
  }
  return g_noalloc_addr[dev];
}

__global__ void k_noalloc_vhv(const double* __restrict__ partials, int n, double* __restrict__ out) {
  __shared__ double red[32];
  double x = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) x += partials[i];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = x;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int k = 0; k < (int)(blockDim.x >> 5); ++k) s += red[k];
    *out = s;
  }
}
}  // namespace

extern "C" int smgpu_matvec_noalloc(smgpu_problem* h, const double* v, double* w, double* vhv) {
  if (!h || !v || !w) return fail(h, SMGPU_ERR_ARG, "null argument");
  if (h->precision != SMGPU_FP64)
    return fail(h, SMGPU_ERR_ARG, "smgpu_matvec_noalloc needs a handle created with SMGPU_FP64");
  if (h->cfg.ntasks > kNoAllocMaxPartials)
    return fail(h, SMGPU_ERR_LIMIT,
                "problem too large for smgpu_matvec_noalloc: the H·v launch needs " + std::to_string(h->cfg.ntasks) +
                    " partial sums, the static scratch holds " + std::to_string(kNoAllocMaxPartials));
  return guarded(h, [&]() {
    double* scratch = noalloc_scratch();
    // the handle's tables viewed in the reference's unpadded layout: block b
    // at tdims[b], rows of stride nn[b]
    DevTables t = h->dt;
    t.stride = h->dt.nn;
    t.off_pad = h->dt.tdims;
    t.len_pad = h->T.mdim;
    HvEpilogue<double> epi{};
    epi.alpha_part = scratch;
    launch_hv_fp64(t, h->tt, h->cfg, h->d_ep, h->d_en, h->c64, v, w, epi, h->st);
    if (vhv) k_noalloc_vhv<<<1, 256, 0, h->st>>>(scratch, h->cfg.ntasks, vhv);
    SMGPU_CUDA_TRY(cudaGetLastError());
    SMGPU_CUDA_TRY(cudaStreamSynchronize(h->st));
    return SMGPU_OK;
  });
}
