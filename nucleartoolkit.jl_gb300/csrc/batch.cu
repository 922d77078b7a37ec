// extern "C" entry points for batches of independent shell-model problems
// (smgpu_batch_*, declared in include/smgpu.h).
//
// The reference solves one problem per main_sm call
// (src/ShellModel/shellmodel_main.jl:89-281); a user with many nuclei or
// interactions calls it in a loop.  Here a batch of problems of uneven
// dimension is set up once (each its own basis, jump tables and
// interaction) and iterated in lockstep in the FP32-mixed form: per Lanczos
// iteration one batched H·v launch over every problem's row tiles, the
// batched re-orthogonalisation kernels and one CTA per problem for the
// eigenvalue test, all captured per restart cycle in a CUDA graph.  The H·v
// launch shape is autotuned on the whole batch.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <limits>
#include <map>
#include <string>
#include <vector>

#include "../../include/smgpu.h"
#include "batch.cuh"
#include "device.cuh"
#include "lanczos.cuh"
#include "problem.h"
#include "setup.h"

namespace {
constexpr int kChunk = 2048;  // elements per streaming chunk (multiple of 4)
constexpr int kMaxBatch = 4096;
}  // namespace

struct smgpu_batch {
  int nprob = 0;
  std::vector<smgpu_problem*> P;
  std::vector<int64_t> voff, moff;
  int64_t LEN = 0, MTOT = 0;
  cudaStream_t st = nullptr, st2 = nullptr;
  int sms = 152;
  DeviceArena arena;
  std::vector<BatchProblemDev> hprobs;
  BatchProblemDev* d_probs = nullptr;
  std::vector<int4> hchunks;
  int4* d_chunks = nullptr;
  std::map<int, std::pair<int4*, int>> tasks;                 // rows per task -> (device list, count)
  std::map<int, std::vector<std::pair<int, int>>> slots;      // rows per task -> per problem (slot0, nslots)
  int cand = 4;
  size_t smem = 0;  // dynamic shared memory of the selected shape
  double tune_ms[16] = {0};
  std::string err;
  double times[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  DeviceArena solver;

  ~smgpu_batch() {
    solver.free_all();
    arena.free_all();
    for (smgpu_problem* p : P) delete p;
    if (st) cudaStreamDestroy(st);
    if (st2) cudaStreamDestroy(st2);
  }

  int rows() const {
    int nc = 0;
    return hv_batch_candidates(&nc)[cand].rows;
  }

  // Row tasks of R rows for every problem, sorted by estimated work (largest
  // first); α slots are contiguous per problem.
  void ensure_tasks(int R) {
    if (tasks.count(R)) return;
    struct Item {
      double cost;
      int4 t;
    };
    std::vector<Item> items;
    std::vector<std::pair<int, int>> sl(nprob);
    int slot = 0;
    for (int p = 0; p < nprob; ++p) {
      const Tables& T = P[p]->T;
      sl[p].first = slot;
      for (int b = 0; b < T.nb; ++b) {
        const double per_row =
            (double)T.nn[b] * (1.0 + (double)(T.ppn_ptr[T.pstart[b + 1]] - T.ppn_ptr[T.pstart[b]]) / T.np[b]);
        for (int p0 = 0; p0 < T.np[b]; p0 += R) {
          const int nr = std::min(R, T.np[b] - p0);
          items.push_back({per_row * nr, make_int4(p, b, p0, slot++)});
        }
      }
      sl[p].second = slot - sl[p].first;
    }
    std::stable_sort(items.begin(), items.end(), [](const Item& a, const Item& b) { return a.cost > b.cost; });
    std::vector<int4> t(items.size());
    for (size_t k = 0; k < items.size(); ++k) t[k] = items[k].t;
    tasks[R] = {arena.upload(t), (int)t.size()};
    slots[R] = sl;
  }

  // Dynamic shared memory of a staged launch shape (the largest over the
  // problems) and whether every problem fits it; 0 / true for the others.
  size_t staged_smem(int c) const {
    int nc = 0;
    const BatchHvConfig& k = hv_batch_candidates(&nc)[c];
    if (!k.staged) return 0;
    const HvConfig hc{k.nt, k.rows, 0, k.minb, 1};
    size_t m = 0;
    for (const smgpu_problem* p : P) m = std::max(m, hv_staged_smem(hc, p->tt));
    return m;
  }
  bool fits(int c) const {
    int nc = 0;
    const BatchHvConfig& k = hv_batch_candidates(&nc)[c];
    if (!k.staged) return true;
    for (const smgpu_problem* p : P)
      if (p->tt.push_ent == nullptr || p->nnmax_raw > hv_batch_staged_cols(k)) return false;
    return staged_smem(c) <= 200 * 1024;
  }

  // Select a launch shape; the per-problem α slot ranges follow its rows.
  void set_cand(int c) {
    if (!fits(c)) throw SetupError{SMGPU_ERR_ARG, "batched H·v launch shape does not fit these problems"};
    cand = c;
    smem = staged_smem(c);
    if (smem > 0) hv_batch_prepare(c, smem);
    const int R = rows();
    ensure_tasks(R);
    for (int p = 0; p < nprob; ++p) {
      hprobs[p].slot0 = slots[R][p].first;
      hprobs[p].nslots = slots[R][p].second;
    }
    SMGPU_CUDA_TRY(cudaMemcpy(d_probs, hprobs.data(), sizeof(BatchProblemDev) * nprob, cudaMemcpyHostToDevice));
  }

  int ntasks() { return tasks[rows()].second; }

  void hv(const float* v, double* w, const BatchEpi& e, cudaStream_t s) {
    const auto& tk = tasks[rows()];
    launch_hv_batch(cand, d_probs, tk.first, tk.second, v, w, e, smem, s);
  }

  BatchDev view() const {
    BatchDev B{};
    B.nprob = nprob;
    B.probs = d_probs;
    B.chunks = d_chunks;
    B.nchunks = (int)hchunks.size();
    B.LEN = LEN;
    return B;
  }

  void autotune();
};

namespace {
thread_local std::string g_batch_create_error;

double now_s() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

int fail(smgpu_batch* h, int code, const std::string& msg) {
  if (h) h->err = msg;
  else g_batch_create_error = msg;
  return code;
}

template <class F>
int guarded(smgpu_batch* h, F&& f) {
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
}  // namespace

// Time every launch shape on the whole batch (3 launches each, the first a
// warm-up) and keep the fastest.  SMGPU_AUTOTUNE=0 keeps the default.
void smgpu_batch::autotune() {
  // SMGPU_BATCH_CAND=k selects candidate k of hv_batch_candidates outright
  // (for tests that run every shape)
  if (const char* c = std::getenv("SMGPU_BATCH_CAND")) {
    int nc = 0;
    hv_batch_candidates(&nc);
    const int k = std::atoi(c);
    if (k < 0 || k >= nc) throw SetupError{SMGPU_ERR_ARG, "SMGPU_BATCH_CAND out of range"};
    set_cand(k);
    return;
  }
  const char* off = std::getenv("SMGPU_AUTOTUNE");
  if (off && std::string(off) == "0") return;
  DeviceArena tmp;
  cudaEvent_t a = nullptr, b = nullptr;
  try {
    const BatchDev B = view();
    double* d_w0 = tmp.alloc<double>(LEN);
    float* d_v = tmp.alloc<float>(LEN);
    double* d_w = tmp.alloc<double>(LEN);
    launch_b_start(B, 1234ull, d_w0, st);
    launch_b_convert(B, d_w0, d_v, st);
    SMGPU_CUDA_TRY(cudaEventCreate(&a));
    SMGPU_CUDA_TRY(cudaEventCreate(&b));
    int nc = 0;
    const BatchHvConfig* cands = hv_batch_candidates(&nc);
    // staged shapes first (usually the fastest); a shape whose warm-up launch
    // takes more than twice the best mean so far is dropped untimed
    std::vector<int> order;
    for (int c = 0; c < nc; ++c)
      if (cands[c].staged) order.push_back(c);
    for (int c = 0; c < nc; ++c)
      if (!cands[c].staged) order.push_back(c);
    int best = -1;
    float best_ms = 1e30f;
    for (int c : order) {
      if (!fits(c)) continue;
      set_cand(c);
      float total = 0.f;
      bool dropped = false;
      for (int rep = 0; rep < 3; ++rep) {
        SMGPU_CUDA_TRY(cudaEventRecord(a, st));
        hv(d_v, d_w, BatchEpi{}, st);
        SMGPU_CUDA_TRY(cudaEventRecord(b, st));
        SMGPU_CUDA_TRY(cudaEventSynchronize(b));
        float ms = 0.f;
        SMGPU_CUDA_TRY(cudaEventElapsedTime(&ms, a, b));
        if (rep > 0) total += ms;
        if (rep == 0 && best >= 0 && ms > 2.f * (best_ms / 2)) {
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
    if (best < 0) best = cand;
    set_cand(best);
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
struct BatchSolve {
  smgpu_batch* H;
  BatchDev B{};
  float* V = nullptr;
  float* U = nullptr;
  double* w = nullptr;
  int* hv_count = nullptr;
  int* task_ctr = nullptr;  // persistent form: per-iteration H·v task queues
  GridSync* gs = nullptr;   // persistent form: grid barrier
  long long launches_first = 0, launches_rest = 0;

  void alloc(int lm, int ls, int num_ev, double tol) {
    DeviceArena& A = H->solver;
    A.free_all();
    B = H->view();
    B.lm = lm;
    B.ls = ls;
    B.num_ev = num_ev;
    B.nh = 3;
    B.tol = tol;
    B.fastnorm = fastnorm_threshold();
    B.nslots = H->ntasks();
    const int np = H->nprob, nch = B.nchunks;
    const int NP = ls * (ls + 1) / 2 + ls;
    V = A.alloc<float>((size_t)lm * B.LEN);
    U = A.alloc<float>((size_t)ls * B.LEN);
    w = A.alloc<double>(B.LEN);
    B.T = A.alloc<double>((size_t)np * lm * lm);
    B.en = A.alloc<double>((size_t)np * B.nh * num_ev);
    B.alpha_part = A.alloc<double>((size_t)lm * B.nslots);
    B.pdot = A.alloc<double>((size_t)(lm + 2) * nch);
    B.pn1 = A.alloc<double>(nch);
    B.pdot2 = A.alloc<double>((size_t)(lm + 2) * nch);
    B.pn2 = A.alloc<double>(nch);
    B.part = A.alloc<double>((size_t)NP * nch);
    B.jacA = A.alloc<double>((size_t)np * lm * lm);
    B.jacZ = A.alloc<double>((size_t)np * lm * lm);
    B.evals = A.alloc<double>((size_t)np * lm);
    B.Yf = A.alloc<float>((size_t)np * (lm - 1) * ls);
    B.wsplit = A.alloc<float>(2 * (size_t)B.LEN);
    B.X = A.alloc<double>((size_t)np * ls * ls);
    B.Xf = A.alloc<float>((size_t)np * (ls * ls + ls));
    B.cvec = A.alloc<double>((size_t)np * ls);
    B.fl = A.alloc<LanczosFlags>(np);
    B.ctl = A.alloc<BatchCtl>(1);
    hv_count = A.alloc<int>(1);
    task_ctr = A.alloc<int>(lm);
    gs = A.alloc<GridSync>(1);
    cudaStream_t st = H->st;
    SMGPU_CUDA_TRY(cudaMemsetAsync(hv_count, 0, sizeof(int), st));
    SMGPU_CUDA_TRY(cudaMemsetAsync(V, 0, sizeof(float) * (size_t)lm * B.LEN, st));
    SMGPU_CUDA_TRY(cudaMemsetAsync(U, 0, sizeof(float) * (size_t)ls * B.LEN, st));
    SMGPU_CUDA_TRY(cudaMemsetAsync(w, 0, sizeof(double) * B.LEN, st));
    SMGPU_CUDA_TRY(cudaMemsetAsync(B.wsplit, 0, sizeof(float) * 2 * B.LEN, st));
    SMGPU_CUDA_TRY(cudaMemsetAsync(B.T, 0, sizeof(double) * (size_t)np * lm * lm, st));
    SMGPU_CUDA_TRY(cudaMemsetAsync(B.fl, 0, sizeof(LanczosFlags) * np, st));
    SMGPU_CUDA_TRY(cudaMemsetAsync(B.ctl, 0, sizeof(BatchCtl), st));
    std::vector<double> en0((size_t)np * B.nh * num_ev, 1.0e4);
    SMGPU_CUDA_TRY(cudaMemcpyAsync(B.en, en0.data(), sizeof(double) * en0.size(), cudaMemcpyHostToDevice, st));
    SMGPU_CUDA_TRY(cudaStreamSynchronize(st));
  }

  void iteration(int it, int lock, cudaEvent_t ev_fork) {
    cudaStream_t s = H->st, s2 = H->st2;
    const int it0 = it - 1;
    BatchEpi e{};
    e.ctl = B.ctl;
    e.fl = B.fl;
    e.T = B.T;
    e.lm = B.lm;
    e.it0 = it0;
    e.alpha_part = B.alpha_part + (size_t)it0 * B.nslots;
    e.count = hv_count;
    if (it0 > lock) e.vprev = V + (size_t)(it0 - 1) * B.LEN;
    H->hv(V + (size_t)it0 * B.LEN, w, e, s);
    SMGPU_CUDA_TRY(cudaEventRecord(ev_fork, s));
    SMGPU_CUDA_TRY(cudaStreamWaitEvent(s2, ev_fork, 0));
    launch_b_sturm(B, it, lock, s2);
    launch_b_orth(B, V, w, it0, s);
  }

  cudaGraphExec_t capture_cycle(int kstart, int lock, long long* nkernels) {
    cudaStream_t s = H->st, s2 = H->st2;
    cudaEvent_t e_fork, e_join;
    SMGPU_CUDA_TRY(cudaEventCreateWithFlags(&e_fork, cudaEventDisableTiming));
    SMGPU_CUDA_TRY(cudaEventCreateWithFlags(&e_join, cudaEventDisableTiming));
    cudaGraph_t g;
    SMGPU_CUDA_TRY(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    for (int it = kstart; it <= B.lm - 1; ++it) iteration(it, lock, e_fork);
    SMGPU_CUDA_TRY(cudaEventRecord(e_join, s2));
    SMGPU_CUDA_TRY(cudaStreamWaitEvent(s, e_join, 0));
    launch_b_cycle_end(B, s);
    launch_b_restart(B, V, U, s);
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
    cudaStream_t st = H->st;
    const int np = H->nprob;
    const double tw0 = now_s();
    alloc(lm, ls, num_ev, tol);
    double* v1dev = nullptr;
    if (v1) {
      v1dev = H->solver.alloc<double>(H->MTOT);
      SMGPU_CUDA_TRY(cudaMemcpyAsync(v1dev, v1, sizeof(double) * H->MTOT, cudaMemcpyHostToDevice, st));
    }
    // the persistent form (one cooperative launch per restart cycle) when the
    // H·v shape has one and the GPU runs it; SMGPU_BATCH_PERSIST=0 selects
    // the graph form (one graph of per-phase launches per cycle)
    const char* pe = std::getenv("SMGPU_BATCH_PERSIST");
    const int pgrid = (pe && std::string(pe) == "0") ? 0 : persist_grid(H->cand, B, H->smem);
    const bool persist = pgrid > 0;
    long long spin_limit = 1ll << 24;  // barrier polls (each at least 32 ns) before a wait gives up
    if (const char* sl = std::getenv("SMGPU_BATCH_SPIN_LIMIT")) spin_limit = std::max(1ll, std::atoll(sl));
    const double tc0 = now_s();
    cudaGraphExec_t g_first = nullptr, g_rest = nullptr;
    if (!persist) {
      g_first = capture_cycle(1, 0, &launches_first);
      g_rest = capture_cycle(ls + 1, ls, &launches_rest);
    }
    H->times[3] = now_s() - tc0;
    cudaEvent_t e0, e1, e2;
    SMGPU_CUDA_TRY(cudaEventCreate(&e0));
    SMGPU_CUDA_TRY(cudaEventCreate(&e1));
    SMGPU_CUDA_TRY(cudaEventCreate(&e2));
    SMGPU_CUDA_TRY(cudaEventRecord(e0, st));
    if (v1dev) launch_b_to_padded(B, v1dev, w, st);
    else launch_b_start(B, 1234ull, w, st);
    launch_b_init(B, w, V, st);
    long long launches = 3;
    int n_restart = 0, status = SMGPU_OK;
    BatchCtl ctl{};
    if (persist) {
      BatchCycle C{};
      const auto& tk = H->tasks[H->rows()];
      C.tasks = tk.first;
      C.ntasks = tk.second;
      C.task_ctr = task_ctr;
      C.hv_count = hv_count;
      C.gs = gs;
      C.spin_limit = spin_limit;
      C.kstart = 1;
      C.lock = 0;
      while (true) {
        SMGPU_CUDA_TRY(cudaMemsetAsync(task_ctr, 0, sizeof(int) * lm, st));
        SMGPU_CUDA_TRY(cudaMemsetAsync(gs, 0, sizeof(GridSync), st));
        launch_b_persist_cycle(H->cand, B, V, w, C, H->smem, pgrid, st);
        launch_b_cycle_end(B, st);
        launches += 2;
        SMGPU_CUDA_TRY(cudaMemcpyAsync(&ctl, B.ctl, sizeof(BatchCtl), cudaMemcpyDeviceToHost, st));
        SMGPU_CUDA_TRY(cudaStreamSynchronize(st));
        if (ctl.sync_err) break;
        if (ctl.all_done) break;
        ++n_restart;
        if (n_restart > max_restarts) {
          status = SMGPU_ERR_NOCONV;
          break;
        }
        launch_b_restart(B, V, U, st);
        launches += 6;
        C.kstart = ls + 1;
        C.lock = ls;
      }
    } else {
      SMGPU_CUDA_TRY(cudaGraphLaunch(g_first, st));
      launches += launches_first;
      while (true) {
        SMGPU_CUDA_TRY(cudaMemcpyAsync(&ctl, B.ctl, sizeof(BatchCtl), cudaMemcpyDeviceToHost, st));
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
    }
    std::vector<double> en((size_t)np * B.nh * num_ev);
    std::vector<LanczosFlags> fl(np);
    int n_hv = 0;
    SMGPU_CUDA_TRY(cudaMemcpyAsync(&n_hv, hv_count, sizeof(int), cudaMemcpyDeviceToHost, st));
    SMGPU_CUDA_TRY(cudaMemcpyAsync(en.data(), B.en, sizeof(double) * en.size(), cudaMemcpyDeviceToHost, st));
    SMGPU_CUDA_TRY(cudaMemcpyAsync(fl.data(), B.fl, sizeof(LanczosFlags) * np, cudaMemcpyDeviceToHost, st));
    SMGPU_CUDA_TRY(cudaEventRecord(e1, st));
    SMGPU_CUDA_TRY(cudaStreamSynchronize(st));
    if (g_first) cudaGraphExecDestroy(g_first);
    if (g_rest) cudaGraphExecDestroy(g_rest);
    if (ctl.sync_err)
      return fail(H, SMGPU_ERR_DEVICE,
                  "a grid barrier of the persistent batch kernel ran out of its wait limit (SMGPU_BATCH_SPIN_LIMIT)");
    for (int p = 0; p < np; ++p) {
      const int nev = (int)std::min<int64_t>(num_ev, H->P[p]->T.mdim);
      for (int j = 0; j < num_ev; ++j)
        evals_out[(size_t)p * num_ev + j] =
            j < nev ? en[(size_t)p * B.nh * num_ev + j] : std::numeric_limits<double>::quiet_NaN();
    }
    for (int p = 0; p < np; ++p)
      if (fl[p].bad) return fail(H, SMGPU_ERR_DEVICE, "restart Gram matrix was not positive definite");
    if (evecs_out) {
      std::memset(evecs_out, 0, sizeof(double) * (size_t)num_ev * H->MTOT);
      int64_t maxlen = 0, maxmdim = 0;
      for (int p = 0; p < np; ++p) {
        maxlen = std::max(maxlen, H->P[p]->T.len_pad);
        maxmdim = std::max(maxmdim, H->P[p]->T.mdim);
      }
      double* R = H->solver.alloc<double>((size_t)num_ev * maxlen);
      double* tmp = H->solver.alloc<double>(maxmdim);
      double* hs = H->solver.alloc<double>(num_ev + 2);
      LanczosDev L{};
      L.G = 2 * H->sms;
      L.partials = H->solver.alloc<double>((size_t)L.G);
      L.h = hs;
      for (int p = 0; p < np; ++p) {
        if (!fl[p].done || fl[p].elit <= 0) continue;
        const Tables& T = H->P[p]->T;
        const int elit = fl[p].elit;
        const int nev = (int)std::min<int64_t>(num_ev, T.mdim);
        L.len = T.len_pad;
        launch_b_jacobi_one(B, p, elit, st);
        launch_b_ritz(B, V, p, elit, nev, T.len_pad, R, st);
        launches += 2;
        for (int e = 0; e < nev; ++e) {
          double* r = R + (size_t)e * T.len_pad;
          launch_multidot<double>(L, r, 1, r, false, st);
          launch_reduce(L, 1, RED_INVNORM, L.h + e, st);
          launch_scale_store<double>(L, r, r, L.h + e, st);
          launch_from_padded(H->P[p]->dt, r, tmp, st);
          launches += 4;
          SMGPU_CUDA_TRY(cudaMemcpyAsync(evecs_out + (size_t)num_ev * H->moff[p] + (size_t)e * T.mdim, tmp,
                                         sizeof(double) * T.mdim, cudaMemcpyDeviceToHost, st));
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
    for (int p = 0; p < np; ++p) all = all && fl[p].done;
    if (stats_out) {
      stats_out[0] = n_hv;
      stats_out[1] = n_restart;
      stats_out[2] = all ? 1 : 0;
      stats_out[3] = num_ev;
      stats_out[4] = (int)launches;
      stats_out[5] = np;
      stats_out[6] = B.nchunks;
      stats_out[7] = B.nslots;
      for (int p = 0; p < np; ++p) {
        stats_out[8 + 4 * p] = fl[p].done ? fl[p].elit : 0;
        stats_out[8 + 4 * p + 1] = fl[p].done ? 1 : 0;
        stats_out[8 + 4 * p + 2] = fl[p].n_second;
        stats_out[8 + 4 * p + 3] = 0;
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

int smgpu_batch_create_from_snt(const char* const* snt_paths, const char* const* nuclei, int nprob,
                                smgpu_batch** out) {
  if (!snt_paths || !nuclei || !out || nprob < 1) return fail(nullptr, SMGPU_ERR_ARG, "bad arguments");
  *out = nullptr;
  if (nprob > kMaxBatch) return fail(nullptr, SMGPU_ERR_LIMIT, "at most 4096 problems per batch");
  for (int p = 0; p < nprob; ++p)
    if (!snt_paths[p] || !nuclei[p]) return fail(nullptr, SMGPU_ERR_ARG, "null snt path or nucleus");
  return guarded(nullptr, [&]() {
    int ndev = 0;
    cudaError_t ce = cudaGetDeviceCount(&ndev);
    if (ce != cudaSuccess || ndev == 0)
      throw SetupError{SMGPU_ERR_CUDA, "no CUDA device available: the GPU library has no CPU path"};
    const double t0 = now_s();
    smgpu_batch* h = new smgpu_batch();
    try {
      h->nprob = nprob;
      int prio_lo = 0, prio_hi = 0;
      SMGPU_CUDA_TRY(cudaDeviceGetStreamPriorityRange(&prio_lo, &prio_hi));
      SMGPU_CUDA_TRY(cudaStreamCreateWithFlags(&h->st, cudaStreamNonBlocking));
      SMGPU_CUDA_TRY(cudaStreamCreateWithPriority(&h->st2, cudaStreamNonBlocking, prio_hi));
      int dev = 0;
      SMGPU_CUDA_TRY(cudaGetDevice(&dev));
      SMGPU_CUDA_TRY(cudaDeviceGetAttribute(&h->sms, cudaDevAttrMultiProcessorCount, dev));
      for (int p = 0; p < nprob; ++p) {
        int A = 0, Z = 0;
        parse_nucleus(nuclei[p], A, Z);
        Interaction I = read_snt(snt_paths[p], A);
        const int vp = Z - I.cp, vn = (A - Z) - I.cn;
        if (vp < 0 || vn < 0)
          throw SetupError{SMGPU_ERR_NUCLEUS, "problem " + std::to_string(p) + ": nucleus lies below the snt core"};
        smgpu_problem* q = new smgpu_problem();
        h->P.push_back(q);
        q->precision = SMGPU_MIXED;
        q->vp = vp;
        q->vn = vn;
        q->mtot2 = (A % 2 == 0) ? 0 : 1;  // shellmodel_main.jl:110
        build_tables(I, vp, vn, q->mtot2, q->T);
        if (q->T.mdim == 0)
          throw SetupError{SMGPU_ERR_EMPTY, "problem " + std::to_string(p) + ": M-scheme dimension is zero"};
        q->upload(false);
      }
      // batch layout: padded vectors and unpadded vectors concatenated, chunks
      h->hprobs.resize(nprob);
      for (int p = 0; p < nprob; ++p) {
        smgpu_problem* q = h->P[p];
        BatchProblemDev& d = h->hprobs[p];
        std::memset(&d, 0, sizeof(d));
        d.a.t = q->dt;
        d.a.tt = q->tt;
        d.a.c = q->c32;
        d.a.ep = q->d_ep;
        d.a.en = q->d_en;
        d.voff = h->LEN;
        d.len = q->T.len_pad;
        d.mdim = q->T.mdim;
        d.moff = h->MTOT;
        h->voff.push_back(h->LEN);
        h->moff.push_back(h->MTOT);
        d.chunk0 = (int)h->hchunks.size();
        for (int64_t b0 = 0; b0 < d.len; b0 += kChunk)
          h->hchunks.push_back(make_int4(p, (int)b0, (int)std::min<int64_t>(b0 + kChunk, d.len), 0));
        d.nchunks = (int)h->hchunks.size() - d.chunk0;
        h->LEN += d.len;
        h->MTOT += d.mdim;
      }
      h->d_chunks = h->arena.upload(h->hchunks);
      h->d_probs = h->arena.alloc<BatchProblemDev>(nprob);
      h->set_cand(h->cand);
      h->autotune();
      SMGPU_CUDA_TRY(cudaStreamSynchronize(h->st));
      h->times[0] = now_s() - t0;
    } catch (...) {
      delete h;
      throw;
    }
    *out = h;
    return SMGPU_OK;
  });
}

int smgpu_batch_destroy(smgpu_batch* h) {
  delete h;
  return SMGPU_OK;
}

const char* smgpu_batch_last_error(const smgpu_batch* h) { return h ? h->err.c_str() : g_batch_create_error.c_str(); }

int smgpu_batch_dims(const smgpu_batch* h, long long* total_mdim, int* nprob, long long* mdims) {
  if (!h) return SMGPU_ERR_ARG;
  if (total_mdim) *total_mdim = h->MTOT;
  if (nprob) *nprob = h->nprob;
  if (mdims)
    for (int p = 0; p < h->nprob; ++p) mdims[p] = h->P[p]->T.mdim;
  return SMGPU_OK;
}

int smgpu_batch_matvec(smgpu_batch* h, const double* v, double* w, int accumulate) {
  if (!h || !v || !w) return fail(h, SMGPU_ERR_ARG, "bad matvec arguments");
  return guarded(h, [&]() {
    DeviceArena tmp;
    try {
      const double t0 = now_s();
      const BatchDev B = h->view();
      double* d_in = tmp.alloc<double>(h->MTOT);
      double* d_out = tmp.alloc<double>(h->MTOT);
      double* d_w0 = tmp.alloc<double>(h->LEN);
      float* d_v = tmp.alloc<float>(h->LEN);
      double* d_w = tmp.alloc<double>(h->LEN);
      SMGPU_CUDA_TRY(cudaMemsetAsync(d_w, 0, sizeof(double) * h->LEN, h->st));
      SMGPU_CUDA_TRY(cudaMemcpyAsync(d_in, v, sizeof(double) * h->MTOT, cudaMemcpyHostToDevice, h->st));
      launch_b_to_padded(B, d_in, d_w0, h->st);
      launch_b_convert(B, d_w0, d_v, h->st);
      h->hv(d_v, d_w, BatchEpi{}, h->st);
      launch_b_from_padded(B, d_w, d_out, h->st);
      std::vector<double> host(h->MTOT);
      SMGPU_CUDA_TRY(cudaMemcpyAsync(host.data(), d_out, sizeof(double) * h->MTOT, cudaMemcpyDeviceToHost, h->st));
      SMGPU_CUDA_TRY(cudaStreamSynchronize(h->st));
      SMGPU_CUDA_TRY(cudaGetLastError());
      if (accumulate)
        for (int64_t i = 0; i < h->MTOT; ++i) w[i] += host[i];
      else
        std::memcpy(w, host.data(), sizeof(double) * h->MTOT);
      h->times[2] = now_s() - t0;
    } catch (...) {
      tmp.free_all();
      throw;
    }
    tmp.free_all();
    return SMGPU_OK;
  });
}

int smgpu_batch_solve(smgpu_batch* h, int num_ev, int lm, int ls, double tol, int max_restarts, const double* v1,
                      double* evals_out, double* evecs_out, int* stats_out) {
  if (!h || !evals_out) return fail(h, SMGPU_ERR_ARG, "null argument");
  if (num_ev < 1 || lm < 3 || ls < 1 || ls > lm - 2 || ls > 60 || lm > 1000 || num_ev > lm - 1 || !(tol > 0.0))
    return fail(h, SMGPU_ERR_ARG, "need 1 <= num_ev < lm, 1 <= ls <= min(lm-2, 60), lm <= 1000, tol > 0");
  return guarded(h, [&]() {
    BatchSolve s{h};
    return s.run(num_ev, lm, ls, tol, max_restarts, v1, evals_out, evecs_out, stats_out);
  });
}

int smgpu_batch_stats(const smgpu_batch* h, long long* s) {
  if (!h || !s) return SMGPU_ERR_ARG;
  int nc = 0;
  const BatchHvConfig* c = hv_batch_candidates(&nc);
  long long upd = 0, bytes = (long long)h->arena.bytes;
  for (const smgpu_problem* p : h->P) {
    upd += p->T.updates;
    bytes += (long long)p->tables.bytes;
  }
  auto it = h->tasks.find(c[h->cand].rows);
  s[0] = upd;
  s[1] = h->nprob;
  s[2] = (long long)h->hchunks.size();
  s[3] = it != h->tasks.end() ? it->second.second : 0;
  s[4] = c[h->cand].nt;
  s[5] = c[h->cand].rows;
  s[6] = c[h->cand].minb;
  s[7] = bytes;
  s[8] = c[h->cand].staged;
  return SMGPU_OK;
}

int smgpu_batch_timings(const smgpu_batch* h, double* t) {
  if (!h || !t) return SMGPU_ERR_ARG;
  for (int k = 0; k < 8; ++k) t[k] = h->times[k];
  return SMGPU_OK;
}

int smgpu_batch_time_matvec(smgpu_batch* h, int reps, int flush_l2, double* ms_out) {
  if (!h || !ms_out || reps < 1) return fail(h, SMGPU_ERR_ARG, "bad time_matvec arguments");
  return guarded(h, [&]() {
    DeviceArena tmp;
    cudaEvent_t a = nullptr, b = nullptr;
    try {
      const BatchDev B = h->view();
      double* d_w0 = tmp.alloc<double>(h->LEN);
      float* d_v = tmp.alloc<float>(h->LEN);
      double* d_w = tmp.alloc<double>(h->LEN);
      char* flush = flush_l2 ? tmp.alloc<char>(256u << 20) : nullptr;
      launch_b_start(B, 1234ull, d_w0, h->st);
      launch_b_convert(B, d_w0, d_v, h->st);
      SMGPU_CUDA_TRY(cudaEventCreate(&a));
      SMGPU_CUDA_TRY(cudaEventCreate(&b));
      double total = 0.0;
      for (int r = 0; r < reps; ++r) {
        if (flush) SMGPU_CUDA_TRY(cudaMemsetAsync(flush, r & 0xff, 256u << 20, h->st));
        SMGPU_CUDA_TRY(cudaEventRecord(a, h->st));
        h->hv(d_v, d_w, BatchEpi{}, h->st);
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

}  // extern "C"
