// The problem handle behind the C ABI (shared by capi.cu and multi.cu).
#pragma once
#include <algorithm>
#include <new>
#include <cstdint>
#include <map>
#include <string>
#include <utility>
#include <vector>

#include "../../include/smgpu.h"
#include "device.cuh"
#include "setup.h"

namespace smgpu {

// Device allocations freed together.  Small requests are carved (256-byte
// aligned) from slabs of doubling size, 1 MB .. 64 MB, so building a
// problem's few dozen tables costs a handful of cudaMalloc calls; a request
// that does not fit the next slab gets its own allocation.
struct DeviceArena {
  std::vector<void*> ptrs;
  size_t bytes = 0;
  char* slab = nullptr;
  size_t slab_left = 0, next_slab = (size_t)1 << 20;
  static constexpr size_t kAlign = 256, kMaxSlab = (size_t)64 << 20;
  void* raw(size_t b) {
    void* p = nullptr;
    cudaError_t e = cudaMalloc(&p, b);
    if (e != cudaSuccess) throw CudaError{e, "cudaMalloc", __FILE__, __LINE__};
    ptrs.push_back(p);
    return p;
  }
  template <class T>
  T* alloc(size_t n) {
    size_t b = sizeof(T) * (n > 0 ? n : 1);
    b = (b + kAlign - 1) & ~(kAlign - 1);
    bytes += b;
    if (b > slab_left) {
      if (b > next_slab) return (T*)raw(b);
      slab = (char*)raw(next_slab);
      slab_left = next_slab;
      next_slab = std::min(next_slab * 2, kMaxSlab);
    }
    T* p = (T*)slab;
    slab += b;
    slab_left -= b;
    return p;
  }
  template <class T>
  T* upload(const std::vector<T>& v) {
    T* p = alloc<T>(v.size());
    if (!v.empty()) SMGPU_CUDA_TRY(cudaMemcpy(p, v.data(), sizeof(T) * v.size(), cudaMemcpyHostToDevice));
    return p;
  }
  void free_all() {
    for (void* p : ptrs) cudaFree(p);
    ptrs.clear();
    bytes = 0;
    slab = nullptr;
    slab_left = 0;
    next_slab = (size_t)1 << 20;
  }
};

// (hi, lo) FP32 pairs with hi + lo = x to about 48 bits.
inline std::vector<float2> to_df(const std::vector<double>& v) {
  std::vector<float2> r(v.size());
  for (size_t i = 0; i < v.size(); ++i) {
    const float hi = (float)v[i];
    r[i] = make_float2(hi, (float)(v[i] - (double)hi));
  }
  return r;
}

template <class T>
std::vector<float> to_f32(const std::vector<T>& v) {
  std::vector<float> r(v.size());
  for (size_t i = 0; i < v.size(); ++i) r[i] = (float)v[i];
  return r;
}

// Per ΔM, the pn table [nA][nB] followed by its negation (the kernels fold
// the neutron sign into the column index).
inline std::vector<double> signed_vtab(const Tables& T) {
  std::vector<double> vt2(2 * T.vtab.size());
  for (size_t k = 0; k + 1 < T.vtab_off_dm.size(); ++k) {
    const int64_t o = T.vtab_off_dm[k], n = T.vtab_off_dm[k + 1] - o;
    for (int64_t x = 0; x < n; ++x) {
      vt2[2 * o + x] = T.vtab[o + x];
      vt2[2 * o + n + x] = -T.vtab[o + x];
    }
  }
  return vt2;
}

}  // namespace smgpu

using namespace smgpu;

struct smgpu_problem {
  int precision = SMGPU_FP64;
  int vp = 0, vn = 0, mtot2 = 0;
  Tables T;
  DeviceArena tables;
  DevTables dt{};
  TileTables tt{};
  CoefTables<double> c64{};
  CoefTables<float> c32{};
  const double* d_ep = nullptr;
  const double* d_en = nullptr;
  const float2* d_ep2 = nullptr;  // one-body diagonals as double-float pairs (FP32-mixed solve)
  const float2* d_en2 = nullptr;
  HvConfig cfg{128, 4, 0, 1, 0};
  int nnmax_raw = 0;  // largest nn[b]
  std::map<int, std::pair<const int*, const int*>> task_arrays;  // rows -> (task_b, task_p0)
  std::map<int, int> task_count;
  cudaStream_t st = nullptr, st2 = nullptr;
  std::string err;
  double times[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  std::vector<HvConfig> tune_shapes;  // candidates timed by the last autotune
  std::vector<double> tune_ms;        // their mean ms per H·v launch
  int sms = 152;
  DeviceArena solver;  // Krylov basis and scratch of the last solve
  Interaction I;       // the interaction the tables were built from
  smgpu_problem* jj_op = nullptr;  // J^2 on the same basis (built on first use)

  ~smgpu_problem() {
    delete jj_op;
    solver.free_all();
    tables.free_all();
    if (st) cudaStreamDestroy(st);
    if (st2) cudaStreamDestroy(st2);
  }

  // Row tasks of R rows each, largest blocks first.
  void ensure_tasks(int R) {
    if (task_arrays.count(R)) return;
    std::vector<int> order(T.nb);
    for (int b = 0; b < T.nb; ++b) order[b] = b;
    std::stable_sort(order.begin(), order.end(), [&](int x, int y) {
      return (int64_t)T.nn[x] * (T.ppn_ptr[T.pstart[x + 1]] - T.ppn_ptr[T.pstart[x]] + 1) >
             (int64_t)T.nn[y] * (T.ppn_ptr[T.pstart[y + 1]] - T.ppn_ptr[T.pstart[y]] + 1);
    });
    std::vector<int> tb, tp;
    for (int b : order)
      for (int p0 = 0; p0 < T.np[b]; p0 += R) {
        tb.push_back(b);
        tp.push_back(p0);
      }
    task_arrays[R] = {tables.upload(tb), tables.upload(tp)};
    task_count[R] = (int)tb.size();
  }
  void set_config(int nt, int R, int minb, int staged = 0) {
    ensure_tasks(R);
    cfg.nt = nt;
    cfg.rows = R;
    cfg.minb = minb;
    cfg.staged = staged;
    cfg.ntasks = task_count[R];
    tt.task_b = task_arrays[R].first;
    tt.task_p0 = task_arrays[R].second;
    if (staged) hv_staged_prepare(cfg, tt);
  }

  // Push lists of the staged pn kernel (hv_staged.cu): every link's neutron
  // pull entries regrouped by source column, each carrying the slot of its
  // output column.  Leaves tt.push_ent null when the packing limits are
  // exceeded (the row-tile kernel is then the only H·v form).
  void build_staged(const std::vector<int>& rl) {
    tt.push_ent = nullptr;
    const size_t nl = T.links.size();
    std::vector<int64_t> poff(nl), pioff(nl);
    std::vector<int> pinfo;
    std::vector<uint32_t> pell;
    int64_t ymax = 0;
    int nbmax = 0, kmax = 0;
    nnmax_raw = 0;
    for (int b = 0; b < T.nb; ++b) nnmax_raw = std::max(nnmax_raw, T.nn[b]);
    if (T.len_pad >= ((int64_t)1 << 31)) return;
    // the links are independent: built in parallel into per-link arrays,
    // then concatenated in link order (the same tables as a serial build)
    struct LinkPush {
      std::vector<uint32_t> ell;  // [k][position]
      std::vector<int> info;      // per position: source column | count << 16
      int64_t y = 0;              // slots of the link
      int bad = 0;                // a packing limit is exceeded
      int nomem = 0;
    };
    std::vector<LinkPush> lp(nl);
#pragma omp parallel for schedule(dynamic, 1)
    for (long lii = 0; lii < (long)nl; ++lii) {
      try {
        const size_t li = (size_t)lii;
        const auto& L = T.links[li];
        const int nno = T.nn[L.b], nns = T.nn[L.s];
        const int64_t* np_ = T.npn_ptr.data() + L.nptr_off;
        std::vector<int64_t> cnt(nns + 1, 0);
        int64_t kw = 0;
        for (int n = 0; n < nno; ++n) {
          kw = std::max(kw, np_[n + 1] - np_[n]);
          for (int64_t g = np_[n]; g < np_[n + 1]; ++g) cnt[(T.npn_ent[g] >> 14) + 1]++;
        }
        if (kw * nno > 65536 || L.nB >= (1 << 15)) {
          lp[li].bad = 1;
          continue;
        }
        lp[li].y = kw * nno;
        // source columns in descending order of their entry counts within
        // windows of 128 consecutive columns: the lanes of a warp carry lists
        // of about the same length, and a warp's loads of v stay inside four
        // 128-byte lines
        std::vector<int> order(nns);
        for (int n = 0; n < nns; ++n) order[n] = n;
        for (int w0 = 0; w0 < nns; w0 += 128) {
          std::stable_sort(order.begin() + w0, order.begin() + std::min(nns, w0 + 128),
                           [&](int x, int y) { return cnt[x + 1] > cnt[y + 1]; });
          // full windows: the four 32-column groups (longest first) rotate over
          // the warps from window to window, so no warp always gets the longest
          if (w0 + 128 <= nns) {
            const int rot = (w0 / 128) % 4;
            std::vector<int> win(order.begin() + w0, order.begin() + w0 + 128);
            for (int g = 0; g < 4; ++g)
              for (int l = 0; l < 32; ++l) order[w0 + ((g + rot) % 4) * 32 + l] = win[g * 32 + l];
          }
        }
        std::vector<int64_t> start(nns + 1, 0);  // entry offset of each source column (position order)
        std::vector<int> posof(nns);
        for (int q = 0; q < nns; ++q) {
          posof[order[q]] = q;
          start[q + 1] = start[q] + cnt[order[q] + 1];
        }
        std::vector<uint32_t> pent(start[nns]);
        std::vector<int64_t> pos(start.begin(), start.end() - 1);
        for (int n = 0; n < nno; ++n)
          for (int64_t g = np_[n]; g < np_[n + 1]; ++g) {
            const uint32_t e = T.npn_ent[g];
            const uint32_t src = e >> 14, ib = (e >> 1) & 0x1fffu, sg = e & 1u;
            const uint32_t slot = (uint32_t)((g - np_[n]) * nno + n);
            pent[pos[posof[src]]++] = slot | (ib << 16) | (sg << 31);
          }
        // each list by operator index: lanes at the same position then tend to
        // read the same or neighbouring coefficient rows (fewer bank conflicts)
        for (int q = 0; q < nns; ++q)
          std::sort(pent.begin() + start[q], pent.begin() + start[q + 1],
                    [](uint32_t x, uint32_t y) { return ((x >> 16) & 0x7fffu) < ((y >> 16) & 0x7fffu); });
        // ELL [k][position] and the per-position descriptors
        int64_t kwp = 0;
        for (int q = 0; q < nns; ++q) kwp = std::max(kwp, start[q + 1] - start[q]);
        if (nns >= 65536 || kwp >= 32768) {
          lp[li].bad = 1;
          continue;
        }
        lp[li].ell.assign((size_t)kwp * nns, 0u);
        lp[li].info.resize(nns);
        for (int q = 0; q < nns; ++q) {
          const int64_t c = start[q + 1] - start[q];
          lp[li].info[q] = order[q] | (int)(c << 16);
          for (int64_t k = 0; k < c; ++k) lp[li].ell[k * nns + q] = pent[start[q] + k];
        }
      } catch (const std::bad_alloc&) {
        lp[(size_t)lii].nomem = 1;
      }
    }
    for (const LinkPush& x : lp)
      if (x.nomem) throw std::bad_alloc();
    for (const LinkPush& x : lp)
      if (x.bad) return;
    // every link's lists must be present before the kernels index them
    for (size_t li = 0; li < nl; ++li)
      if (lp[li].info.size() != (size_t)T.nn[T.links[li].s])
        throw SetupError{SMGPU_ERR_LIMIT, "staged push lists incomplete"};
    for (size_t li = 0; li < nl; ++li) {
      ymax = std::max(ymax, lp[li].y);
      nbmax = std::max(nbmax, T.links[li].nB);
      poff[li] = (int64_t)pell.size();
      pioff[li] = (int64_t)pinfo.size();
      pell.insert(pell.end(), lp[li].ell.begin(), lp[li].ell.end());
      pinfo.insert(pinfo.end(), lp[li].info.begin(), lp[li].info.end());
      std::vector<uint32_t>().swap(lp[li].ell);
    }
    for (size_t k = 0; k + 1 < rl.size(); ++k) kmax = std::max(kmax, rl[k + 1] - rl[k]);
    // nn lists as ELL [k][n] per block
    std::vector<int64_t> eoff(T.nb);
    std::vector<int> ew(T.nb), ecol;
    std::vector<float> evl;
    for (int b = 0; b < T.nb; ++b) {
      const int nnb = T.nn[b], g0 = T.nstart[b];
      int w = 0;
      for (int n = 0; n < nnb; ++n) w = std::max(w, T.nn_ptr[g0 + n + 1] - T.nn_ptr[g0 + n]);
      eoff[b] = (int64_t)ecol.size();
      ew[b] = w;
      ecol.resize(ecol.size() + (size_t)w * nnb);
      evl.resize(ecol.size());
      for (int n = 0; n < nnb; ++n) {
        const int kb = T.nn_ptr[g0 + n], ke = T.nn_ptr[g0 + n + 1];
        for (int k = 0; k < w; ++k) {
          const size_t o = (size_t)eoff[b] + (size_t)k * nnb + n;
          ecol[o] = kb + k < ke ? T.nn_col[kb + k] : n;
          evl[o] = kb + k < ke ? (float)T.nn_val[kb + k] : 0.f;
        }
      }
    }
    tt.nnell_off = tables.upload(eoff);
    tt.nnell_w = tables.upload(ew);
    tt.nnell_col = tables.upload(ecol);
    tt.nnell_val = tables.upload(evl);
    tt.push_off = tables.upload(poff);
    tt.push_ioff = tables.upload(pioff);
    tt.push_info = tables.upload(pinfo);
    tt.push_ent = tables.upload(pell);
    tt.ymax = (int)((ymax + 3) & ~(int64_t)3);
    tt.nnmax = (nnmax_raw + 3) & ~3;
    tt.nbmax = std::max(nbmax, 1);
    tt.kpad = std::max(4, (kmax + 3) & ~3);
    tt.astride = (tt.kpad % 8 == 0) ? tt.kpad + 4 : tt.kpad;
    build_2b_tasks();
  }

  // Tasks of the two-body pass (hv_2b.cu), largest estimated work first:
  // pp tasks of 32 columns x kPPRows rows, nn tasks of 32 rows x kNNCols
  // columns, covering every element of every block; and its output array.
  void build_2b_tasks() {
    struct Item {
      double cost;
      int4 t;
    };
    std::vector<Item> pp, nn;
    for (int b = 0; b < T.nb; ++b) {
      const int npb = T.np[b], nnb = T.nn[b];
      for (int r0 = 0; r0 < npb; r0 += kPPRows) {
        const int nr = std::min(kPPRows, npb - r0);
        const double e = (double)(T.pp_ptr[T.pstart[b] + r0 + nr] - T.pp_ptr[T.pstart[b] + r0]) + nr;
        for (int n0 = 0; n0 < nnb; n0 += 32) pp.push_back({e, make_int4(b, r0, n0, nr)});
      }
      for (int c0 = 0; c0 < nnb; c0 += kNNCols) {
        const int nc = std::min(kNNCols, nnb - c0);
        const double e = (double)(T.nn_ptr[T.nstart[b] + c0 + nc] - T.nn_ptr[T.nstart[b] + c0]) + nc + nnb / 8.0;
        for (int r0 = 0; r0 < npb; r0 += 32) nn.push_back({e, make_int4(b, r0, c0, nc)});
      }
    }
    auto order = [](std::vector<Item>& v) {
      std::stable_sort(v.begin(), v.end(), [](const Item& x, const Item& y) { return x.cost > y.cost; });
      std::vector<int4> out(v.size());
      for (size_t k = 0; k < v.size(); ++k) out[k] = v[k].t;
      return out;
    };
    const std::vector<int4> ppt = order(pp), nnt = order(nn);
    tt.pp_tasks = tables.upload(ppt);
    tt.nn_tasks = tables.upload(nnt);
    tt.n_pp_tasks = (int)ppt.size();
    tt.n_nn_tasks = (int)nnt.size();
    tt.npmax = 1;
    for (int b = 0; b < T.nb; ++b) tt.npmax = std::max(tt.npmax, T.np[b]);
    tt.s2b = tables.alloc<float>(2 * (size_t)T.len_pad);
  }

  // Device copies of the tables.  with_streams = false for problems that run
  // on a batch's streams.
  void upload(bool with_streams = true) {
    if (with_streams) {
      // the eigenvalue test runs beside the main chain on st2: highest
      // priority, so its single CTA is scheduled as soon as an SM frees
      int prio_lo = 0, prio_hi = 0;
      SMGPU_CUDA_TRY(cudaDeviceGetStreamPriorityRange(&prio_lo, &prio_hi));
      SMGPU_CUDA_TRY(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
      SMGPU_CUDA_TRY(cudaStreamCreateWithPriority(&st2, cudaStreamNonBlocking, prio_hi));
    }
    int dev = 0;
    SMGPU_CUDA_TRY(cudaGetDevice(&dev));
    SMGPU_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    const int nb = T.nb;
    dt.nb = nb;
    dt.len_pad = T.len_pad;
    dt.np = tables.upload(T.np);
    dt.nn = tables.upload(T.nn);
    dt.stride = tables.upload(T.stride);
    dt.off_pad = tables.upload(T.off_pad);
    dt.pstart = tables.upload(T.pstart);
    dt.nstart = tables.upload(T.nstart);
    dt.tdims = tables.upload(T.tdims);
    dt.pp_ptr = tables.upload(T.pp_ptr);
    dt.pp_col = tables.upload(T.pp_col);
    dt.nn_ptr = tables.upload(T.nn_ptr);
    dt.nn_col = tables.upload(T.nn_col);
    std::vector<int4> la(T.links.size());
    std::vector<int64_t> lv(T.links.size()), ln(T.links.size());
    for (size_t k = 0; k < T.links.size(); ++k) {
      la[k] = make_int4(T.links[k].s, T.links[k].nB, T.links[k].dm, 0);
      lv[k] = 2 * T.links[k].vtab_off;  // signed (V, -V) table
      ln[k] = T.links[k].nptr_off;
    }
    dt.link_a = tables.upload(la);
    dt.link_v = tables.upload(lv);
    dt.link_n = tables.upload(ln);
    dt.ppn_src = tables.upload(T.ppn_src);
    dt.ppn_meta = tables.upload(T.ppn_meta);
    d_ep = tables.upload(T.ep);
    d_en = tables.upload(T.en);
    // row-tile tables: per (row, link slot) first proton entry
    std::vector<int64_t> rl_base(nb);
    std::vector<int> rl;
    for (int b = 0; b < nb; ++b) {
      rl_base[b] = (int64_t)rl.size();
      const int lb = T.link_begin[b], nl = T.link_begin[b + 1] - lb;
      for (int g = T.pstart[b]; g < T.pstart[b + 1]; ++g) {
        int e = T.ppn_ptr[g];
        for (int j = 0; j <= nl; ++j) {
          while (e < T.ppn_ptr[g + 1] && (int)(T.ppn_meta[e] >> 16) < lb + j) ++e;
          rl.push_back(e);
        }
      }
    }
    tt.link_begin = tables.upload(T.link_begin);
    tt.rl_base = tables.upload(rl_base);
    tt.rl = tables.upload(rl);
    tt.npn_ptr = tables.upload(T.npn_ptr);
    // neutron entries with the sign folded into the (V, -V) table index
    std::vector<uint32_t> ent(T.npn_ent.size());
    for (size_t li = 0; li < T.links.size(); ++li) {
      const auto& L = T.links[li];
      const uint32_t nab = (uint32_t)(L.nA * L.nB);
      for (int64_t j = T.npn_ptr[L.nptr_off]; j < T.npn_ptr[L.nptr_off + T.nn[L.b]]; ++j) {
        uint32_t e = T.npn_ent[j];
        uint32_t col = ((e >> 1) & 0x1fffu) + ((e & 1u) ? nab : 0u);
        if (col >= (1u << 14)) throw SetupError{SMGPU_ERR_LIMIT, "pn coefficient table too large for the packing"};
        ent[j] = (e & ~0x3fffu) | col;
      }
    }
    tt.npn_ent = tables.upload(ent);
    if (precision != SMGPU_FP64) build_staged(rl);
    // signed coefficient tables
    const std::vector<double> vt2 = signed_vtab(T);
    if (precision == SMGPU_FP64) {
      c64.pp_val = tables.upload(T.pp_val);
      c64.nn_val = tables.upload(T.nn_val);
      c64.vtab = tables.upload(vt2);
    } else {
      c32.pp_val = tables.upload(to_f32(T.pp_val));
      c32.nn_val = tables.upload(to_f32(T.nn_val));
      c32.vtab = tables.upload(to_f32(vt2));
      d_ep2 = tables.upload(to_df(T.ep));
      d_en2 = tables.upload(to_df(T.en));
    }
    set_config(128, 4, 1);
    // the synchronous uploads run on the legacy stream; the handle's streams
    // are non-blocking, so finish them before any kernel reads the tables
    SMGPU_CUDA_TRY(cudaDeviceSynchronize());
  }

  // FP64 coefficient tables for a handle created in the mixed form (the
  // J-projected solve always runs in FP64).
  void ensure_fp64() {
    if (c64.pp_val) return;
    c64.pp_val = tables.upload(T.pp_val);
    c64.nn_val = tables.upload(T.nn_val);
    c64.vtab = tables.upload(signed_vtab(T));
  }

  void hv(const double* v, double* w, const HvEpilogue<double>& epi, cudaStream_t s) {
    launch_hv_fp64(dt, tt, cfg, d_ep, d_en, c64, v, w, epi, s);
  }
  void hv(const float* v, double* w, const HvEpilogue<float>& epi, cudaStream_t s) {
    if (cfg.staged) launch_hv_staged_mixed(dt, tt, cfg, d_ep, d_en, c32, v, w, epi, s);
    else launch_hv_mixed(dt, tt, cfg, d_ep, d_en, c32, v, w, epi, s);
  }
  // FP32-mixed H·v with the Lanczos epilogue in double-float (w = wh + wl)
  void hv_df(const float* v, float* wh, float* wl, const HvEpilogue<float>& epi, cudaStream_t s) {
    if (cfg.staged) launch_hv_staged_mixed_df(dt, tt, cfg, d_ep2, d_en2, c32, v, wh, wl, epi, s);
    else launch_hv_mixed_df(dt, tt, cfg, d_ep2, d_en2, c32, v, wh, wl, epi, s);
  }

  // Time every candidate launch shape on a device vector and keep the fastest
  // (defined in capi.cu, next to the shape-class cache).
  void autotune();
};
