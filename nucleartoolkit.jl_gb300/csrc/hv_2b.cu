// Two-body (pp and nn) terms of the staged FP32-mixed H·v, as a pass of its
// own ahead of the staged pn kernel (hv_staged.cu).
//
// On block b the Lanczos vector is an np × nn matrix V (rows: proton Slater
// determinants, columns: neutron ones).  The like-particle terms of
// operate_H! (src/ShellModel/lanczos_methods.jl:153-248, the pp_2bjump and
// nn_2bjump loops) are two sparse products on that matrix:
//
//   pp:  W[p, n] += Σ_{(p', c) ∈ pp(p)} c V[p', n]      rows mix, columns ride along
//   nn:  W[p, n] += Σ_{(n', c) ∈ nn(n)} c V[p, n']      columns mix, rows ride along
//
// Each is computed with the 32 lanes of a warp along the index that rides
// along, so a sparse list entry is read once per 32 lanes instead of once per
// row or column (the staged kernel used to re-read every nn list once per
// row: 1.9 GB of index and coefficient loads per 48Cr H·v):
//   pp task = 32 columns (the lanes) × up to kPPRows rows (a contiguous range
//             per warp); the block's 32-column slab of V is staged in shared
//             memory, [p'][lane], so every gather is conflict-free.
//   nn task = 32 rows (the lanes) × up to kNNCols columns (kNNGroup per warp
//             pass); the 32 rows of V are staged with an odd row stride, so
//             the lanes' gathers V[lane, n'] hit 32 distinct banks; a
//             finished column is stored by its 32 lanes (one row each).
// Staging uses cp.async (all of a thread's copies in flight at once).  A warp
// streams the concatenated lists of its rows (pp) or columns (nn) —
// contiguous in the CSR tables — in coalesced 32-entry chunks, the next chunk
// loaded while the current one is applied from shared memory; a list
// boundary closes the running sum.  Sums are FP32 (two interleaved partial
// sums per list, added at its end); the staged kernel adds them to its
// Kahan-compensated pn sum.  Every element of every block is written (zero
// when its list is empty).
#include <algorithm>

#include "device.cuh"

namespace smgpu {

namespace {

constexpr int kNT2 = 512;  // 16 warps: two CTAs per SM fill 32 warp slots beside ~77 KB of staged rows each
constexpr int kW2 = kNT2 / 32;
constexpr int kNNGroup = 16;  // columns of an nn task per warp pass
constexpr unsigned kFull = 0xffffffffu;

// Asynchronous global -> shared copies (cp.async): a thread issues all of its
// copies of a staging loop back to back and waits once, so the staging costs
// about one memory latency instead of one per loop trip.
__device__ __forceinline__ void cp_async4(float* dst, const float* src) {
  const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(d), "l"(src) : "memory");
}
// 16 bytes; both addresses 16-byte aligned
__device__ __forceinline__ void cp_async16(float* dst, const float* src) {
  const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }

// Applies the entries [ebeg, eend) of a CSR list stream, whose sub-list
// boundaries are lend[0..nl) (nl <= 32; the end of sub-list k is lane k's
// `lend`), to the lane's gather source: entry (c, x) adds x * src[c * ss].
// emit(k, sum) is called once per sub-list, in order, empty ones included.
// The entries go through the warp's two 32-entry buffers in shared memory
// (buf: 2 x 32 int2): a chunk is loaded coalesced into registers while the
// previous one is applied from its buffer, every entry is one broadcast
// 8-byte shared load (column premultiplied by ss), and the running sum
// alternates between two FP32 accumulators (pairs of consecutive entries of
// a chunk; their sum closes a list).  Warp-uniform control flow throughout;
// every pass of the inner loop consumes at least one entry, so the loops end
// even on inconsistent tables.
template <class Emit>
__device__ __forceinline__ void stream_lists(const int* __restrict__ col, const float* __restrict__ val, int ebeg,
                                             int eend, int lend, int nl, const float* src, int ss, int2* buf,
                                             Emit emit) {
  const int lane = threadIdx.x & 31;
  int k = 0;
  int kend = __shfl_sync(kFull, lend, 0);
  while (k < nl && ebeg == kend) {  // leading empty lists
    emit(k, 0.f);
    ++k;
    kend = __shfl_sync(kFull, lend, k & 31);
  }
  float acc0 = 0.f, acc1 = 0.f;
  int cn = 0;
  float vn = 0.f;
  if (ebeg + lane < eend) {
    cn = col[ebeg + lane];
    vn = val[ebeg + lane];
  }
  int cur = 0;
  for (int e0 = ebeg; e0 < eend; e0 += 32) {
    int2* b = buf + 32 * cur;
    b[lane] = make_int2(cn * ss, __float_as_int(vn));
    __syncwarp();
    const int cnt = min(32, eend - e0);
    if (e0 + 32 + lane < eend) {  // the next chunk, in flight while this one is applied
      cn = col[e0 + 32 + lane];
      vn = val[e0 + 32 + lane];
    }
    int j = 0;
    while (j < cnt) {
      // entries [j, run) of this chunk belong to sub-list k (kend > e0 + j for
      // consistent tables; at least one entry per pass in any case)
      const int run = min(cnt, max(j + 1, kend - e0));
#pragma unroll 2
      for (; j + 1 < run; j += 2) {  // pairs of entries into the two accumulators
        const int2 ea = b[j], eb = b[j + 1];
        acc0 = __fmaf_rn(__int_as_float(ea.y), src[ea.x], acc0);
        acc1 = __fmaf_rn(__int_as_float(eb.y), src[eb.x], acc1);
      }
      if (j < run) {
        const int2 ea = b[j];
        acc0 = __fmaf_rn(__int_as_float(ea.y), src[ea.x], acc0);
        ++j;
      }
      if (e0 + j == kend) {  // sub-list k ends here (uniform); then any empty ones
        emit(k, __fadd_rn(acc0, acc1));
        acc0 = 0.f;
        acc1 = 0.f;
        ++k;
        kend = __shfl_sync(kFull, lend, k & 31);
        while (k < nl && e0 + j == kend) {
          emit(k, 0.f);
          ++k;
          kend = __shfl_sync(kFull, lend, k & 31);
        }
      }
    }
    cur ^= 1;
  }
}

// pp task tk = (block, first row, first column, rows).
__device__ __forceinline__ void pp_task(const DevTables& t, const int4 tk, const float* __restrict__ pp_val,
                                        const float* __restrict__ v, float* __restrict__ s_pp, float* sm,
                                        int2 (*ebuf)[64]) {
  const int b = tk.x, r0 = tk.y, n0 = tk.z, nr = tk.w;
  const int np = t.np[b], nn = t.nn[b], stride = t.stride[b];
  const int64_t blk = t.off_pad[b];
  const int pst = t.pstart[b];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int n = n0 + lane;
  const bool act = n < nn;
  // the block's 32-column slab, [row][lane], in 16-byte pieces (rows start
  // 16-byte aligned, stride and n0 are multiples of 4); pieces past the
  // padded row are zero (their lanes' results are not stored)
  for (int idx = threadIdx.x; idx < np * 8; idx += kNT2) {
    const int p = idx >> 3, c4 = n0 + 4 * (idx & 7);
    float* dst = sm + p * 32 + 4 * (idx & 7);
    if (c4 < stride) cp_async16(dst, v + blk + (int64_t)p * stride + c4);
    else *reinterpret_cast<float4*>(dst) = make_float4(0.f, 0.f, 0.f, 0.f);
  }
  cp_async_wait_all();
  __syncthreads();
  // warp w: rows [ra, rb), at most 32
  const int per = (nr + kW2 - 1) / kW2;
  const int ra = r0 + min(nr, w * per), rb = r0 + min(nr, (w + 1) * per);
  if (ra >= rb) return;
  const int nrw = rb - ra;
  const int lend = lane < nrw ? t.pp_ptr[pst + ra + lane + 1] : 0;
  const int ebeg = t.pp_ptr[pst + ra], eend = __shfl_sync(kFull, lend, nrw - 1);
  stream_lists(t.pp_col, pp_val, ebeg, eend, lend, nrw, sm + lane, 32, ebuf[w], [&](int k, float sum) {
    if (act) s_pp[blk + (int64_t)(ra + k) * stride + n] = sum;
  });
}

// nn task tk = (block, first row, first column, columns).
__device__ __forceinline__ void nn_task(const DevTables& t, const int4 tk, const float* __restrict__ nn_val,
                                        const float* __restrict__ v, float* __restrict__ s_nn, float* sm,
                                        int2 (*ebuf)[64]) {
  const int b = tk.x, r0 = tk.y, c0 = tk.z, nc = tk.w;
  const int np = t.np[b], nn = t.nn[b], stride = t.stride[b];
  const int nr = min(32, np - r0);
  const int64_t blk = t.off_pad[b];
  const int nst = t.nstart[b];
  const int ls = nn | 1;  // odd row stride: lane r reads bank (r*ls + n') mod 32, distinct over r
  float* vs = sm;         // [32][ls] rows r0 .. r0+31 of the block (zero beyond nr)
  for (int idx = threadIdx.x; idx < 32 * nn; idx += kNT2) {
    const int r = idx / nn, c = idx - r * nn;
    if (r < nr) cp_async4(vs + r * ls + c, v + blk + (int64_t)(r0 + r) * stride + c);
    else vs[r * ls + c] = 0.f;
  }
  cp_async_wait_all();
  __syncthreads();
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  float* __restrict__ out = s_nn + blk + (int64_t)(r0 + lane) * stride;  // row `lane`
  for (int g0 = c0 + kNNGroup * w; g0 < c0 + nc; g0 += kNNGroup * kW2) {
    const int gc = min(kNNGroup, c0 + nc - g0);
    const int lend = lane < gc ? t.nn_ptr[nst + g0 + lane + 1] : 0;
    const int ebeg = t.nn_ptr[nst + g0], eend = __shfl_sync(kFull, lend, gc - 1);
    // column g0 + k of the 32 rows (one store per lane)
    stream_lists(t.nn_col, nn_val, ebeg, eend, lend, gc, vs + lane * ls, 1, ebuf[w], [&](int k, float sum) {
      if (lane < nr) out[g0 + k] = sum;
    });
  }
}

// One launch for both terms: CTAs [0, n_nn) take the nn tasks, the rest the
// pp tasks (each list largest first), so the short pp tasks fill the tail
// of the nn ones.
__global__ void __launch_bounds__(kNT2) k_hv_2b(const DevTables t, const int4* __restrict__ nn_tasks, int n_nn,
                                                const int4* __restrict__ pp_tasks, const float* __restrict__ nn_val,
                                                const float* __restrict__ pp_val, const float* __restrict__ v,
                                                float* __restrict__ s2b, const LanczosFlags* fl) {
  if (fl != nullptr && cta_gate(threadIdx.x == 0 && (fl->done || fl->exhausted))) return;
  extern __shared__ float sm[];
  __shared__ int2 ebuf[kW2][64];
  const int c = blockIdx.x;
  if (c < n_nn) nn_task(t, nn_tasks[c], nn_val, v, s2b + t.len_pad, sm, ebuf);
  else pp_task(t, pp_tasks[c - n_nn], pp_val, v, s2b, sm, ebuf);
}

}  // namespace

size_t hv_2b_nn_smem(const TileTables& tt) { return sizeof(float) * (size_t)32 * (size_t)((tt.nnmax) | 1); }

size_t hv_2b_pp_smem(const TileTables& tt) { return sizeof(float) * 32 * (size_t)tt.npmax; }

static size_t hv_2b_smem(const TileTables& tt) { return std::max(hv_2b_nn_smem(tt), hv_2b_pp_smem(tt)); }

void hv_2b_prepare(const TileTables& tt) {
  SMGPU_CUDA_TRY(cudaFuncSetAttribute(k_hv_2b, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)hv_2b_smem(tt)));
}

void launch_hv_2b(const DevTables& t, const TileTables& tt, const CoefTables<float>& c, const float* v,
                  const LanczosFlags* fl, cudaStream_t st) {
  const int n = tt.n_nn_tasks + tt.n_pp_tasks;
  if (n > 0)
    k_hv_2b<<<n, kNT2, hv_2b_smem(tt), st>>>(t, tt.nn_tasks, tt.n_nn_tasks, tt.pp_tasks, c.nn_val, c.pp_val, v,
                                             tt.s2b, fl);
}

}  // namespace smgpu
