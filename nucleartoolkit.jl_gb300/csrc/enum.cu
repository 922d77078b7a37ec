// Device-side enumeration of the basis and the jump tables.
//
// Replaces the host loops of the reference's set-up (paths relative to the
// NuclearToolkit.jl tree):
//   occ (basis: lexicographic SDs, M buckets, blocks)   src/ShellModel/shellmodel_main.jl:769-848
//   one-body diagonal dot(SPEs, jocc)                    :808-848 (jocc), lanczos_methods.jl:228-246
//   prep_2bjumps (pp / nn jump lists)                    :1115-1137
//   prep_pn / calc_1b_jumps! (pn jump lists)             :1139-1199
// with kernels: every SD (or every (link, neutron SD) row) is one thread,
// and every variable-length list is built in two passes (count, exclusive
// scan, fill) so the entries come out in the reference's loop order without
// atomics.  The interaction-dependent operator lists (prep_Hamil_T1 /
// prep_Hamil_pn) and the block links are small and stay on the host
// (setup.cpp).  The tables are copied into the host Tables as well: the
// device copies used by H·v are uploaded from there (problem.h), and the
// parity exports read them.
#include <algorithm>
#include <vector>

#include "../../include/smgpu.h"
#include "device.cuh"
#include "problem.h"
#include "sdbits.h"
#include "setup.h"

namespace smgpu {

namespace {
constexpr int kT = 256;

inline int grid_for(int64_t n) {
  int64_t g = (n + kT - 1) / kT;
  if (g > 152 * 16) g = 152 * 16;
  return (int)(g < 1 ? 1 : g);
}

// ------------------------------------------------------------------ scan
template <class TI>
__global__ void __launch_bounds__(kT) k_scan_block(const TI* __restrict__ in, int64_t n, int64_t* __restrict__ out,
                                                   int64_t* __restrict__ bsum) {
  __shared__ int64_t sh[kT];
  const int64_t i = blockIdx.x * (int64_t)kT + threadIdx.x;
  const int64_t x = i < n ? (int64_t)in[i] : 0;
  sh[threadIdx.x] = x;
  __syncthreads();
  for (int o = 1; o < kT; o <<= 1) {
    const int64_t y = threadIdx.x >= o ? sh[threadIdx.x - o] : 0;
    __syncthreads();
    sh[threadIdx.x] += y;
    __syncthreads();
  }
  if (i < n) out[i] = sh[threadIdx.x] - x;
  if (threadIdx.x == kT - 1) bsum[blockIdx.x] = sh[kT - 1];
}

__global__ void k_scan_add(int64_t* __restrict__ out, int64_t n, const int64_t* __restrict__ boff) {
  const int64_t i = blockIdx.x * (int64_t)kT + threadIdx.x;
  if (i < n) out[i] += boff[blockIdx.x];
}

// Exclusive scan of n counts into out (n entries); returns the total.
template <class TI>
int64_t scan_exclusive(DeviceArena& A, const TI* in, int64_t n, int64_t* out, cudaStream_t st) {
  if (n == 0) return 0;
  const int64_t nblk = (n + kT - 1) / kT;
  int64_t* bsum = A.alloc<int64_t>(nblk);
  k_scan_block<TI><<<(unsigned)nblk, kT, 0, st>>>(in, n, out, bsum);
  if (nblk > 1) {
    int64_t* boff = A.alloc<int64_t>(nblk);
    scan_exclusive<int64_t>(A, bsum, nblk, boff, st);
    k_scan_add<<<(unsigned)nblk, kT, 0, st>>>(out, n, boff);
  }
  int64_t last_off = 0;
  TI last_in = 0;
  SMGPU_CUDA_TRY(cudaMemcpyAsync(&last_off, out + n - 1, sizeof(int64_t), cudaMemcpyDeviceToHost, st));
  SMGPU_CUDA_TRY(cudaMemcpyAsync(&last_in, in + n - 1, sizeof(TI), cudaMemcpyDeviceToHost, st));
  SMGPU_CUDA_TRY(cudaStreamSynchronize(st));
  return last_off + (int64_t)last_in;
}

__device__ __forceinline__ int block_of(const int* __restrict__ start, int nb, int64_t g) {
  int lo = 0, hi = nb - 1;  // largest b with start[b] <= g
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (start[mid] <= g) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

// ------------------------------------------------------------------ basis
// r-th k-combination of L m-states in lexicographic order (occ's
// `combinations`), as a bit string, and its doubled M.  C holds the binomial
// coefficients C(n, j) at [n*(L+1) + j].
__global__ void __launch_bounds__(kT) k_combos(int L, int k, const uint64_t* __restrict__ C,
                                               const int* __restrict__ m2, int64_t N, uint64_t* __restrict__ bits,
                                               int* __restrict__ M) {
  for (int64_t r = blockIdx.x * (int64_t)kT + threadIdx.x; r < N; r += (int64_t)gridDim.x * kT) {
    uint64_t rem = (uint64_t)r, b = 0;
    int m = 0, c = 0;
    for (int i = 0; i < k; ++i) {
      while (true) {
        const uint64_t cnt = C[(int64_t)(L - c - 1) * (L + 1) + (k - i - 1)];
        if (rem < cnt) break;
        rem -= cnt;
        ++c;
      }
      b |= sd_bit(L, c);
      m += m2[c];
      ++c;
    }
    bits[r] = b;
    M[r] = m;
  }
}

__global__ void k_bucket_count(const int* __restrict__ M, int64_t N, int Mmin, int* __restrict__ cnt) {
  for (int64_t r = blockIdx.x * (int64_t)kT + threadIdx.x; r < N; r += (int64_t)gridDim.x * kT)
    atomicAdd(&cnt[(M[r] - Mmin) >> 1], 1);
}

// Stable partition of the SDs by M: one CTA per M bucket walks all SDs in
// lexicographic order and appends the ones of its bucket.
__global__ void __launch_bounds__(kT) k_bucket_scatter(const uint64_t* __restrict__ bits, const int* __restrict__ M,
                                                       int64_t N, int Mmin, const int64_t* __restrict__ off,
                                                       uint64_t* __restrict__ out) {
  __shared__ int sh[kT];
  __shared__ int64_t base;
  const int Mv = Mmin + 2 * (int)blockIdx.x;
  if (threadIdx.x == 0) base = off[blockIdx.x];
  __syncthreads();
  for (int64_t r0 = 0; r0 < N; r0 += kT) {
    const int64_t r = r0 + threadIdx.x;
    const int f = (r < N && M[r] == Mv) ? 1 : 0;
    sh[threadIdx.x] = f;
    __syncthreads();
    for (int o = 1; o < kT; o <<= 1) {
      const int y = threadIdx.x >= o ? sh[threadIdx.x - o] : 0;
      __syncthreads();
      sh[threadIdx.x] += y;
      __syncthreads();
    }
    if (f) out[base + sh[threadIdx.x] - 1] = bits[r];
    __syncthreads();
    if (threadIdx.x == kT - 1) base += sh[kT - 1];
    __syncthreads();
  }
}

// dot(SPEs, jocc) per SD, in orbit order, without contraction (as the host).
__global__ void k_onebody(const uint64_t* __restrict__ bits, int64_t N, const uint64_t* __restrict__ omask,
                          const double* __restrict__ spe, int norb, double* __restrict__ e) {
  for (int64_t g = blockIdx.x * (int64_t)kT + threadIdx.x; g < N; g += (int64_t)gridDim.x * kT) {
    double s = 0.0;
    for (int o = 0; o < norb; ++o) s = __dadd_rn(s, __dmul_rn(spe[o], (double)sd_popc(bits[g] & omask[o])));
    e[g] = s;
  }
}

// ------------------------------------------------------- pp / nn pull CSR
// Rows are the SDs of one species (block by block); row g lists, for every
// operator a†b†dc of the species in list order, the SD it reaches in the
// same block (prep_2bjumps).  A pair below the diagonal takes the value and
// sign of the conjugate operator, as the reference stores it on the other
// row.
// One warp per row: lane l takes the l-th contiguous slice of the operator
// list, so the lanes' entries concatenated in lane order are in list order.
__device__ __forceinline__ void op_slice(int nops, int lane, int& k0, int& k1) {
  const int per = (nops + 31) / 32;
  k0 = min(nops, lane * per);
  k1 = min(nops, k0 + per);
}

__global__ void __launch_bounds__(kT) k_2b_count(const Op2* __restrict__ ops, int nops,
                                                 const uint64_t* __restrict__ bits, const int* __restrict__ start,
                                                 int nb, int64_t nrow, int* __restrict__ cnt) {
  const int lane = threadIdx.x & 31;
  const int64_t nwarps = (int64_t)gridDim.x * (kT / 32);
  int k0, k1;
  op_slice(nops, lane, k0, k1);
  for (int64_t g = blockIdx.x * (int64_t)(kT / 32) + (threadIdx.x >> 5); g < nrow; g += nwarps) {
    const int b = block_of(start, nb, g);
    const uint64_t* blk = bits + start[b];
    const int n = start[b + 1] - start[b];
    const uint64_t sd = bits[g];
    int c = 0;
    for (int k = k0; k < k1; ++k) {
      const Op2 o = ops[k];
      if (o.v == 0.0) continue;
      uint64_t f;
      int odd;
      if (!sd_apply2(sd, o.a, o.b, o.c, o.d, f, odd)) continue;
      if (sd_find_desc(blk, n, f) < 0) continue;
      ++c;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
    if (lane == 0) cnt[g] = c;
  }
}

__global__ void __launch_bounds__(kT) k_2b_fill(const Op2* __restrict__ ops, const long* __restrict__ conj, int nops,
                                                const uint64_t* __restrict__ bits, const int* __restrict__ start,
                                                int nb, int64_t nrow, const int64_t* __restrict__ off,
                                                int* __restrict__ col, double* __restrict__ val) {
  const int lane = threadIdx.x & 31;
  const int64_t nwarps = (int64_t)gridDim.x * (kT / 32);
  int k0, k1;
  op_slice(nops, lane, k0, k1);
  for (int64_t g = blockIdx.x * (int64_t)(kT / 32) + (threadIdx.x >> 5); g < nrow; g += nwarps) {
    const int b = block_of(start, nb, g);
    const uint64_t* blk = bits + start[b];
    const int n = start[b + 1] - start[b];
    const int i = (int)(g - start[b]);
    const uint64_t sd = bits[g];
    // this lane's count, then its offset by an exclusive warp scan
    int c = 0;
    for (int k = k0; k < k1; ++k) {
      const Op2 o = ops[k];
      if (o.v == 0.0) continue;
      uint64_t f;
      int odd;
      if (!sd_apply2(sd, o.a, o.b, o.c, o.d, f, odd)) continue;
      if (sd_find_desc(blk, n, f) < 0) continue;
      ++c;
    }
    int incl = c;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += y;
    }
    int64_t w = off[g] + (incl - c);
    for (int k = k0; k < k1; ++k) {
      const Op2 o = ops[k];
      if (o.v == 0.0) continue;
      uint64_t f;
      int odd;
      if (!sd_apply2(sd, o.a, o.b, o.c, o.d, f, odd)) continue;
      const int j = sd_find_desc(blk, n, f);
      if (j < 0) continue;
      double v = o.v;
      if (j < i && conj[k] >= 0) {
        const Op2 oc = ops[conj[k]];
        uint64_t f2;
        int odd2;
        if (sd_apply2(f, oc.a, oc.b, oc.c, oc.d, f2, odd2) && f2 == sd && oc.v != 0.0) {
          v = oc.v;
          odd = odd2;
        }
      }
      col[w] = j;
      val[w] = odd ? -v : v;
      ++w;
    }
  }
}

// Per row: stable sort by column, then sum equal columns in list order.
// One warp per row: the row's entries go to shared memory, each lane ranks
// its entries (entries with a smaller column, plus equal columns earlier in
// the list: a stable order) and scatters them; then each group of equal
// columns is summed left to right by one lane — the same additions in the
// same order as the sequential merge.  Rows longer than kMergeMax entries
// take the sequential merge in global memory (one lane).
constexpr int kMergeWarps = 8;
constexpr int kMergeMax = 512;
size_t merge_smem() { return (size_t)kMergeWarps * kMergeMax * 2 * (sizeof(int) + sizeof(double)); }

__device__ void merge_row_serial(int* c, double* v, int n, int* mout) {
  for (int a = 1; a < n; ++a) {
    const int kc = c[a];
    const double kv = v[a];
    int p = a - 1;
    while (p >= 0 && c[p] > kc) {
      c[p + 1] = c[p];
      v[p + 1] = v[p];
      --p;
    }
    c[p + 1] = kc;
    v[p + 1] = kv;
  }
  int m = 0;
  for (int a = 0; a < n; ++a) {
    if (m > 0 && c[m - 1] == c[a]) {
      v[m - 1] = __dadd_rn(v[m - 1], v[a]);
    } else {
      c[m] = c[a];
      v[m] = v[a];
      ++m;
    }
  }
  *mout = m;
}

__global__ void __launch_bounds__(kMergeWarps * 32) k_2b_merge(int64_t nrow, const int64_t* __restrict__ off,
                                                               const int* __restrict__ cnt, int* __restrict__ col,
                                                               double* __restrict__ val, int* __restrict__ mcnt) {
  extern __shared__ double msm[];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  double* vin = msm + (size_t)wid * kMergeMax * 2;
  double* vs = vin + kMergeMax;
  int* cin = reinterpret_cast<int*>(msm + (size_t)kMergeWarps * kMergeMax * 2) + (size_t)wid * kMergeMax * 2;
  int* cs = cin + kMergeMax;
  const unsigned full = 0xffffffffu;
  for (int64_t g = blockIdx.x * (int64_t)kMergeWarps + wid; g < nrow; g += (int64_t)gridDim.x * kMergeWarps) {
    int* c = col + off[g];
    double* v = val + off[g];
    const int n = cnt[g];
    if (n > kMergeMax) {
      if (lane == 0) merge_row_serial(c, v, n, mcnt + g);
      __syncwarp();
      continue;
    }
    for (int a = lane; a < n; a += 32) {
      cin[a] = c[a];
      vin[a] = v[a];
    }
    __syncwarp();
    for (int a = lane; a < n; a += 32) {
      const int ca = cin[a];
      int r = 0;
      for (int b = 0; b < n; ++b) {
        const int cb = cin[b];
        r += (cb < ca || (cb == ca && b < a)) ? 1 : 0;
      }
      cs[r] = ca;
      vs[r] = vin[a];
    }
    __syncwarp();
    // groups of equal columns: the lane at a group's first entry sums it
    int base = 0;
    for (int a0 = 0; a0 < n; a0 += 32) {
      const int a = a0 + lane;
      const bool start = a < n && (a == 0 || cs[a] != cs[a - 1]);
      const unsigned bal = __ballot_sync(full, start);
      if (start) {
        const int m = base + __popc(bal & ((1u << lane) - 1u));
        double s = vs[a];
        for (int e = a + 1; e < n && cs[e] == cs[a]; ++e) s = __dadd_rn(s, vs[e]);
        c[m] = cs[a];
        v[m] = s;
      }
      base += __popc(bal);
    }
    if (lane == 0) mcnt[g] = base;
    __syncwarp();
  }
}

__global__ void __launch_bounds__(kT) k_2b_write(int64_t nrow, const int64_t* __restrict__ off,
                                                 const int64_t* __restrict__ moff, const int* __restrict__ mcnt,
                                                 const int* __restrict__ craw, const double* __restrict__ vraw,
                                                 int* __restrict__ col, double* __restrict__ val,
                                                 int* __restrict__ ptr) {
  for (int64_t g = blockIdx.x * (int64_t)kT + threadIdx.x; g < nrow; g += (int64_t)gridDim.x * kT) {
    const int64_t s = off[g], d = moff[g];
    for (int a = 0; a < mcnt[g]; ++a) {
      col[d + a] = craw[s + a];
      val[d + a] = vraw[s + a];
    }
    ptr[g] = (int)d;
    if (g == nrow - 1) ptr[nrow] = (int)(d + mcnt[g]);
  }
}

// ------------------------------------------------------------- pn tables
struct DLink {
  int b, s, dm, nA, nB, pad;
  int64_t nptr_off;
  int64_t row0;  // first (link, neutron SD) row
};

__device__ __forceinline__ int link_of_row(const DLink* __restrict__ L, int nl, int64_t t) {
  int lo = 0, hi = nl - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (L[mid].row0 <= t) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

// One-body jump of a species inside a link: forward links (source block
// after the output block) apply the operator itself, backward ones the
// transpose, keeping the sign of the forward jump (calc_1b_jumps!).
__device__ __forceinline__ bool pull1(bool fwd, uint64_t sd, uint64_t op_cr, uint64_t op_an, uint64_t& f, int& odd) {
  if (fwd) return sd_apply1(sd, op_cr, op_an, f, odd);
  uint64_t back;
  int dummy;
  if (!sd_apply1(sd, op_an, op_cr, f, dummy)) return false;
  return sd_apply1(f, op_cr, op_an, back, odd) && back == sd;
}

// neutron pull CSR: row (link, n) lists (n', ib, sign) for every neutron
// operator ib of the link's ΔM table that reaches n' in the source block.
template <bool FILL>
__global__ void __launch_bounds__(kT) k_npn(const DLink* __restrict__ links, int nl, int64_t nrows,
                                            const uint64_t* __restrict__ nbits, const int* __restrict__ nstart,
                                            const int* __restrict__ nn, const uint64_t* __restrict__ bops,
                                            const int64_t* __restrict__ boff, int* __restrict__ cnt,
                                            const int64_t* __restrict__ off, uint32_t* __restrict__ ent,
                                            int64_t* __restrict__ ptr, int* __restrict__ err) {
  for (int64_t t = blockIdx.x * (int64_t)kT + threadIdx.x; t < nrows; t += (int64_t)gridDim.x * kT) {
    const int li = link_of_row(links, nl, t);
    const DLink L = links[li];
    const int n = (int)(t - L.row0);
    const bool fwd = L.s >= L.b;
    const uint64_t* src = nbits + nstart[L.s];
    const int nsrc = nn[L.s];
    const uint64_t sd = nbits[nstart[L.b] + n];
    const uint64_t* ops = bops + 2 * boff[L.dm];
    int c = 0;
    int64_t w = FILL ? off[t] : 0;
    for (int ib = 0; ib < L.nB; ++ib) {
      uint64_t f;
      int odd;
      if (!pull1(fwd, sd, ops[2 * ib], ops[2 * ib + 1], f, odd)) continue;
      const int j = sd_find_desc(src, nsrc, f);
      if (j < 0) continue;
      if (FILL) {
        if (j >= (1 << 18)) atomicExch(err, 1);
        ent[w++] = ((uint32_t)j << 14) | ((uint32_t)ib << 1) | (uint32_t)odd;
      }
      ++c;
    }
    if (FILL) {
      ptr[L.nptr_off + n] = off[t];
      if (n == nn[L.b] - 1) ptr[L.nptr_off + n + 1] = off[t] + c;
    } else {
      cnt[t] = c;
    }
  }
}

// proton pull entries: row g lists (p', link, ia, sign) over the links of
// its block and the proton operators of each link's ΔM table.
template <bool FILL>
__global__ void __launch_bounds__(kT) k_ppn(const DLink* __restrict__ links, const int* __restrict__ link_begin,
                                            int64_t NP, const uint64_t* __restrict__ pbits,
                                            const int* __restrict__ pstart, int nb, const int* __restrict__ np,
                                            const uint64_t* __restrict__ aops, const int64_t* __restrict__ aoff,
                                            int* __restrict__ cnt, const int64_t* __restrict__ off,
                                            uint32_t* __restrict__ src_out, uint32_t* __restrict__ meta_out) {
  for (int64_t g = blockIdx.x * (int64_t)kT + threadIdx.x; g < NP; g += (int64_t)gridDim.x * kT) {
    const int b = block_of(pstart, nb, g);
    const uint64_t sd = pbits[g];
    int c = 0;
    int64_t w = FILL ? off[g] : 0;
    for (int li = link_begin[b]; li < link_begin[b + 1]; ++li) {
      const DLink L = links[li];
      const bool fwd = L.s >= L.b;
      const uint64_t* src = pbits + pstart[L.s];
      const int nsrc = np[L.s];
      const uint64_t* ops = aops + 2 * aoff[L.dm];
      for (int ia = 0; ia < L.nA; ++ia) {
        uint64_t f;
        int odd;
        if (!pull1(fwd, sd, ops[2 * ia], ops[2 * ia + 1], f, odd)) continue;
        const int j = sd_find_desc(src, nsrc, f);
        if (j < 0) continue;
        if (FILL) {
          src_out[w] = (uint32_t)j;
          meta_out[w] = ((uint32_t)li << 16) | ((uint32_t)ia << 1) | (uint32_t)odd;
          ++w;
        }
        ++c;
      }
    }
    if (!FILL) cnt[g] = c;
  }
}

template <class T>
void download(std::vector<T>& dst, const T* src, int64_t n, cudaStream_t st) {
  dst.resize((size_t)n);
  if (n > 0) SMGPU_CUDA_TRY(cudaMemcpyAsync(dst.data(), src, sizeof(T) * n, cudaMemcpyDeviceToHost, st));
}

// All SDs of one species grouped by M: grouped bits (lexicographic inside a
// bucket), bucket offsets and counts on the host.
struct Species {
  uint64_t* grouped = nullptr;
  int Mmin = 0, nbuck = 0;
  std::vector<int> count;
  std::vector<int64_t> offset;
};

Species enumerate_species(DeviceArena& A, const std::vector<MState>& ms, int k, cudaStream_t st) {
  Species S;
  const int L = (int)ms.size();
  std::vector<uint64_t> C((size_t)(L + 1) * (L + 1), 0);
  for (int n = 0; n <= L; ++n) {
    C[(size_t)n * (L + 1)] = 1;
    for (int j = 1; j <= n; ++j) C[(size_t)n * (L + 1) + j] = C[(size_t)(n - 1) * (L + 1) + j - 1] + (j <= n - 1 ? C[(size_t)(n - 1) * (L + 1) + j] : 0);
  }
  const uint64_t N = C[(size_t)L * (L + 1) + k];
  if (N > (1ull << 27)) throw SetupError{SMGPU_ERR_LIMIT, "more than 2^27 Slater determinants for one species"};
  std::vector<int> m2(L);
  for (int i = 0; i < L; ++i) m2[i] = ms[i].m2;
  std::vector<int> sorted = m2;
  std::sort(sorted.begin(), sorted.end());
  int Mmin = 0, Mmax = 0;
  for (int i = 0; i < k; ++i) {
    Mmin += sorted[i];
    Mmax += sorted[L - 1 - i];
  }
  S.Mmin = Mmin;
  S.nbuck = (Mmax - Mmin) / 2 + 1;
  uint64_t* d_C = A.upload(C);
  int* d_m2 = A.upload(m2);
  uint64_t* bits = A.alloc<uint64_t>(N);
  int* M = A.alloc<int>(N);
  int* cnt = A.alloc<int>(S.nbuck);
  int64_t* off = A.alloc<int64_t>(S.nbuck);
  S.grouped = A.alloc<uint64_t>(N);
  SMGPU_CUDA_TRY(cudaMemsetAsync(cnt, 0, sizeof(int) * S.nbuck, st));
  k_combos<<<grid_for((int64_t)N), kT, 0, st>>>(L, k, d_C, d_m2, (int64_t)N, bits, M);
  k_bucket_count<<<grid_for((int64_t)N), kT, 0, st>>>(M, (int64_t)N, Mmin, cnt);
  scan_exclusive<int>(A, cnt, S.nbuck, off, st);
  k_bucket_scatter<<<S.nbuck, kT, 0, st>>>(bits, M, (int64_t)N, Mmin, off, S.grouped);
  download(S.count, cnt, S.nbuck, st);
  download(S.offset, off, S.nbuck, st);
  SMGPU_CUDA_TRY(cudaStreamSynchronize(st));
  return S;
}

// pp or nn pull CSR of one species on the device, copied into ptr/col/val.
void build_2b_device(DeviceArena& A, const std::vector<Op2>& ops, const uint64_t* d_bits,
                     const std::vector<int>& start, int nb, std::vector<int>& ptr, std::vector<int>& col,
                     std::vector<double>& val, cudaStream_t st) {
  const int64_t nrow = start[nb];
  const std::vector<long> conj = conjugate_index(ops);
  const Op2* d_ops = A.upload(ops);
  const long* d_conj = A.upload(conj);
  const int* d_start = A.upload(start);
  int* cnt = A.alloc<int>(nrow);
  int64_t* off = A.alloc<int64_t>(nrow);
  const int nops = (int)ops.size();
  const int gw = (int)std::min<int64_t>((nrow + kT / 32 - 1) / (kT / 32), 65535);  // one warp per row
  k_2b_count<<<gw, kT, 0, st>>>(d_ops, nops, d_bits, d_start, nb, nrow, cnt);
  const int64_t raw = scan_exclusive<int>(A, cnt, nrow, off, st);
  int* craw = A.alloc<int>(raw);
  double* vraw = A.alloc<double>(raw);
  int* mcnt = A.alloc<int>(nrow);
  int64_t* moff = A.alloc<int64_t>(nrow);
  k_2b_fill<<<gw, kT, 0, st>>>(d_ops, d_conj, nops, d_bits, d_start, nb, nrow, off, craw, vraw);
  {
    SMGPU_CUDA_TRY(cudaFuncSetAttribute(k_2b_merge, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)merge_smem()));
    int64_t gm = (nrow + kMergeWarps - 1) / kMergeWarps;
    if (gm > 152 * 8) gm = 152 * 8;
    k_2b_merge<<<(int)(gm < 1 ? 1 : gm), kMergeWarps * 32, merge_smem(), st>>>(nrow, off, cnt, craw, vraw, mcnt);
  }
  const int64_t total = scan_exclusive<int>(A, mcnt, nrow, moff, st);
  if (total >= (1ll << 31)) throw SetupError{SMGPU_ERR_LIMIT, "two-body jump table too large"};
  int* d_col = A.alloc<int>(total);
  double* d_val = A.alloc<double>(total);
  int* d_ptr = A.alloc<int>(nrow + 1);
  k_2b_write<<<grid_for(nrow), kT, 0, st>>>(nrow, off, moff, mcnt, craw, vraw, d_col, d_val, d_ptr);
  download(ptr, d_ptr, nrow + 1, st);
  download(col, d_col, total, st);
  download(val, d_val, total, st);
  SMGPU_CUDA_TRY(cudaStreamSynchronize(st));
}
}  // namespace

void build_tables(const Interaction& I, int vp, int vn, int mtot2, Tables& T) {
  T = Tables();
  T.msp = mstates(I.porb);
  T.msn = mstates(I.norb);
  T.Lp = (int)T.msp.size();
  T.Ln = (int)T.msn.size();
  if (T.Lp > 63 || T.Ln > 63) throw SetupError{SMGPU_ERR_LIMIT, "more than 63 m-states per species"};
  if (vp < 0 || vn < 0 || vp > T.Lp || vn > T.Ln) throw SetupError{SMGPU_ERR_NUCLEUS, "invalid valence particle numbers"};
  cudaStream_t st = nullptr;
  SMGPU_CUDA_TRY(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
  DeviceArena A;
  try {
    // ---- basis (occ): SDs of both species, grouped by M on the device
    Species P = enumerate_species(A, T.msp, vp, st);
    Species N = enumerate_species(A, T.msn, vn, st);
    // blocks: ascending proton M, the partner neutron M = Mtot - Mp; the
    // reference's lists of all M values (Mps ascending, Mns descending)
    std::vector<int> Mps, Mns;
    for (int q = 0; q < P.nbuck; ++q)
      if (P.count[q] > 0) Mps.push_back(P.Mmin + 2 * q);
    for (int q = N.nbuck - 1; q >= 0; --q)
      if (N.count[q] > 0) Mns.push_back(N.Mmin + 2 * q);
    std::vector<int64_t> psrc, nsrc;  // bucket offsets of every block's lists
    T.tdims.push_back(0);
    T.off_pad.push_back(0);
    T.pstart.push_back(0);
    T.nstart.push_back(0);
    for (int Mp : Mps)
      for (int Mn : Mns) {
        if (Mp + Mn != mtot2) continue;
        const int qp = (Mp - P.Mmin) / 2, qn = (Mn - N.Mmin) / 2;
        const int np = P.count[qp], nn = N.count[qn];
        const int stride = (nn + 3) & ~3;
        psrc.push_back(P.offset[qp]);
        nsrc.push_back(N.offset[qn]);
        T.np.push_back(np);
        T.nn.push_back(nn);
        T.stride.push_back(stride);
        T.mp2.push_back(Mp);
        T.mn2.push_back(Mn);
        T.tdims.push_back(T.tdims.back() + (int64_t)np * nn);
        T.off_pad.push_back(T.off_pad.back() + (int64_t)np * stride);
        T.pstart.push_back(T.pstart.back() + np);
        T.nstart.push_back(T.nstart.back() + nn);
      }
    T.nb = (int)T.np.size();
    T.mdim = T.tdims.back();
    T.len_pad = T.off_pad.back();
    if (T.mdim == 0) {
      A.free_all();
      cudaStreamDestroy(st);
      return;
    }
    const int nb = T.nb;
    const int64_t NP = T.pstart[nb], NN = T.nstart[nb];
    uint64_t* d_pbits = A.alloc<uint64_t>(NP);
    uint64_t* d_nbits = A.alloc<uint64_t>(NN);
    for (int b = 0; b < nb; ++b) {
      SMGPU_CUDA_TRY(cudaMemcpyAsync(d_pbits + T.pstart[b], P.grouped + psrc[b], sizeof(uint64_t) * T.np[b],
                                     cudaMemcpyDeviceToDevice, st));
      SMGPU_CUDA_TRY(cudaMemcpyAsync(d_nbits + T.nstart[b], N.grouped + nsrc[b], sizeof(uint64_t) * T.nn[b],
                                     cudaMemcpyDeviceToDevice, st));
    }
    // ---- one-body diagonal
    {
      std::vector<uint64_t> pm(I.lp, 0), nm(I.ln, 0);
      for (int k = 0; k < T.Lp; ++k) pm[T.msp[k].orbit] |= sd_bit(T.Lp, k);
      for (int k = 0; k < T.Ln; ++k) nm[T.msn[k].orbit] |= sd_bit(T.Ln, k);
      double* d_ep = A.alloc<double>(NP);
      double* d_en = A.alloc<double>(NN);
      k_onebody<<<grid_for(NP), kT, 0, st>>>(d_pbits, NP, A.upload(pm), A.upload(I.spe_p), I.lp, d_ep);
      k_onebody<<<grid_for(NN), kT, 0, st>>>(d_nbits, NN, A.upload(nm), A.upload(I.spe_n), I.ln, d_en);
      download(T.ep, d_ep, NP, st);
      download(T.en, d_en, NN, st);
      download(T.pbits, d_pbits, NP, st);
      download(T.nbits, d_nbits, NN, st);
    }
    // ---- operator lists (host), pp / nn pull CSR (device)
    build_operators(I, T);
    build_2b_device(A, T.vpp, d_pbits, T.pstart, nb, T.pp_ptr, T.pp_col, T.pp_val, st);
    build_2b_device(A, T.vnn, d_nbits, T.nstart, nb, T.nn_ptr, T.nn_col, T.nn_val, st);
    // ---- links (host), pn pull tables (device)
    build_links(T, Mps);
    const int nl = (int)T.links.size();
    std::vector<int64_t> aoff(T.delMs.size() + 1, 0), boff(T.delMs.size() + 1, 0);
    std::vector<uint64_t> aops, bops;
    for (size_t k = 0; k < T.delMs.size(); ++k) {
      aops.insert(aops.end(), T.Aops_dm[k].begin(), T.Aops_dm[k].end());
      bops.insert(bops.end(), T.Bops_dm[k].begin(), T.Bops_dm[k].end());
      aoff[k + 1] = (int64_t)aops.size() / 2;
      boff[k + 1] = (int64_t)bops.size() / 2;
    }
    T.npn_ptr.assign(nl == 0 ? 0 : (size_t)(T.links.back().nptr_off + T.nn[T.links.back().b] + 1), 0);
    T.ppn_ptr.assign(NP + 1, 0);
    if (nl > 0) {
      std::vector<DLink> dl(nl);
      int64_t rows = 0;
      for (int li = 0; li < nl; ++li) {
        const auto& L = T.links[li];
        dl[li] = DLink{L.b, L.s, L.dm, L.nA, L.nB, 0, L.nptr_off, rows};
        rows += T.nn[L.b];
      }
      const DLink* d_links = A.upload(dl);
      const int* d_nstart = A.upload(T.nstart);
      const int* d_pstart = A.upload(T.pstart);
      const int* d_nn = A.upload(T.nn);
      const int* d_np = A.upload(T.np);
      const int* d_lb = A.upload(T.link_begin);
      const uint64_t* d_aops = A.upload(aops);
      const uint64_t* d_bops = A.upload(bops);
      const int64_t* d_aoff = A.upload(aoff);
      const int64_t* d_boff = A.upload(boff);
      int* d_err = A.alloc<int>(1);
      SMGPU_CUDA_TRY(cudaMemsetAsync(d_err, 0, sizeof(int), st));
      // neutron pull CSR
      int* ncnt = A.alloc<int>(rows);
      int64_t* noff = A.alloc<int64_t>(rows);
      k_npn<false><<<grid_for(rows), kT, 0, st>>>(d_links, nl, rows, d_nbits, d_nstart, d_nn, d_bops, d_boff, ncnt,
                                                  nullptr, nullptr, nullptr, nullptr);
      const int64_t nent = scan_exclusive<int>(A, ncnt, rows, noff, st);
      uint32_t* d_ent = A.alloc<uint32_t>(nent);
      int64_t* d_nptr = A.alloc<int64_t>(T.npn_ptr.size());
      k_npn<true><<<grid_for(rows), kT, 0, st>>>(d_links, nl, rows, d_nbits, d_nstart, d_nn, d_bops, d_boff, ncnt,
                                                 noff, d_ent, d_nptr, d_err);
      // proton pull entries
      int* pcnt = A.alloc<int>(NP);
      int64_t* poff = A.alloc<int64_t>(NP);
      k_ppn<false><<<grid_for(NP), kT, 0, st>>>(d_links, d_lb, NP, d_pbits, d_pstart, nb, d_np, d_aops, d_aoff,
                                                pcnt, nullptr, nullptr, nullptr);
      const int64_t pent = scan_exclusive<int>(A, pcnt, NP, poff, st);
      if (pent >= (1ll << 31)) throw SetupError{SMGPU_ERR_LIMIT, "proton pull table too large"};
      uint32_t* d_psrc = A.alloc<uint32_t>(pent);
      uint32_t* d_pmeta = A.alloc<uint32_t>(pent);
      k_ppn<true><<<grid_for(NP), kT, 0, st>>>(d_links, d_lb, NP, d_pbits, d_pstart, nb, d_np, d_aops, d_aoff, pcnt,
                                               poff, d_psrc, d_pmeta);
      int err = 0;
      std::vector<int64_t> po;
      download(T.npn_ptr, d_nptr, (int64_t)T.npn_ptr.size(), st);
      download(T.npn_ent, d_ent, nent, st);
      download(po, poff, NP, st);
      download(T.ppn_src, d_psrc, pent, st);
      download(T.ppn_meta, d_pmeta, pent, st);
      SMGPU_CUDA_TRY(cudaMemcpyAsync(&err, d_err, sizeof(int), cudaMemcpyDeviceToHost, st));
      SMGPU_CUDA_TRY(cudaStreamSynchronize(st));
      if (err) throw SetupError{SMGPU_ERR_LIMIT, "neutron block too large"};
      for (int64_t g = 0; g < NP; ++g) T.ppn_ptr[g] = (int)po[g];
      T.ppn_ptr[NP] = (int)pent;
    }
    SMGPU_CUDA_TRY(cudaStreamSynchronize(st));
    SMGPU_CUDA_TRY(cudaGetLastError());
    count_updates(T);
  } catch (...) {
    cudaStreamSynchronize(st);
    A.free_all();
    cudaStreamDestroy(st);
    throw;
  }
  A.free_all();
  cudaStreamDestroy(st);
}

}  // namespace smgpu
