// Device helpers shared by the single-vector (lanczos.cu) and the
// multi-sample (multi_lanczos.cu) Lanczos kernels.
#pragma once
#include <cfloat>
#include <cstdint>

#include "device.cuh"

namespace smgpu {
namespace dev {

constexpr int kNT = 256;  // threads of the streaming kernels

// (volatile: the persistent batch kernel reads flags that other CTAs of the
// same launch set, so they must come from L2, not from a line in L1)
__device__ __forceinline__ bool stopped(const LanczosFlags* fl) {
  return *(volatile const int*)&fl->done || *(volatile const int*)&fl->exhausted;
}

__device__ __forceinline__ double warp_sum(double x) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
  return x;
}

// Deterministic block sum, result returned to every thread.  The warps'
// sums are added by one thread and broadcast: on this GPU FP64 adds are
// scarce, and letting every thread add them up costs NT/32 times as many.
template <int NT>
__device__ __forceinline__ double block_sum_all(double x, double* red) {
  __shared__ double s_bcast;
  x = warp_sum(x);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) red[wid] = x;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
#pragma unroll
    for (int k = 0; k < NT / 32; ++k) s += red[k];
    s_bcast = s;
  }
  __syncthreads();
  return s_bcast;
}

// Eight deterministic block sums at once (a[q] per thread, q < 8); the sum of
// value q is returned in thread q, other threads get an unspecified value.
// The warp stage is a reduce-scatter: each of three halving exchanges keeps
// half of the values, so a lane does 9 FP64 adds for all eight sums instead
// of 40 (5 per value), then lane l holds the warp's sum of value l >> 2.
// red: (NT/32) x 8 doubles of shared memory.
template <int NT>
__device__ __forceinline__ double block_sum8(const double (&a)[8], double* red) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const bool b4 = lane & 16, b3 = lane & 8, b2 = lane & 4;
  double h[4];
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const double keep = b4 ? a[4 + q] : a[q];
    const double give = b4 ? a[q] : a[4 + q];
    h[q] = keep + __shfl_xor_sync(0xffffffffu, give, 16);
  }
  double g[2];
#pragma unroll
  for (int q = 0; q < 2; ++q) {
    const double keep = b3 ? h[2 + q] : h[q];
    const double give = b3 ? h[q] : h[2 + q];
    g[q] = keep + __shfl_xor_sync(0xffffffffu, give, 8);
  }
  double u = (b2 ? g[1] : g[0]) + __shfl_xor_sync(0xffffffffu, b2 ? g[0] : g[1], 4);
  u += __shfl_xor_sync(0xffffffffu, u, 2);
  u += __shfl_xor_sync(0xffffffffu, u, 1);
  __syncthreads();
  if ((lane & 3) == 0) red[wid * 8 + (lane >> 2)] = u;
  __syncthreads();
  double s = 0.0;
  if (threadIdx.x < 8) {
#pragma unroll
    for (int k = 0; k < NT / 32; ++k) s += red[k * 8 + threadIdx.x];
  }
  return s;
}

// Sum of n partials in a fixed order (every thread gets the same value).
template <int NT>
__device__ __forceinline__ double sum_partials(const double* __restrict__ p, int n, double* red) {
  double x = 0.0;
  for (int i = threadIdx.x; i < n; i += NT) x += p[i];
  return block_sum_all<NT>(x, red);
}

// m sums of G partials each, one warp per sum; results into smem out[0..m).
template <int NT>
__device__ __forceinline__ void sum_partials_many(const double* __restrict__ p, int G, int m, double* out) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  for (int j = wid; j < m; j += NT / 32) {
    double x = 0.0;
    for (int g = lane; g < G; g += 32) x += p[(int64_t)j * G + g];
    x = warp_sum(x);
    if (lane == 0) out[j] = x;
  }
  __syncthreads();
}

__device__ __forceinline__ void chunk_of(int64_t len, int G, int64_t& b, int64_t& e) {
  int64_t per = (len + G - 1) / G;
  per = (per + 31) & ~(int64_t)31;
  b = (int64_t)blockIdx.x * per;
  e = b + per;
  if (e > len) e = len;
  if (b > len) b = len;
}

__device__ __forceinline__ int find_block(const int64_t* off, int nb, int64_t i) {
  int lo = 0, hi = nb - 1;
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if (off[mid] <= i) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

// Four consecutive elements (16-byte aligned: vector lengths and chunk starts
// are multiples of 4) widened to FP64.
__device__ __forceinline__ void load4(const float* p, double (&o)[4]) {
  const float4 f = *reinterpret_cast<const float4*>(p);
  o[0] = widen(f.x);
  o[1] = widen(f.y);
  o[2] = widen(f.z);
  o[3] = widen(f.w);
}
__device__ __forceinline__ void load4(const double* p, double (&o)[4]) {
  const double2 a = *reinterpret_cast<const double2*>(p);
  const double2 b = *reinterpret_cast<const double2*>(p + 2);
  o[0] = a.x;
  o[1] = a.y;
  o[2] = b.x;
  o[3] = b.y;
}
__device__ __forceinline__ void store4(double* p, const double (&o)[4]) {
  *reinterpret_cast<double2*>(p) = make_double2(o[0], o[1]);
  *reinterpret_cast<double2*>(p + 2) = make_double2(o[2], o[3]);
}

// Kahan-compensated FP32 sum.
struct KahanF {
  float s, c;
  __device__ __forceinline__ void init() { s = 0.f; c = 0.f; }
  __device__ __forceinline__ void add(float x) {
    float y = __fsub_rn(x, c);
    float t = __fadd_rn(s, y);
    c = __fsub_rn(__fsub_rn(t, s), y);
    s = t;
  }
  // += a·b, the product rounded once inside the compensated step
  __device__ __forceinline__ void add_prod(float a, float b) {
    const float y = __fmaf_rn(a, b, -c);
    const float t = __fadd_rn(s, y);
    c = __fsub_rn(__fsub_rn(t, s), y);
    s = t;
  }
  __device__ __forceinline__ float get() const { return __fsub_rn(s, c); }
};

// Seeded start vector (replaces Random.seed!(1234); randn(mdim),
// shellmodel_main.jl:939-948): v[M] = u0+u1+u2+u3-2 with
// u_k = (splitmix64(seed + φ·(4M+k+1)) >> 11)·2^-53.  Integer and exactly
// rounded double operations only, so host and device agree bit for bit.
__device__ __forceinline__ double start_elem(uint64_t seed, int64_t i) {
  double u[4];
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    uint64_t z = seed + 0x9E3779B97F4A7C15ull * (uint64_t)(4 * i + k + 1);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z = z ^ (z >> 31);
    u[k] = (double)(z >> 11) * 0x1.0p-53;
  }
  return __dsub_rn(__dadd_rn(__dadd_rn(u[0], u[1]), __dadd_rn(u[2], u[3])), 2.0);
}

// ---------------------------------------------------------------------------
// Lowest eigenvalues of the k x k Lanczos matrix by Sturm counts
// (diagonalize_T!, lanczos_methods.jl:250-258).  After a thick restart T is
// an arrowhead (rows 0..lock-1 diagonal, coupled to row `lock`) followed by a
// tridiagonal tail; the LDLᵀ inertia of T - σI is evaluated in O(k) for that
// shape.  A group of kLPE lanes bisects one eigenvalue with kLPE trial shifts
// per step (FP64 division throughput, not latency, bounds this kernel).
constexpr int kLPE = 4;

__device__ inline int sturm_count(const double* a, const double* c2, const double* b2, int lock, int k, double sigma,
                           double pivmin) {
  int cnt = 0;
  double acc = 0.0;
  for (int i = 0; i < lock; ++i) {
    double d = a[i] - sigma;
    if (fabs(d) < pivmin) d = -pivmin;
    if (d < 0.0) ++cnt;
    acc += c2[i] / d;
  }
  double d = (a[lock] - sigma) - acc;
  if (fabs(d) < pivmin) d = -pivmin;
  if (d < 0.0) ++cnt;
  for (int i = lock + 1; i < k; ++i) {
    d = (a[i] - sigma) - b2[i - 1] / d;
    if (fabs(d) < pivmin) d = -pivmin;
    if (d < 0.0) ++cnt;
  }
  return cnt;
}

// Eigenvalue update of one Lanczos matrix (T[k-1][k-1] already holds α):
// lowest num_ev eigenvalues of T[0:k,0:k] by Sturm bisection, the 3-deep
// history `en` and the convergence test.  One CTA; dynamic shared memory
// 3*lm + num_ev doubles.
__device__ inline void sturm_step(double* __restrict__ T, int lm, int k, int lock, int num_ev, double* en, int nh,
                                  double tol, int64_t mdim, LanczosFlags* fl) {
  extern __shared__ double sm[];
  double* a = sm;            // k
  double* c2 = a + lm;       // lock
  double* b2 = c2 + lm;      // k-1
  double* lam = b2 + lm;     // num_ev
  __shared__ double s_lo, s_hi, s_piv;
  const int tid = threadIdx.x;
  for (int i = tid; i < k; i += blockDim.x) {
    a[i] = T[(int64_t)i * lm + i];
    if (i < lock) { double x = T[(int64_t)i * lm + lock]; c2[i] = x * x; }
    if (i >= lock && i + 1 < k) { double x = T[(int64_t)i * lm + i + 1]; b2[i] = x * x; }
  }
  __syncthreads();
  if (tid == 0) {
    // Gershgorin interval and pivot floor
    double lo = INFINITY, hi = -INFINITY, mx = 1.0;
    for (int i = 0; i < k; ++i) {
      double r = 0.0;
      if (i < lock) r = sqrt(c2[i]);
      else {
        if (i == lock) for (int j = 0; j < lock; ++j) r += sqrt(c2[j]);
        if (i > lock) r += sqrt(b2[i - 1]);
        if (i + 1 < k) r += sqrt(b2[i]);
      }
      lo = fmin(lo, a[i] - r);
      hi = fmax(hi, a[i] + r);
    }
    for (int i = 0; i < lock; ++i) mx = fmax(mx, c2[i]);
    for (int i = lock; i + 1 < k; ++i) mx = fmax(mx, b2[i]);
    double w = hi - lo;
    s_lo = lo - 1e-3 * w - 1e-300;
    s_hi = hi + 1e-3 * w + 1e-300;
    s_piv = DBL_MIN * mx;
  }
  __syncthreads();
  const int n = min(num_ev, k);
  const int lane = tid & 31;
  const int grp = tid / kLPE, sub = tid % kLPE, ngrp = blockDim.x / kLPE;
  const unsigned gmask = ((1u << kLPE) - 1u) << (lane & ~(kLPE - 1));
  for (int e0 = 0; e0 < n; e0 += ngrp) {
    const int e = e0 + grp;
    const bool live = e < n;
    double lo = s_lo, hi = s_hi;
    // Warm start.  T_k grows from T_{k-1} by a row and a column (and after a
    // restart its leading block holds the kept Ritz values, the previous
    // test's eigenvalues), so by Cauchy interlacing λ_e(T_k) <= λ_e(T_{k-1})
    // = en[e]; the new eigenvalue is expected within a few times its last
    // change below that.  The bracket [l, h] around that guess is taken only
    // when two Sturm counts (two lanes of the group, in parallel) confirm it
    // holds λ_e: count(l) <= e < count(h); otherwise the Gershgorin bracket
    // stays.  The bisection then runs to the same final width as before.
    {
      const double prev = live ? en[e] : 0.0, prev2 = live ? en[num_ev + e] : 0.0;
      const bool warm = live && prev < hi && prev > lo;
      const double h = prev + 8.0 * DBL_EPSILON * fabs(prev) + 1e-300;
      const double l = h - fmax(4.0 * fabs(prev2 - prev), 64.0 * DBL_EPSILON * fabs(prev) + 1e-300);
      int cnt = -1;
      if (warm && l > lo && h < hi && sub < 2) cnt = sturm_count(a, c2, b2, lock, k, sub == 0 ? l : h, s_piv);
      const int base = lane & ~(kLPE - 1);
      const int cl = __shfl_sync(0xffffffffu, cnt, base), ch = __shfl_sync(0xffffffffu, cnt, base + 1);
      if (warm && cl >= 0 && ch >= 0 && cl <= e && ch >= e + 1) {
        lo = l;
        hi = h;
      }
    }
    for (int step = 0; step < 200; ++step) {
      const double sigma = lo + (hi - lo) * (double)(sub + 1) * (1.0 / (kLPE + 1));
      const int cnt = live ? sturm_count(a, c2, b2, lock, k, sigma, s_piv) : 0;
      const unsigned le = __ballot_sync(0xffffffffu, cnt <= e) & gmask;
      const unsigned ge = __ballot_sync(0xffffffffu, cnt >= e + 1) & gmask;
      const double s_le = __shfl_sync(0xffffffffu, sigma, le ? 31 - __clz(le) : lane);
      const double s_ge = __shfl_sync(0xffffffffu, sigma, ge ? __ffs(ge) - 1 : lane);
      if (le) lo = s_le;
      if (ge) hi = s_ge;
      const bool fin = !live || (hi - lo <= 4.0 * DBL_EPSILON * fmax(fabs(lo), fabs(hi)) + 1e-300);
      if (__all_sync(0xffffffffu, fin)) break;
    }
    if (live && sub == 0) lam[e] = 0.5 * (lo + hi);
  }
  __syncthreads();
  if (tid == 0) {
    for (int hh = nh - 1; hh >= 1; --hh)
      for (int j = 0; j < num_ev; ++j) en[hh * num_ev + j] = en[(hh - 1) * num_ev + j];
    for (int j = 0; j < n; ++j) en[j] = lam[j];
    bool conv = true;
    for (int j = 0; j < num_ev; ++j)
      if (!(en[num_ev + j] - en[j] < tol)) conv = false;
    if (conv || (int64_t)k == mdim || (fl->exhausted && k == fl->exh_k)) {
      fl->done = 1;
      fl->elit = k;
    }
  }
}

// Symmetric eigen-decomposition of T[0:n,0:n] by parallel cyclic Jacobi
// (round-robin pairing, n/2 disjoint rotations per round) in one CTA.
// Output: evals ascending, A = eigenvectors (column-major, ld n).  Dynamic
// shared memory: see the launchers.
// Matrices up to this order are rotated in shared memory by jacobi_eig.
constexpr int kJacobiSmemN = 48;
// Dynamic shared memory of jacobi_eig for order n.
__host__ __device__ inline size_t jacobi_smem_bytes(int n) {
  const int N = n + (n & 1);
  size_t b = sizeof(double) * (N / 2) * 2 + sizeof(double) * N + sizeof(int) * (N / 2) * 2 + 16;
  if (n <= kJacobiSmemN) b += 2 * sizeof(double) * (size_t)n * n;
  return b;
}

template <int NT>
__device__ inline void jacobi_eig(const double* __restrict__ T, int ldt, int n, double* A, double* Z,
                                  double* evals) {
  __shared__ double red[NT / 32];
  __shared__ int s_stop;
  extern __shared__ double shj[];
  const int N = n + (n & 1);
  const int npair = N / 2;
  // small matrices rotate in shared memory, larger ones in the global A / Z
  const bool in_smem = n <= kJacobiSmemN;
  double* A_ = in_smem ? shj : A;
  double* Z_ = in_smem ? shj + n * n : Z;
  double* cc = shj + (in_smem ? 2 * n * n : 0);
  double* ss = cc + npair;
  double* dg = ss + npair;
  int* pp = (int*)(dg + N);
  int* qq = pp + npair;
  const int tid = threadIdx.x;
  for (int idx = tid; idx < n * n; idx += NT) {
    int i = idx % n, j = idx / n;
    A_[idx] = T[(int64_t)j * ldt + i];
    Z_[idx] = (i == j) ? 1.0 : 0.0;
  }
  __syncthreads();
  double fro = 0.0;
  for (int idx = tid; idx < n * n; idx += NT) fro += A_[idx] * A_[idx];
  fro = block_sum_all<NT>(fro, red);
  for (int sweep = 0; sweep < 64; ++sweep) {
    double off = 0.0;
    for (int idx = tid; idx < n * n; idx += NT) {
      int i = idx % n, j = idx / n;
      if (i < j) off += A_[idx] * A_[idx];
    }
    off = block_sum_all<NT>(off, red);
    if (tid == 0) s_stop = (off <= 1e-34 * fro || off == 0.0) ? 1 : 0;
    __syncthreads();
    if (s_stop) break;
    for (int r = 0; r < N - 1; ++r) {
      for (int k = tid; k < npair; k += NT) {
        int p, q;
        if (k == 0) { p = N - 1; q = r; }
        else { p = (r + k) % (N - 1); q = (r - k + (N - 1)) % (N - 1); }
        if (p > q) { int x = p; p = q; q = x; }
        double c = 1.0, s = 0.0;
        if (q < n) {
          double apq = A_[(int64_t)q * n + p];
          if (apq != 0.0) {
            double app = A_[(int64_t)p * n + p], aqq = A_[(int64_t)q * n + q];
            double theta = (aqq - app) / (2.0 * apq);
            double t = (fabs(theta) > 1e150) ? 0.5 / theta
                                              : (theta >= 0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(1.0 + theta * theta));
            c = 1.0 / sqrt(1.0 + t * t);
            s = t * c;
          }
        }
        pp[k] = p; qq[k] = q; cc[k] = c; ss[k] = s;
      }
      __syncthreads();
      // the rotations applied to A's columns p, q and, independently, to Z
      for (int idx = tid; idx < 2 * npair * n; idx += NT) {
        const bool onz = idx >= npair * n;
        double* M = onz ? Z_ : A_;
        const int id2 = onz ? idx - npair * n : idx;
        int k = id2 / n, i = id2 % n;
        if (ss[k] == 0.0) continue;
        int p = pp[k], q = qq[k];
        double c = cc[k], s = ss[k];
        double aip = M[(int64_t)p * n + i], aiq = M[(int64_t)q * n + i];
        M[(int64_t)p * n + i] = c * aip - s * aiq;
        M[(int64_t)q * n + i] = s * aip + c * aiq;
      }
      __syncthreads();
      // then to A's rows p, q; the pair's own off-diagonal entries, which
      // the rotation annihilates, are written as exact zeros
      for (int idx = tid; idx < npair * n; idx += NT) {
        int k = idx / n, j = idx % n;
        if (ss[k] == 0.0) continue;
        int p = pp[k], q = qq[k];
        double c = cc[k], s = ss[k];
        double apj = A_[(int64_t)j * n + p], aqj = A_[(int64_t)j * n + q];
        A_[(int64_t)j * n + p] = (j == q) ? 0.0 : c * apj - s * aqj;
        A_[(int64_t)j * n + q] = (j == p) ? 0.0 : s * apj + c * aqj;
      }
      __syncthreads();
    }
  }
  for (int i = tid; i < n; i += NT) dg[i] = A_[(int64_t)i * n + i];
  __syncthreads();
  for (int i = tid; i < n; i += NT) {
    double d = dg[i];
    int rank = 0;
    for (int j = 0; j < n; ++j)
      if (dg[j] < d || (dg[j] == d && j < i)) ++rank;
    evals[rank] = d;
    for (int r = 0; r < n; ++r) A[(int64_t)rank * n + r] = Z_[(int64_t)i * n + r];
  }
}

// ---------------------------------------------------------------------------
// FP64 Jacobi preconditioned by an FP32 one (the FP32-mixed solve's restart
// and Ritz eigenproblems, order n <= kJacobiRefineN).  One SM's FP64 pipe runs
// a from-scratch FP64 Jacobi of order ~30 for most of a millisecond on this
// GPU; most of that goes into the early sweeps, whose rotations an FP32
// Jacobi does on the FP32 pipe.  So:
//   1. FP32 Jacobi sweeps on T give an approximate eigenbasis Z0 (~1e-6);
//   2. Q = Z0 made orthonormal in FP64 by two Newton-Schulz steps
//      Q <- Q (3I - QᵀQ) / 2 (orthonormal to FP64 rounding);
//   3. A1 = Qᵀ T Q in FP64 — an FP64 similarity transform of T, nearly
//      diagonal;
//   4. FP64 Jacobi sweeps on A1 (a pair is rotated while
//      a_pq² > 1e-34 ||A1||_F², as jacobi_eig's stopping test);
//   5. eigenvectors Q Z1 in FP64, eigenvalues diag(A1) ascending.
// The result is an FP64 Jacobi eigendecomposition of T.
constexpr int kJacobiRefineN = 32;
__host__ __device__ inline size_t jacobi_refined_smem_bytes(int n) {
  const int N = n + (n & 1);
  return sizeof(double) * (4 * (size_t)n * n + N + N) + sizeof(float) * (2 * (size_t)n * n + N) +
         sizeof(int) * (size_t)N + 64;
}

// Parallel cyclic Jacobi sweeps (round-robin pairing, n/2 disjoint rotations
// per round) on the symmetric matrix A_ (n x n, column-major, shared memory),
// accumulating the rotations into Z_.  A pair is rotated while a_pq² > thr;
// the sweeps stop when a sweep starts with no such pair, or after maxsweep.
template <int NT, class R>
__device__ void jacobi_sweeps(R* A_, R* Z_, int n, R thr, int maxsweep, R* cc, R* ss, int* pp, int* qq) {
  const int N = n + (n & 1);
  const int npair = N / 2;
  const int tid = threadIdx.x;
  for (int sweep = 0; sweep < maxsweep; ++sweep) {
    int above = 0;
    for (int idx = tid; idx < n * n; idx += NT) {
      const int i = idx % n, j = idx / n;
      const R a = A_[idx];
      if (i < j && a * a > thr) above = 1;
    }
    if (!__syncthreads_or(above)) break;
    for (int r = 0; r < N - 1; ++r) {
      for (int k = tid; k < npair; k += NT) {
        int p, q;
        if (k == 0) { p = N - 1; q = r; }
        else { p = (r + k) % (N - 1); q = (r - k + (N - 1)) % (N - 1); }
        if (p > q) { const int x = p; p = q; q = x; }
        R c = R(1), sn = R(0);
        if (q < n) {
          const R apq = A_[(int64_t)q * n + p];
          if (apq * apq > thr) {
            const R app = A_[(int64_t)p * n + p], aqq = A_[(int64_t)q * n + q];
            const R theta = (aqq - app) / (R(2) * apq);
            const R t = (fabs(theta) > R(1e18)) ? R(0.5) / theta
                                                 : (theta >= R(0) ? R(1) : R(-1)) / (fabs(theta) + sqrt(R(1) + theta * theta));
            c = R(1) / sqrt(R(1) + t * t);
            sn = t * c;
          }
        }
        pp[k] = p; qq[k] = q; cc[k] = c; ss[k] = sn;
      }
      __syncthreads();
      // the rotations applied to A's columns p, q and, independently, to Z
      for (int idx = tid; idx < 2 * npair * n; idx += NT) {
        const bool onz = idx >= npair * n;
        const int id2 = onz ? idx - npair * n : idx;
        const int k = id2 / n, i = id2 % n;
        const R sk = ss[k];
        if (sk == R(0)) continue;
        const int p = pp[k], q = qq[k];
        const R ck = cc[k];
        R* M = onz ? Z_ : A_;
        const R aip = M[(int64_t)p * n + i], aiq = M[(int64_t)q * n + i];
        M[(int64_t)p * n + i] = ck * aip - sk * aiq;
        M[(int64_t)q * n + i] = sk * aip + ck * aiq;
      }
      __syncthreads();
      // then to A's rows p, q; the pair's own off-diagonal entries, which
      // the rotation annihilates, are written as exact zeros
      for (int idx = tid; idx < npair * n; idx += NT) {
        const int k = idx / n, j = idx % n;
        const R sk = ss[k];
        if (sk == R(0)) continue;
        const int p = pp[k], q = qq[k];
        const R ck = cc[k];
        const R apj = A_[(int64_t)j * n + p], aqj = A_[(int64_t)j * n + q];
        A_[(int64_t)j * n + p] = (j == q) ? R(0) : ck * apj - sk * aqj;
        A_[(int64_t)j * n + q] = (j == p) ? R(0) : sk * apj + ck * aqj;
      }
      __syncthreads();
    }
  }
}

// out = op(X) Y for n x n column-major matrices in shared memory, FP64;
// op(X) = Xᵀ when tx.  out must not alias X or Y.
template <int NT>
__device__ void small_matmul(const double* X, bool tx, const double* Y, double* out, int n) {
  for (int idx = threadIdx.x; idx < n * n; idx += NT) {
    const int i = idx % n, j = idx / n;
    double acc = 0.0;
    for (int k = 0; k < n; ++k) acc = fma(tx ? X[(int64_t)i * n + k] : X[(int64_t)k * n + i], Y[(int64_t)j * n + k], acc);
    out[idx] = acc;
  }
  __syncthreads();
}

template <int NT>
__device__ void jacobi_eig_refined(const double* __restrict__ T, int ldt, int n, double* A_out, double* evals) {
  __shared__ double red[NT / 32];
  extern __shared__ double shj[];
  const int N = n + (n & 1);
  const int npair = N / 2;
  const int nn = n * n;
  double* Ad = shj;           // T, then Qᵀ T Q
  double* Q = Ad + nn;
  double* W = Q + nn;
  double* Zd = W + nn;
  double* ccd = Zd + nn;
  double* ssd = ccd + npair;
  double* dg = ssd + npair;
  float* Af = reinterpret_cast<float*>(dg + N);
  float* Zf = Af + nn;
  float* ccf = Zf + nn;
  float* ssf = ccf + npair;
  int* pp = reinterpret_cast<int*>(ssf + npair);
  int* qq = pp + npair;
  const int tid = threadIdx.x;
  // 1. FP32 Jacobi on T
  float frf = 0.f;
  for (int idx = tid; idx < nn; idx += NT) {
    const int i = idx % n, j = idx / n;
    const double x = T[(int64_t)j * ldt + i];
    Ad[idx] = x;
    Af[idx] = (float)x;
    Zf[idx] = (i == j) ? 1.f : 0.f;
    frf += (float)x * (float)x;
  }
  frf = (float)block_sum_all<NT>((double)frf, red);  // also the barrier after the loads
  jacobi_sweeps<NT, float>(Af, Zf, n, 1e-12f * frf, 12, ccf, ssf, pp, qq);
  // 2. Q = Z0 made orthonormal in FP64 (Newton-Schulz, twice)
  for (int idx = tid; idx < nn; idx += NT) Q[idx] = (double)Zf[idx];
  __syncthreads();
  for (int it = 0; it < 2; ++it) {
    small_matmul<NT>(Q, true, Q, W, n);  // W = QᵀQ
    for (int idx = tid; idx < nn; idx += NT) {
      const int i = idx % n, j = idx / n;
      W[idx] = 0.5 * ((i == j ? 3.0 : 0.0) - W[idx]);
    }
    __syncthreads();
    small_matmul<NT>(Q, false, W, Zd, n);  // Zd = Q (3I - QᵀQ)/2
    for (int idx = tid; idx < nn; idx += NT) Q[idx] = Zd[idx];
    __syncthreads();
  }
  // 3. A1 = Qᵀ T Q, symmetrised
  small_matmul<NT>(Ad, false, Q, W, n);  // W = T Q
  small_matmul<NT>(Q, true, W, Zd, n);   // Zd = Qᵀ T Q
  double fro = 0.0;
  for (int idx = tid; idx < nn; idx += NT) {
    const int i = idx % n, j = idx / n;
    const double a = 0.5 * (Zd[idx] + Zd[(int64_t)i * n + j]);
    Ad[idx] = a;
    fro += a * a;
  }
  fro = block_sum_all<NT>(fro, red);
  for (int idx = tid; idx < nn; idx += NT) Zd[idx] = (idx % n == idx / n) ? 1.0 : 0.0;
  __syncthreads();
  // 4. FP64 Jacobi sweeps
  jacobi_sweeps<NT, double>(Ad, Zd, n, 1e-34 * fro, 64, ccd, ssd, pp, qq);
  // 5. eigenvectors Q Z1, eigenvalues ascending
  small_matmul<NT>(Q, false, Zd, W, n);
  for (int i = tid; i < n; i += NT) dg[i] = Ad[(int64_t)i * n + i];
  __syncthreads();
  for (int i = tid; i < n; i += NT) {
    const double d = dg[i];
    int rank = 0;
    for (int j = 0; j < n; ++j)
      if (dg[j] < d || (dg[j] == d && j < i)) ++rank;
    evals[rank] = d;
    for (int r = 0; r < n; ++r) A_out[(int64_t)rank * n + r] = W[(int64_t)i * n + r];
  }
}

template <int NT>
__device__ __forceinline__ float2 block_sum_df2(float h, float l, float2* red);

// (h, l) = (ah + al)(bh + bl) in double-float.
__device__ __forceinline__ void df_mul(float ah, float al, float bh, float bl, float& h, float& l) {
  const float p = __fmul_rn(ah, bh);
  float e = __fmaf_rn(ah, bh, -p);
  e = __fmaf_rn(ah, bl, __fmaf_rn(al, bh, e));
  fast_two_sum(p, e, h, l);
}

// jacobi_eig in double-float arithmetic on the FP32 pipe (about 2^-47
// relative), for the FP32-mixed solvers: GB300's FP64 pipe makes the FP64
// rotations of jacobi_eig latency-bound.  Matrices of order n <= kJacobiSmemN
// only (callers fall back to jacobi_eig above that); same shared memory as
// jacobi_eig.  The rotation angle of a pair is taken in FP32 from the leading
// parts; (c, s) are then made orthonormal to double-float precision
// (c = (1 + t²)^(-1/2) by one Newton step, s = t c), and the rotated entries
// are computed rather than set to zero, so an inexact angle costs convergence,
// never orthogonality.  A pair is rotated while a_pq² > 1e-28 ||A||_F²; the
// sweeps stop when no pair is above that.
template <int NT>
__device__ inline void jacobi_eig_df(const double* __restrict__ T, int ldt, int n, double* A, double* evals) {
  __shared__ double red[NT / 32];
  extern __shared__ double shj[];
  const int N = n + (n & 1);
  const int npair = N / 2;
  float2* A_ = reinterpret_cast<float2*>(shj);
  float2* Z_ = A_ + n * n;
  float2* cc = Z_ + n * n;
  float2* ss = cc + npair;
  double* dg = reinterpret_cast<double*>(ss + npair);
  int* pp = (int*)(dg + N);
  int* qq = pp + npair;
  const int tid = threadIdx.x;
  for (int idx = tid; idx < n * n; idx += NT) {
    const int i = idx % n, j = idx / n;
    float h, l;
    df_from_double(T[(int64_t)j * ldt + i], h, l);
    A_[idx] = make_float2(h, l);
    Z_[idx] = make_float2(i == j ? 1.f : 0.f, 0.f);
  }
  __syncthreads();
  // the Frobenius norm² in double-float and the per-sweep test by a barrier
  // vote: no FP64 reduction (slow on this GPU) in the sweep loop
  float fh = 0.f, fl = 0.f;
  for (int idx = tid; idx < n * n; idx += NT) {
    const float h = A_[idx].x;
    const float p = __fmul_rn(h, h);
    df_add(fh, fl, p, __fmaf_rn(h, h, -p));
  }
  const float2 fro2 = block_sum_df2<NT>(fh, fl, reinterpret_cast<float2*>(red));
  const float thr = 1e-28f * fro2.x;
  for (int sweep = 0; sweep < 64; ++sweep) {
    int above = 0;
    for (int idx = tid; idx < n * n; idx += NT) {
      const int i = idx % n, j = idx / n;
      const float a = A_[idx].x;
      if (i < j && a * a > thr) above = 1;
    }
    if (!__syncthreads_or(above)) break;
  for (int r = 0; r < N - 1; ++r) {
      for (int k = tid; k < npair; k += NT) {
        int p, q;
        if (k == 0) { p = N - 1; q = r; }
        else { p = (r + k) % (N - 1); q = (r - k + (N - 1)) % (N - 1); }
        if (p > q) { int x = p; p = q; q = x; }
        float2 c = make_float2(1.f, 0.f), sn = make_float2(0.f, 0.f);
        if (q < n) {
          const float2 apq = A_[(int64_t)q * n + p];
          if (apq.x * apq.x > thr) {
            const float2 app = A_[(int64_t)p * n + p], aqq = A_[(int64_t)q * n + q];
            float dh = aqq.x, dl = aqq.y;
            df_add(dh, dl, -app.x, -app.y);
            const float theta = dh / (2.f * apq.x);
            const float t = (fabsf(theta) > 1e18f) ? 0.5f / theta
                                                    : copysignf(1.f, theta) / (fabsf(theta) + sqrtf(1.f + theta * theta));
            // r = 1 + t² (double-float), c = r^(-1/2) by one Newton step from rsqrtf
            float rh, rl;
            {
              const float t2 = __fmul_rn(t, t), e = __fmaf_rn(t, t, -t2);
              float s0, e0;
              two_sum(1.f, t2, s0, e0);
              fast_two_sum(s0, __fadd_rn(e0, e), rh, rl);
            }
            const float y = rsqrtf(rh);
            float zh, zl;
            {
              const float y2 = __fmul_rn(y, y), ye = __fmaf_rn(y, y, -y2);
              df_mul(rh, rl, y2, ye, zh, zl);
            }
            float oh = 1.f, ol = 0.f;
            df_add(oh, ol, -zh, -zl);  // 1 - r y² (small)
            float ch, cl;
            fast_two_sum(y, __fmul_rn(0.5f * y, oh), ch, cl);
            c = make_float2(ch, cl);
            float sh, sl;
            df_mul(t, 0.f, ch, cl, sh, sl);
            sn = make_float2(sh, sl);
          }
        }
        pp[k] = p; qq[k] = q; cc[k] = c; ss[k] = sn;
      }
      __syncthreads();
      // rows p, q of A together with those of Z (independent), then the
      // columns of A; x' = c x - s y, y' = s x + c y
      for (int pass = 0; pass < 2; ++pass) {
        const int nwork = (pass == 0 ? 2 : 1) * npair * n;
        for (int idx = tid; idx < nwork; idx += NT) {
          const bool onz = idx >= npair * n;
          float2* M = onz ? Z_ : A_;
          const int id2 = onz ? idx - npair * n : idx;
          const int k = id2 / n, i = id2 % n;
          const float2 sk = ss[k];
          if (sk.x == 0.f && sk.y == 0.f) continue;
          const float2 ck = cc[k];
          const int p = pp[k], q = qq[k];
          const int64_t ip = pass == 1 ? (int64_t)i * n + p : (int64_t)p * n + i;
          const int64_t iq = pass == 1 ? (int64_t)i * n + q : (int64_t)q * n + i;
          const float2 x = M[ip], yv = M[iq];
          float a1h, a1l, a2h, a2l, b1h, b1l, b2h, b2l;
          df_mul(ck.x, ck.y, x.x, x.y, a1h, a1l);
          df_mul(sk.x, sk.y, yv.x, yv.y, a2h, a2l);
          df_mul(sk.x, sk.y, x.x, x.y, b1h, b1l);
          df_mul(ck.x, ck.y, yv.x, yv.y, b2h, b2l);
          df_add(a1h, a1l, -a2h, -a2l);
          df_add(b1h, b1l, b2h, b2l);
          M[ip] = make_float2(a1h, a1l);
          M[iq] = make_float2(b1h, b1l);
        }
        __syncthreads();
      }
    }
  }
  for (int i = tid; i < n; i += NT) dg[i] = (double)A_[(int64_t)i * n + i].x + (double)A_[(int64_t)i * n + i].y;
  __syncthreads();
  for (int i = tid; i < n; i += NT) {
    const double d = dg[i];
    int rank = 0;
    for (int j = 0; j < n; ++j)
      if (dg[j] < d || (dg[j] == d && j < i)) ++rank;
    evals[rank] = d;
    for (int r = 0; r < n; ++r) {
      const float2 z = Z_[(int64_t)i * n + r];
      A[(int64_t)rank * n + r] = (double)z.x + (double)z.y;
    }
  }
}

// Double-float accumulator: exact FP32 products (two-product by FMA) summed
// with TwoSum into an unevaluated (hi, lo) pair — about 2^-48 relative, on
// the FP32 pipe.  Used for the restart Gram matrix of FP32-stored vectors.
struct DFAcc {
  float hi, lo;
  __device__ __forceinline__ void init() { hi = 0.f; lo = 0.f; }
  __device__ __forceinline__ void add_prod(float a, float b) {
    const float p = __fmul_rn(a, b);
    const float e = __fmaf_rn(a, b, -p);
    const float s = __fadd_rn(hi, p);
    const float bb = __fsub_rn(s, hi);
    const float err = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bb)), __fsub_rn(p, bb));
    hi = s;
    lo = __fadd_rn(lo, __fadd_rn(err, e));
  }
  // += a·(bh + bl): a·bh exactly (two-product), a·bl rounded — the product
  // of an FP32 value with a double-float pair.
  __device__ __forceinline__ void add_prod2(float a, float bh, float bl) {
    const float p = __fmul_rn(a, bh);
    const float e = __fmaf_rn(a, bh, -p);
    const float s = __fadd_rn(hi, p);
    const float bb = __fsub_rn(s, hi);
    const float err = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bb)), __fsub_rn(p, bb));
    hi = s;
    lo = __fadd_rn(lo, __fadd_rn(err, __fmaf_rn(a, bl, e)));
  }
  __device__ __forceinline__ double get() const { return (double)hi + (double)lo; }
};

// Sums of NQ double-float accumulators over a CTA, all on the FP32 pipe
// (warp shuffles and the sum of the warp totals in double-float; on GB300
// even a handful of dependent FP64 adds per CTA costs microseconds).  Thread
// q < NQ gets value q as an unevaluated (hi, lo) pair in *out; red holds
// (NT/32)*NQ doubles of shared memory (used as float2).
template <int NT, int NQ>
__device__ __forceinline__ void block_sum_df(DFAcc (&acc)[NQ], double* red, float2& out) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  float2* r2 = reinterpret_cast<float2*>(red);
#pragma unroll
  for (int q = 0; q < NQ; ++q) {
    float h = acc[q].hi, l = acc[q].lo;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const float oh = __shfl_xor_sync(0xffffffffu, h, o);
      const float ol = __shfl_xor_sync(0xffffffffu, l, o);
      df_add(h, l, oh, ol);
    }
    acc[q].hi = h;
    acc[q].lo = l;
  }
  __syncthreads();
  if (lane == 0) {
#pragma unroll
    for (int q = 0; q < NQ; ++q) r2[wid * NQ + q] = make_float2(acc[q].hi, acc[q].lo);
  }
  __syncthreads();
  out = make_float2(0.f, 0.f);
  if (threadIdx.x < NQ) {
    float h = 0.f, l = 0.f;
    for (int k = 0; k < NT / 32; ++k) {
      const float2 x = r2[k * NQ + threadIdx.x];
      df_add(h, l, x.x, x.y);
    }
    out = make_float2(h, l);
  }
}

// Double-float sum over a CTA on the FP32 pipe; every thread gets the same
// (hi, lo).  red: NT/32 float2 of shared memory.
template <int NT>
__device__ __forceinline__ float2 block_sum_df2(float h, float l, float2* red) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const float oh = __shfl_xor_sync(0xffffffffu, h, o);
    const float ol = __shfl_xor_sync(0xffffffffu, l, o);
    df_add(h, l, oh, ol);
  }
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) red[wid] = make_float2(h, l);
  __syncthreads();
  float sh = red[0].x, sl = red[0].y;
#pragma unroll
  for (int k = 1; k < NT / 32; ++k) df_add(sh, sl, red[k].x, red[k].y);
  return make_float2(sh, sl);
}

// Sum of n double-float partials (float2 pairs) in a fixed order, every
// thread gets the same value.
template <int NT>
__device__ __forceinline__ float2 sum_partials_df(const float2* __restrict__ p, int n, float2* red) {
  float h = 0.f, l = 0.f;
#pragma unroll 4
  for (int i = threadIdx.x; i < n; i += NT) {
    const float2 x = p[i];
    df_add(h, l, x.x, x.y);
  }
  return block_sum_df2<NT>(h, l, red);
}

// Sum of n FP64 partials reduced in double-float on the FP32 pipe (each
// partial split once); the double result in every thread.  red: NT/32 doubles.
template <int NT>
__device__ __forceinline__ double sum_partials_d2(const double* __restrict__ p, int n, double* red) {
  float h = 0.f, l = 0.f;
#pragma unroll 4
  for (int i = threadIdx.x; i < n; i += NT) {
    float xh, xl;
    df_from_double(p[i], xh, xl);
    df_add(h, l, xh, xl);
  }
  const float2 s = block_sum_df2<NT>(h, l, reinterpret_cast<float2*>(red));
  return (double)s.x + (double)s.y;
}

// Block sum of one FP64 value per thread, reduced in double-float (FP32
// pipe); the double result in every thread.  red: NT/32 doubles.
template <int NT>
__device__ __forceinline__ double block_sum_d2(double x, double* red) {
  float h, l;
  df_from_double(x, h, l);
  const float2 s = block_sum_df2<NT>(h, l, reinterpret_cast<float2*>(red));
  return (double)s.x + (double)s.y;
}

// m sums of G double-float partials each (one warp per sum), results as
// (hi, lo) into shared hh[j], hl[j].
template <int NT>
__device__ __forceinline__ void sum_partials_many_df(const float2* __restrict__ p, int G, int m, float* hh,
                                                     float* hl) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  for (int j = wid; j < m; j += NT / 32) {
    float h = 0.f, l = 0.f;
#pragma unroll 4
    for (int g = lane; g < G; g += 32) {
      const float2 x = p[(int64_t)j * G + g];
      df_add(h, l, x.x, x.y);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const float oh = __shfl_xor_sync(0xffffffffu, h, o);
      const float ol = __shfl_xor_sync(0xffffffffu, l, o);
      df_add(h, l, oh, ol);
    }
    if (lane == 0) {
      hh[j] = h;
      hl[j] = l;
    }
  }
  __syncthreads();
}

// Double-float scalar arithmetic for one warp's small dense algebra
// (division and square root: an FP32 estimate and one Newton correction).
__device__ __forceinline__ float2 dfw_sub(float2 a, float2 b) {
  df_add(a.x, a.y, -b.x, -b.y);
  return a;
}
__device__ __forceinline__ float2 dfw_mul(float2 a, float2 b) {
  float h, l;
  df_mul(a.x, a.y, b.x, b.y, h, l);
  return make_float2(h, l);
}
__device__ __forceinline__ float2 dfw_div(float2 a, float2 b) {
  const float q1 = __fdiv_rn(a.x, b.x);
  const float2 r = dfw_sub(a, dfw_mul(make_float2(q1, 0.f), b));
  const float q2 = __fdiv_rn(r.x, b.x);
  float h, l;
  fast_two_sum(q1, q2, h, l);
  return make_float2(h, l);
}
__device__ __forceinline__ float2 dfw_sqrt(float2 a) {
  const float s = __fsqrt_rn(a.x);
  const float2 r = dfw_sub(a, dfw_mul(make_float2(s, 0.f), make_float2(s, 0.f)));
  float h, l;
  fast_two_sum(s, __fdiv_rn(r.x, 2.f * s), h, l);
  return make_float2(h, l);
}

// ThickRestart's Cholesky G = RᵀR, X = R⁻¹ and c = Xᵀ g in double-float
// arithmetic on one warp (the FP32 pipe; a single-thread FP64 form is
// latency-bound on GB300's FP64 unit).  gram(idx) reads the packed upper
// triangle (row by row) followed by g; putX(j, i, x) stores X(i, j)
// (zero below the diagonal); putc(k, c).  Right-looking factorisation with
// the lanes over the columns of the trailing update, the inverse by back
// substitution one column per lane.  ls <= 32.  Returns true (in every lane)
// when a pivot was not positive.
template <class GF, class XF, class CF>
__device__ inline bool chol_df_warp(int ls, GF gram, XF putX, CF putc) {
  __shared__ float2 A[32 * 32];   // A[j*32 + i]: the Gram matrix (upper), then R(i,j) in place
  __shared__ float2 Xs[32 * 32];
  const int lane = threadIdx.x & 31;
  int bad = 0;
  for (int k = 0, off = 0; k < ls; off += ls - k, ++k)
    for (int l = k + lane; l < ls; l += 32) {
      float h, lo;
      df_from_double(gram(off + (l - k)), h, lo);
      A[l * 32 + k] = make_float2(h, lo);
    }
  __syncwarp();
  for (int k = 0; k < ls; ++k) {
    float2 d = A[k * 32 + k];
    if (!(d.x > 0.f)) {
      bad = 1;
      d = make_float2(1e-30f, 0.f);
    }
    const float2 rkk = dfw_sqrt(d);
    __syncwarp();
    if (lane == 0) A[k * 32 + k] = rkk;
    for (int j = k + 1 + lane; j < ls; j += 32) A[j * 32 + k] = dfw_div(A[j * 32 + k], rkk);
    __syncwarp();
    for (int j = k + 1 + lane; j < ls; j += 32) {
      const float2 rkj = A[j * 32 + k];
      for (int i = k + 1; i <= j; ++i) A[j * 32 + i] = dfw_sub(A[j * 32 + i], dfw_mul(A[i * 32 + k], rkj));
    }
    __syncwarp();
  }
  for (int j = lane; j < ls; j += 32) {
    for (int i = ls - 1; i >= 0; --i) {
      float2 sacc = make_float2(0.f, 0.f);
      if (i <= j) {
        sacc.x = i == j ? 1.f : 0.f;
        for (int k = i + 1; k <= j; ++k) sacc = dfw_sub(sacc, dfw_mul(A[k * 32 + i], Xs[j * 32 + k]));
        sacc = dfw_div(sacc, A[i * 32 + i]);
      }
      Xs[j * 32 + i] = sacc;
    }
  }
  __syncwarp();
  for (int idx = lane; idx < ls * ls; idx += 32) {
    const int j = idx / ls, i = idx % ls;
    putX(j, i, (double)Xs[j * 32 + i].x + (double)Xs[j * 32 + i].y);
  }
  const int gofs = ls * (ls + 1) / 2;
  for (int k = lane; k < ls; k += 32) {
    float2 sacc = make_float2(0.f, 0.f);
    for (int j = 0; j <= k; ++j) {
      float gh, gl;
      df_from_double(gram(gofs + j), gh, gl);
      const float2 p = dfw_mul(Xs[k * 32 + j], make_float2(gh, gl));
      df_add(sacc.x, sacc.y, p.x, p.y);
    }
    putc(k, (double)sacc.x + (double)sacc.y);
  }
  __syncwarp();
  return bad != 0;
}

// x = hi + lo with hi = x rounded to FP32 and lo the FP32 rounding of the rest.
__device__ __forceinline__ void df_split(double x, float& hi, float& lo) {
  hi = __double2float_rn(x);
  lo = __double2float_rn(x - (double)hi);
}

__device__ __forceinline__ void gram_pair(int pr, int ls, int& k, int& l) {
  if (pr < ls * (ls + 1) / 2) {
    k = 0;
    int rem = pr;
    while (rem >= ls - k) { rem -= ls - k; ++k; }
    l = k + rem;
  } else {
    k = pr - ls * (ls + 1) / 2;
    l = ls;  // v_last
  }
}

}  // namespace dev
}  // namespace smgpu
