// Slater-determinant bit operations shared by the host set-up (setup.cpp)
// and the device-side enumeration (enum.cu).  An SD is a bit string over
// the m-states of one species; m-state k (0-based, construct_msps order) is
// bit L-1-k, so m-state 1 of the reference is the most significant bit
// (bitarr_to_int, src/ShellModel/shellmodel_main.jl:732-739).
#pragma once
#include <cstdint>

#ifdef __CUDACC__
#define SMGPU_HD __host__ __device__ __forceinline__
#else
#define SMGPU_HD inline
#endif

namespace smgpu {

SMGPU_HD int sd_popc(uint64_t x) {
#ifdef __CUDA_ARCH__
  return __popcll(x);
#else
  return __builtin_popcountll(x);
#endif
}

SMGPU_HD uint64_t sd_bit(int L, int k0) { return 1ull << (L - 1 - k0); }

// ⟨f|a†c|i⟩ for one-hot masks a (create) and c (annihilate).  Returns false
// when not connectable.  `odd` = parity of the fermion sign count: occupied
// states at or above c in i, then at or above a after removing c
// (calc_phase_1!, shellmodel_main.jl:887-897, without its constant offset,
// which cancels between the proton and neutron factors).
SMGPU_HD bool sd_apply1(uint64_t i, uint64_t a, uint64_t c, uint64_t& f, int& odd) {
  if ((i & c) == 0) return false;
  const uint64_t r = i & ~c;
  if (r & a) return false;
  const int cnt = sd_popc(i & ~(c - 1)) + sd_popc(r & ~(a - 1));
  f = r | a;
  odd = cnt & 1;
  return true;
}

// ⟨f|a†b†dc|i⟩ (TF_connectable + calc_phase!, shellmodel_main.jl:850-885).
SMGPU_HD bool sd_apply2(uint64_t i, uint64_t a, uint64_t b, uint64_t c, uint64_t d, uint64_t& f, int& odd) {
  if ((i & c) != c || (i & d) != d) return false;
  const uint64_t r = i & ~c & ~d;
  if ((r & a) || (r & b)) return false;
  int cnt = sd_popc(i & ~(c - 1));
  uint64_t x = i & ~c;
  cnt += sd_popc(x & ~(d - 1));
  x &= ~d;
  cnt += sd_popc(x & ~(b - 1));
  x |= b;
  cnt += sd_popc(x & ~(a - 1));
  f = x | a;
  odd = cnt & 1;
  return true;
}

// Index of `x` in a descending list, or -1 (bisearch!, :1068-1083).
SMGPU_HD int sd_find_desc(const uint64_t* v, int n, uint64_t x) {
  int lo = 0, hi = n - 1;
  while (lo <= hi) {
    const int mid = (lo + hi) >> 1;
    if (v[mid] > x) lo = mid + 1;
    else if (v[mid] < x) hi = mid - 1;
    else return mid;
  }
  return -1;
}

}  // namespace smgpu
