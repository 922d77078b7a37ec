// The row body of the staged FP32-mixed H·v (hv_staged.cu), shared by the
// single-problem kernel and the batched kernel (hv_batch.cu).  See
// hv_staged.cu for the algorithm.
#pragma once
#include "device.cuh"
#include "hv_tile.cuh"

namespace smgpu {

// The rows p0 .. p0+R-1 of block b (one CTA): w = H v on those rows with the
// tables of `a` (its vector fields are not read; the vectors are the explicit
// arguments).  vprev: three-term correction w -= beta*vprev (null: none);
// alpha_out: where the CTA's partial of v·Hv goes (null: none; DF: a (hi, lo)
// float pair in the FP64 slot).  DF: the epilogue writes w as (a.wh, a.wl).
// EXT: the pp and nn sums of every element come from the two-body pass
// (hv_2b.cu, in a.tt.s2b) instead of being computed here.
template <int NT, int R, int QM, bool DF, bool EXT = false>
__device__ __forceinline__ void hv_staged_rows(const HvArgs<float, float>& a, const float* __restrict__ v_in,
                                               double* w_out, const float* vprev, const double beta, const int b,
                                               const int p0, double* alpha_out) {
  const DevTables& t = a.t;
  const TileTables& tt = a.tt;
  extern __shared__ float4 sm4[];
  float* Y = reinterpret_cast<float*>(sm4);          // [R][ymax] slots
  float* A = Y + R * tt.ymax;                        // [R][nbmax][astride] coefficients
  float* vrow = A + R * tt.nbmax * tt.astride;       // [R][nnmax] the CTA's rows of v (not with EXT)
  int* so = reinterpret_cast<int*>(vrow + (EXT ? 0 : R * tt.nnmax));  // [R][kpad] source-row offsets into v
  const int tid = threadIdx.x;
  const int np = t.np[b];
  const int nr = min(R, np - p0);
  const int nn = t.nn[b];
  const int stride = t.stride[b];
  const int64_t blk = t.off_pad[b];
  const int pst = t.pstart[b], nst = t.nstart[b];
  const int lb = tt.link_begin[b];
  const int nl = tt.link_begin[b + 1] - lb;
  const int64_t rlb = tt.rl_base[b] + (int64_t)p0 * (nl + 1);
  const float* __restrict__ v = v_in;
  const int as = tt.astride, kpad = tt.kpad;

  if constexpr (!EXT) {
    for (int idx = tid; idx < nr * nn; idx += NT) {
      const int r = idx / nn, n = idx - r * nn;
      vrow[r * tt.nnmax + n] = v[blk + (int64_t)(p0 + r) * stride + n];
    }
  }

  AccKahan pn[R][QM];
#pragma unroll
  for (int r = 0; r < R; ++r)
#pragma unroll
    for (int q = 0; q < QM; ++q) pn[r][q].init();

  for (int j = 0; j < nl; ++j) {
    const int L = lb + j;
    int kr[R];
    int eb[R];
    int kmx = 0;
#pragma unroll
    for (int r = 0; r < R; ++r) {
      kr[r] = 0;
      eb[r] = 0;
      if (r < nr) {
        eb[r] = tt.rl[rlb + (int64_t)r * (nl + 1) + j];
        kr[r] = tt.rl[rlb + (int64_t)r * (nl + 1) + j + 1] - eb[r];
      }
      kmx = max(kmx, kr[r]);
    }
    if (kmx == 0) continue;  // no proton entry of these rows uses the link (uniform over the CTA)
    const int4 la = t.link_a[L];
    const int s = la.x, nB = la.y;
    const float* __restrict__ vt = a.c.vtab + t.link_v[L];  // V; the negated copy is not used here
    const int kp = (kmx + 3) & ~3;
    const int64_t soff = t.off_pad[s];
    const int sstride = t.stride[s];
    const int nns = t.nn[s];
    // coefficient matrices A_r[ib][j] = ±V[ia_j][ib] (zero-padded to kp) and source offsets
#pragma unroll
    for (int r = 0; r < R; ++r) {
      if (r >= nr || kr[r] == 0) continue;
      float* Ar = A + r * tt.nbmax * as;
      // one thread per row ib: the proton entries' metadata are uniform
      // (broadcast) loads, V[ia][ib] coalesced over ib, and the row goes out
      // as 16-byte stores (row stride = 4 mod 8 floats: no bank conflicts)
      for (int ib = tid; ib < nB; ib += NT) {
        float4* row = reinterpret_cast<float4*>(Ar + ib * as);
        for (int j4 = 0; j4 < kp; j4 += 4) {
          float x4[4];
#pragma unroll
          for (int u = 0; u < 4; ++u) {
            const int jj = j4 + u;
            float val = 0.f;
            if (jj < kr[r]) {
              const uint32_t meta = t.ppn_meta[eb[r] + jj];
              val = vt[(int)((meta >> 1) & 0x7fffu) * nB + ib];
              if (meta & 1u) val = -val;
            }
            x4[u] = val;
          }
          row[j4 >> 2] = make_float4(x4[0], x4[1], x4[2], x4[3]);
        }
      }
      for (int jj = tid; jj < kr[r]; jj += NT) so[r * kpad + jj] = (int)(soff + (int64_t)t.ppn_src[eb[r] + jj] * sstride);
    }
    __syncthreads();
    // stage 1: one thread per source column, columns in descending order of
    // list length; the entry loop stops at the warp's longest list
    const uint32_t* __restrict__ pell = tt.push_ent + tt.push_off[L];
    const int* __restrict__ pinfo = tt.push_info + tt.push_ioff[L];
    for (int i0 = 0; i0 < nns; i0 += NT) {
      // every lane of the warp runs this loop body (the warp reductions need them all)
      const int i = i0 + tid;
      const bool act = i < nns;
      const int info = act ? pinfo[i] : 0;
      const int n = info & 0xffff, cnt = info >> 16;
      for (int ec = 0;; ec += 16) {
        const int ne = max(0, min(16, cnt - ec));
        const int kw = (int)__reduce_max_sync(0xffffffffu, (unsigned)ne);
        if (kw == 0) break;
        // the lane's entries, in groups of four up to the warp's longest list
        uint32_t ent[16];
#pragma unroll
        for (int k0 = 0; k0 < 16; k0 += 4) {
#pragma unroll
          for (int u = 0; u < 4; ++u) ent[k0 + u] = 0u;
          if (k0 >= kw) continue;
#pragma unroll
          for (int u = 0; u < 4; ++u)
            if (k0 + u < ne) ent[k0 + u] = pell[(int64_t)(ec + k0 + u) * nns + i];
        }
#pragma unroll
        for (int r = 0; r < R; ++r) {
          if (r >= nr || kr[r] == 0) continue;
          const float* Ar = A + r * tt.nbmax * as;
          const int* sor = so + r * kpad;
          float* Yr = Y + r * tt.ymax;
          // proton entries in blocks of 16: v[s,p'_j,n'] of the block in registers
          for (int j0 = 0; j0 < kr[r]; j0 += 16) {
            const int kq = min(16, kr[r] - j0);
            // kq is uniform over the CTA: groups of four past it are skipped
            float x[16];
#pragma unroll
            for (int jc = 0; jc < 16; jc += 4) {
#pragma unroll
              for (int u = 0; u < 4; ++u) x[jc + u] = 0.f;
              if (jc >= kq) continue;
#pragma unroll
              for (int u = 0; u < 4; ++u)
                if (jc + u < kq) x[jc + u] = v[sor[j0 + jc + u] + n];
            }
            // four entries at a time, branch-free inside a group (entries past
            // the lane's list read row 0 of A and are not stored)
#pragma unroll
            for (int k0 = 0; k0 < 16; k0 += 4) {
              if (k0 >= kw) break;
              const float* a0 = Ar + (int)((ent[k0] >> 16) & 0x7fffu) * as + j0;
              const float* a1 = Ar + (int)((ent[k0 + 1] >> 16) & 0x7fffu) * as + j0;
              const float* a2 = Ar + (int)((ent[k0 + 2] >> 16) & 0x7fffu) * as + j0;
              const float* a3 = Ar + (int)((ent[k0 + 3] >> 16) & 0x7fffu) * as + j0;
              float y0 = 0.f, y1 = 0.f, y2 = 0.f, y3 = 0.f;
#pragma unroll
              for (int jc = 0; jc < 16; jc += 4) {
                if (jc >= kq) break;
                const float4 b0 = *reinterpret_cast<const float4*>(a0 + jc);
                const float4 b1 = *reinterpret_cast<const float4*>(a1 + jc);
                const float4 b2 = *reinterpret_cast<const float4*>(a2 + jc);
                const float4 b3 = *reinterpret_cast<const float4*>(a3 + jc);
                y0 = __fmaf_rn(b0.w, x[jc + 3], __fmaf_rn(b0.z, x[jc + 2], __fmaf_rn(b0.y, x[jc + 1], __fmaf_rn(b0.x, x[jc], y0))));
                y1 = __fmaf_rn(b1.w, x[jc + 3], __fmaf_rn(b1.z, x[jc + 2], __fmaf_rn(b1.y, x[jc + 1], __fmaf_rn(b1.x, x[jc], y1))));
                y2 = __fmaf_rn(b2.w, x[jc + 3], __fmaf_rn(b2.z, x[jc + 2], __fmaf_rn(b2.y, x[jc + 1], __fmaf_rn(b2.x, x[jc], y2))));
                y3 = __fmaf_rn(b3.w, x[jc + 3], __fmaf_rn(b3.z, x[jc + 2], __fmaf_rn(b3.y, x[jc + 1], __fmaf_rn(b3.x, x[jc], y3))));
              }
              const float yv[4] = {y0, y1, y2, y3};
#pragma unroll
              for (int u = 0; u < 4; ++u) {
                const uint32_t e = ent[k0 + u];
                const float y = (e >> 31) ? -yv[u] : yv[u];
                if (k0 + u < ne) {
                  const uint32_t slot = e & 0xffffu;
                  Yr[slot] = (j0 == 0) ? y : __fadd_rn(Yr[slot], y);
                }
              }
            }
          }
        }
      }
    }
    __syncthreads();
    // stage 2: one thread per output column; slots [t][n]
    const int64_t* __restrict__ nptr = tt.npn_ptr + t.link_n[L];
#pragma unroll
    for (int q = 0; q < QM; ++q) {
      const int n = tid + q * NT;
      if (n < nn) {
        const int K = (int)(nptr[n + 1] - nptr[n]);
#pragma unroll
        for (int r = 0; r < R; ++r) {
          if (r >= nr || kr[r] == 0) continue;
          const float* Yr = Y + r * tt.ymax + n;
          float sacc = 0.f;
#pragma unroll 4
          for (int k = 0; k < K; ++k) sacc = __fadd_rn(sacc, Yr[k * nn]);
          pn[r][q].add(sacc);
        }
      }
    }
  }
  __syncthreads();  // vrow complete (also when the block has no links)

  double apart = 0.0;
  float ah = 0.f, al = 0.f;  // DF: α partial
  float bh = 0.f, bl = 0.f;  // DF: β
  if constexpr (DF) df_from_double(beta, bh, bl);
  // pp and nn of all the thread's columns, entry-outer so that every entry
  // issues one independent load per column (memory-level parallelism);
  // FP32 partial sums, one compensated add per (row, column) each
  float sp[R][QM], sn[R][QM];
#pragma unroll
  for (int r = 0; r < R; ++r)
#pragma unroll
    for (int q = 0; q < QM; ++q) {
      sp[r][q] = 0.f;
      sn[r][q] = 0.f;
    }
  if constexpr (EXT) {
    // the two-body pass has left them in s2b
#pragma unroll
    for (int r = 0; r < R; ++r) {
      if (r >= nr) break;
#pragma unroll
      for (int q = 0; q < QM; ++q)
        if (tid + q * NT < nn) {
          const int64_t o = blk + (int64_t)(p0 + r) * stride + tid + q * NT;
          sp[r][q] = tt.s2b[o];
          sn[r][q] = tt.s2b[t.len_pad + o];
        }
    }
  }
  // pp: other proton rows of the block, same neutron column (coalesced)
#pragma unroll
  for (int r = 0; r < R; ++r) {
    if (EXT || r >= nr) break;
    const int g = pst + p0 + r;
    const int kb = t.pp_ptr[g], ke = t.pp_ptr[g + 1];
#pragma unroll 8
    for (int k = kb; k < ke; ++k) {
      const float pv = a.c.pp_val[k];
      const float* __restrict__ src = v + blk + (int64_t)t.pp_col[k] * stride + tid;
#pragma unroll
      for (int q = 0; q < QM; ++q)
        if (tid + q * NT < nn) sp[r][q] = __fmaf_rn(pv, src[q * NT], sp[r][q]);
    }
  }
  // nn: same proton row, other neutron columns (ELL lists [k][n], rows of v
  // in shared memory)
  if constexpr (!EXT) {
    const int W = tt.nnell_w[b];
    const int* __restrict__ ecol = tt.nnell_col + tt.nnell_off[b] + tid;
    const float* __restrict__ eval = tt.nnell_val + tt.nnell_off[b] + tid;
#pragma unroll 8
    for (int k = 0; k < W; ++k) {
#pragma unroll
      for (int q = 0; q < QM; ++q) {
        if (tid + q * NT < nn) {
          const int c = ecol[(int64_t)k * nn + q * NT];
          const float cv = eval[(int64_t)k * nn + q * NT];
#pragma unroll
          for (int r = 0; r < R; ++r)
            if (r < nr) sn[r][q] = __fmaf_rn(cv, vrow[r * tt.nnmax + c], sn[r][q]);
        }
      }
    }
  }
#pragma unroll
  for (int q = 0; q < QM; ++q) {
    const int n = tid + q * NT;
    if (n >= nn) continue;
    AccKahan acc[R];
#pragma unroll
    for (int r = 0; r < R; ++r) {
      acc[r] = pn[r][q];
      acc[r].add(sn[r][q]);
      acc[r].add(sp[r][q]);
    }
    // one-body term, Lanczos epilogue, store
    if constexpr (DF) {
      const float2 en2 = a.en2[nst + n];
#pragma unroll
      for (int r = 0; r < R; ++r) {
        if (r >= nr) break;
        const int64_t o = blk + (int64_t)(p0 + r) * stride + n;
        const float x = EXT ? v[o] : vrow[r * tt.nnmax + n];
        float hh, hl;
        fast_two_sum(acc[r].s, -acc[r].c, hh, hl);
        const float2 ep2 = a.ep2[pst + p0 + r];
        float dh = ep2.x, dl = ep2.y;
        df_add(dh, dl, en2.x, en2.y);
        df_fma(hh, hl, x, dh, dl);
        {
          const float p = __fmul_rn(x, hh);
          const float pe = __fmaf_rn(x, hh, -p);
          float s2, e2;
          two_sum(ah, p, s2, e2);
          ah = s2;
          al = __fadd_rn(al, __fadd_rn(e2, __fmaf_rn(x, hl, pe)));
        }
        if (vprev != nullptr) df_fma(hh, hl, vprev[o], -bh, -bl);
        a.wh[o] = hh;
        a.wl[o] = hl;
      }
    } else {
      const double enn = a.en[nst + n];
#pragma unroll
      for (int r = 0; r < R; ++r) {
        if (r >= nr) break;
        const int64_t o = blk + (int64_t)(p0 + r) * stride + n;
        const double x = widen(EXT ? v[o] : vrow[r * tt.nnmax + n]);
        double hv = fma(a.ep[pst + p0 + r] + enn, x, acc[r].result());
        apart = fma(x, hv, apart);
        if (vprev != nullptr) hv = fma(-beta, widen(vprev[o]), hv);
        w_out[o] = hv;
      }
    }
  }
  if (alpha_out != nullptr) {
    __shared__ double red[NT / 32];
    if constexpr (DF) {
      // double-float all the way; the partial is stored as a (hi, lo) pair
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        const float oh = __shfl_down_sync(0xffffffffu, ah, o);
        const float ol = __shfl_down_sync(0xffffffffu, al, o);
        df_add(ah, al, oh, ol);
      }
      float2* r2 = reinterpret_cast<float2*>(red);
      if ((tid & 31) == 0) r2[tid >> 5] = make_float2(ah, al);
      __syncthreads();
      if (tid == 0) {
        float h = r2[0].x, l = r2[0].y;
        for (int k = 1; k < NT / 32; ++k) df_add(h, l, r2[k].x, r2[k].y);
        *reinterpret_cast<float2*>(alpha_out) = make_float2(h, l);
      }
      return;
    } else {
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) apart += __shfl_down_sync(0xffffffffu, apart, o);
    }
    if ((tid & 31) == 0) red[tid >> 5] = apart;
    __syncthreads();
    if (tid == 0) {
      double s2 = 0.0;
      for (int k = 0; k < NT / 32; ++k) s2 += red[k];
      *alpha_out = s2;
    }
  }
}

}  // namespace smgpu
