// Column-block k-pair contraction (layout in dmd_layout.h).
//
// One warp per work item: a run of row blocks of one column block J. Lane s owns column
// c = 32 J + s: it keeps rt_c and st_c in registers and accumulates the reverse (k' side) sums
//   X_c[a] += sum_b conj(P2[a][b]) rt_k[b],   Y_c[b] += sum_a st_k[a] conj(P1[a][b])
// across all row blocks of the item without any cross-lane traffic. For each row block the
// forward sums of the active lanes
//   X_k[a] = sum_b P1[a][b] rt_c[b],           Y_k[b] = sum_a st_c[a] P2[a][b]
// are reduced across the warp through shared memory and added to the row's accumulator with
// FP64 atomics (a few per row block); the reverse sums are flushed once per work item.
//
// Arithmetic policies:
//   ArithF64 -- complex128 elements, FP64 fused multiply-adds (exact FP64 path).
//   ArithDF  -- (hi, lo) FP32 pairs for P and the vectors; products are error-free transformed
//               (p = xh*yh, e = fma(xh,yh,-p) + xh*yl + xl*yh) and sums use TwoSum on the high
//               parts, so each product carries ~2^-47 relative error and the FP32 pipes (64x the
//               FP64 rate on this part) do the work.
#pragma once
#include "dmd_common.cuh"
#include "dmd_layout.h"
#include "dmd_tma.cuh"

namespace dmd {

// ---------------------------------------------------------------------------------------------
// double-float helpers (no contraction: every operation is an explicit round-to-nearest op)
// ---------------------------------------------------------------------------------------------
struct dfc {  // complex (re_hi, re_lo, im_hi, im_lo)
  float rh, rl, ih, il;
};

__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
  s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

// (hi, lo) += x * y, x and y double-float
__device__ __forceinline__ void df_mac(float& hi, float& lo, float xh, float xl, float yh, float yl) {
  const float p = __fmul_rn(xh, yh);
  float e = __fmaf_rn(xh, yh, -p);
  e = __fmaf_rn(xh, yl, e);
  e = __fmaf_rn(xl, yh, e);
  float s, t;
  two_sum(hi, p, s, t);
  hi = s;
  lo = __fadd_rn(lo, __fadd_rn(t, e));
}

__device__ __forceinline__ void df_renorm(float& hi, float& lo) {
  const float s = __fadd_rn(hi, lo);
  lo = __fsub_rn(lo, __fsub_rn(s, hi));
  hi = s;
}

// (hi, lo) += (bh, bl)
__device__ __forceinline__ void df_add(float& hi, float& lo, float bh, float bl) {
  float s, t;
  two_sum(hi, bh, s, t);
  hi = s;
  lo = __fadd_rn(lo, __fadd_rn(t, bl));
}

__device__ __forceinline__ float4 split_df(double2 v) {
  const float rh = __double2float_rn(v.x), ih = __double2float_rn(v.y);
  return make_float4(rh, __double2float_rn(v.x - (double)rh), ih, __double2float_rn(v.y - (double)ih));
}

struct ArithDF {
  typedef float4 elem;  // P and vector element: (re_h, re_l, im_h, im_l)
  struct acc {
    float rh, rl, ih, il;
  };
  static __device__ __forceinline__ void zero(acc& a) { a.rh = a.rl = a.ih = a.il = 0.f; }
  // a += x * y
  static __device__ __forceinline__ void mac(acc& a, const elem& x, const elem& y) {
    df_mac(a.rh, a.rl, x.x, x.y, y.x, y.y);
    df_mac(a.rh, a.rl, -x.z, -x.w, y.z, y.w);
    df_mac(a.ih, a.il, x.x, x.y, y.z, y.w);
    df_mac(a.ih, a.il, x.z, x.w, y.x, y.y);
  }
  // a += conj(x) * y
  static __device__ __forceinline__ void mac_cx(acc& a, const elem& x, const elem& y) {
    df_mac(a.rh, a.rl, x.x, x.y, y.x, y.y);
    df_mac(a.rh, a.rl, x.z, x.w, y.z, y.w);
    df_mac(a.ih, a.il, x.x, x.y, y.z, y.w);
    df_mac(a.ih, a.il, -x.z, -x.w, y.x, y.y);
  }
  static __device__ __forceinline__ void renorm(acc& a) {
    df_renorm(a.rh, a.rl);
    df_renorm(a.ih, a.il);
  }
  static __device__ __forceinline__ void acc_add(acc& a, const acc& b) {
    df_add(a.rh, a.rl, b.rh, b.rl);
    df_add(a.ih, a.il, b.ih, b.il);
  }
  // reduction scratch entry: one real (hi, lo)
  typedef float2 red_t;
  static __device__ __forceinline__ float2 red_re(const acc& a) { return make_float2(a.rh, a.rl); }
  static __device__ __forceinline__ float2 red_im(const acc& a) { return make_float2(a.ih, a.il); }
  static __device__ __forceinline__ float2 red_zero() { return make_float2(0.f, 0.f); }
  static __device__ __forceinline__ void red_add(float2& s, float2 b) { df_add(s.x, s.y, b.x, b.y); }
  static __device__ __forceinline__ float2 red_shfl_xor(float2 v, int m) {
    return make_float2(__shfl_xor_sync(0xffffffffu, v.x, m), __shfl_xor_sync(0xffffffffu, v.y, m));
  }
  static __device__ __forceinline__ double red_to_double(float2 v) { return (double)v.x + (double)v.y; }
  static __device__ __forceinline__ double re_d(const acc& a) { return (double)a.rh + (double)a.rl; }
  static __device__ __forceinline__ double im_d(const acc& a) { return (double)a.ih + (double)a.il; }
  static __device__ __forceinline__ elem from_double2(double2 v) { return split_df(v); }
};

struct ArithF64 {
  typedef double2 elem;
  struct acc {
    double x, y;
  };
  static __device__ __forceinline__ void zero(acc& a) { a.x = a.y = 0.0; }
  static __device__ __forceinline__ void mac(acc& a, const elem& x, const elem& y) {
    a.x = fma(x.x, y.x, fma(-x.y, y.y, a.x));
    a.y = fma(x.x, y.y, fma(x.y, y.x, a.y));
  }
  static __device__ __forceinline__ void mac_cx(acc& a, const elem& x, const elem& y) {
    a.x = fma(x.x, y.x, fma(x.y, y.y, a.x));
    a.y = fma(x.x, y.y, fma(-x.y, y.x, a.y));
  }
  static __device__ __forceinline__ void renorm(acc&) {}
  static __device__ __forceinline__ void acc_add(acc& a, const acc& b) {
    a.x += b.x;
    a.y += b.y;
  }
  typedef double red_t;
  static __device__ __forceinline__ double red_re(const acc& a) { return a.x; }
  static __device__ __forceinline__ double red_im(const acc& a) { return a.y; }
  static __device__ __forceinline__ double red_zero() { return 0.0; }
  static __device__ __forceinline__ void red_add(double& s, double b) { s += b; }
  static __device__ __forceinline__ double red_shfl_xor(double v, int m) { return __shfl_xor_sync(0xffffffffu, v, m); }
  static __device__ __forceinline__ double red_to_double(double v) { return v; }
  static __device__ __forceinline__ double re_d(const acc& a) { return a.x; }
  static __device__ __forceinline__ double im_d(const acc& a) { return a.y; }
  static __device__ __forceinline__ elem from_double2(double2 v) { return v; }
};

template <typename E>
__device__ __forceinline__ E ld_stream(const E* p) {
  return __ldcs(p);
}

// rs: [nk][2][NB2] vectors in position (energy-rank) order; acc: [nk][2][NB2] double2
template <typename A, int NB>
__global__ void __launch_bounds__(128) k_pairs_cb(const WorkItem* __restrict__ items, int nitems,
                                                  const RowBlock* __restrict__ rbs,
                                                  const typename A::elem* __restrict__ P,
                                                  const typename A::elem* __restrict__ rs, double* __restrict__ acc,
                                                  int nk) {
  constexpr int NB2 = NB * NB, NB4 = NB2 * NB2, NV = 4 * NB2;  // NV reals per forward block (X, Y)
  typedef typename A::elem E;
  typedef typename A::acc Acc;
  typedef typename A::red_t R;
  __shared__ R red[4][NV][32];
  const int wib = threadIdx.x >> 5;
  const int lane = threadIdx.x & 31;
  const int item = blockIdx.x * 4 + wib;
  if (item >= nitems) return;
  const WorkItem w = items[item];
  const int col = w.J * 32 + lane;
  const bool colok = col < nk;
  E rc[NB2], sc[NB2];
#pragma unroll
  for (int i = 0; i < NB2; ++i) {
    rc[i] = colok ? rs[(size_t)col * 2 * NB2 + i] : E();
    sc[i] = colok ? rs[(size_t)col * 2 * NB2 + NB2 + i] : E();
  }
  Acc rX[NB2], rY[NB2];
#pragma unroll
  for (int i = 0; i < NB2; ++i) {
    A::zero(rX[i]);
    A::zero(rY[i]);
  }
  bool any_rev = false;
  const unsigned lt = (1u << lane) - 1u;
  for (int r = w.rb0; r < w.rb1; ++r) {
    const RowBlock b = rbs[r];
    const bool active = (b.mask >> lane) & 1u;
    const bool rev = (b.revmask >> lane) & 1u;
    any_rev |= rev;
    const int n = __popc(b.mask);
    const int slot = __popc(b.mask & lt);
    if (active) {
      const E* rrow = rs + (size_t)b.row * 2 * NB2;
      const E* base = P + (size_t)b.pair0 * 2 * NB4 + slot;
      {  // P1 block: X_k[a] += P1[a][c] rt_col[c];  Y_col[c] += st_k[a] conj(P1[a][c])
        E sr[NB2];
        Acc f[NB2];
#pragma unroll
        for (int i = 0; i < NB2; ++i) {
          sr[i] = rrow[NB2 + i];
          A::zero(f[i]);
        }
#pragma unroll
        for (int a = 0; a < NB2; ++a)
#pragma unroll
          for (int c = 0; c < NB2; ++c) {
            const E p1 = ld_stream(base + (size_t)(a * NB2 + c) * n);
            A::mac(f[a], p1, rc[c]);
            if (rev) A::mac_cx(rY[c], p1, sr[a]);
          }
#pragma unroll
        for (int i = 0; i < NB2; ++i) {
          red[wib][2 * i][lane] = A::red_re(f[i]);
          red[wib][2 * i + 1][lane] = A::red_im(f[i]);
        }
      }
      {  // P2 block: Y_k[c] += st_col[a] P2[a][c];  X_col[a] += conj(P2[a][c]) rt_k[c]
        E rr[NB2];
        Acc f[NB2];
#pragma unroll
        for (int i = 0; i < NB2; ++i) {
          rr[i] = rrow[i];
          A::zero(f[i]);
        }
#pragma unroll
        for (int a = 0; a < NB2; ++a)
#pragma unroll
          for (int c = 0; c < NB2; ++c) {
            const E p2 = ld_stream(base + (size_t)(NB4 + c * NB2 + a) * n);  // P2 stored column-major
            A::mac(f[c], p2, sc[a]);
            if (rev) A::mac_cx(rX[a], p2, rr[c]);
          }
#pragma unroll
        for (int i = 0; i < NB2; ++i) {
          red[wib][2 * NB2 + 2 * i][lane] = A::red_re(f[i]);
          red[wib][2 * NB2 + 2 * i + 1][lane] = A::red_im(f[i]);
        }
      }
      if (rev) {
#pragma unroll
        for (int i = 0; i < NB2; ++i) {
          A::renorm(rX[i]);
          A::renorm(rY[i]);
        }
      }
    }
    __syncwarp();
    constexpr int LPV = 32 / NV > 0 ? 32 / NV : 1;  // lanes per value
    for (int v0 = 0; v0 < NV; v0 += 32 / LPV) {
      const int v = v0 + lane / LPV;
      const int part = lane % LPV;
      R s = A::red_zero();
      if (v < NV) {
        const int span = 32 / LPV;
        for (int j = part * span; j < (part + 1) * span; ++j)
          if ((b.mask >> j) & 1u) A::red_add(s, red[wib][v][j]);
      }
#pragma unroll
      for (int m = 1; m < LPV; m <<= 1) A::red_add(s, A::red_shfl_xor(s, m));
      if (v < NV && part == 0) atomicAdd(acc + (size_t)b.row * 2 * NB2 * 2 + v, A::red_to_double(s));
    }
    __syncwarp();
  }
  // reverse sums of this item's column
  if (colok && any_rev) {
    double* dst = acc + (size_t)col * 2 * NB2 * 2;
#pragma unroll
    for (int i = 0; i < NB2; ++i) {
      atomicAdd(dst + 2 * i, A::re_d(rX[i]));
      atomicAdd(dst + 2 * i + 1, A::im_d(rX[i]));
      atomicAdd(dst + 2 * NB2 + 2 * i, A::re_d(rY[i]));
      atomicAdd(dst + 2 * NB2 + 2 * i + 1, A::im_d(rY[i]));
    }
  }
}

// prep for the column-block kernels: rt, st per k written at pos[k] in the arithmetic's element
// format, accumulators zeroed. One thread per (k, element).
template <typename A, int NB>
__global__ void k_prep_cb(int nk, int nbdm, int bs, const double2* __restrict__ y, const double* __restrict__ ew,
                          const int* __restrict__ pos, TimeArg ta, int phase, typename A::elem* __restrict__ rs,
                          double2* __restrict__ acc) {
  constexpr int NB2 = NB * NB;
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= nk * NB2) return;
  const int k = idx / NB2, ab = idx - k * NB2, i = ab / NB, j = ab - i * NB;
  const double2 r = y[(size_t)k * nbdm * nbdm + (bs + i) * nbdm + bs + j];
  const double2 s = (i == j) ? mk2(1.0 - r.x, 0.0 - r.y) : mk2(-r.x, -r.y);
  double2 rt = r, st = s;
  if (phase) {
    const double t = eval_time(ta);
    const double2 d = ccis((ew[k * NB + i] - ew[k * NB + j]) * t);
    rt = cmul_rn(cconj(d), r);
    st = cmul_rn(cconj(d), s);
  }
  const int p = pos[k];
  rs[(size_t)p * 2 * NB2 + ab] = A::from_double2(rt);
  rs[(size_t)p * 2 * NB2 + NB2 + ab] = A::from_double2(st);
  acc[(size_t)p * 2 * NB2 + ab] = mk2(0.0, 0.0);
  acc[(size_t)p * 2 * NB2 + NB2 + ab] = mk2(0.0, 0.0);
}


// ---------------------------------------------------------------------------------------------
// The same contraction with the P elements staged through shared memory by bulk copies.
//
// In this layout each pair stores P1 row-major and P2 column-major, so both halves are consumed
// "line by line": a P1 row a completes the forward output X_k[a] and a P2 column c completes
// Y_k[c], while the lane's reverse sums Y_col (indexed by P1's column) and X_col (indexed by P2's
// row) stay in registers with compile-time indices. A row block is consumed in chunks of LINES
// lines; each warp double-buffers its chunks, issuing the copy of chunk i + 2 while it computes
// chunk i. The row's vectors rt_k, st_k are staged in shared memory once per row block. Waits are
// bounded (dmd_tma.cuh); a timeout sets *errflag.
// ---------------------------------------------------------------------------------------------
template <typename A, int NB, int LINES>
struct CbTmaSmem {
  static constexpr int NB2 = NB * NB, NB4 = NB2 * NB2, NV = 4 * NB2;
  static constexpr int CPM = NB2 / LINES;  // chunks per matrix
  static constexpr int CPR = 2 * CPM;      // chunks per row block
  static constexpr size_t stage_bytes = (size_t)LINES * NB2 * 32 * sizeof(typename A::elem);
  static constexpr size_t red_bytes = (size_t)NV * 32 * sizeof(typename A::red_t);
  static constexpr size_t row_bytes = (size_t)2 * NB2 * sizeof(typename A::elem);
  static constexpr size_t warp_bytes = ((2 * stage_bytes + red_bytes + row_bytes + 16) + 127) / 128 * 128;
  static constexpr size_t cta_bytes = 4 * warp_bytes;
};

template <typename A, int NB, int LINES, int MINB>
__global__ void __launch_bounds__(128, MINB) k_pairs_cb_tma(const WorkItem* __restrict__ items, int nitems,
                                                            const RowBlock* __restrict__ rbs,
                                                            const typename A::elem* __restrict__ P,
                                                            const typename A::elem* __restrict__ rs,
                                                            double* __restrict__ acc, int nk,
                                                            unsigned int* __restrict__ errflag) {
  typedef CbTmaSmem<A, NB, LINES> S;
  constexpr int NB2 = S::NB2, NB4 = S::NB4, NV = S::NV, CPM = S::CPM, CPR = S::CPR;
  constexpr size_t SE = S::stage_bytes / sizeof(typename A::elem);  // elements per stage
  typedef typename A::elem E;
  typedef typename A::acc Acc;
  typedef typename A::red_t R;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  const int wib = threadIdx.x >> 5;
  const int lane = threadIdx.x & 31;
  const int item = blockIdx.x * 4 + wib;
  if (item >= nitems) return;
  unsigned char* wbase = smem_raw + (size_t)wib * S::warp_bytes;
  E* const stage0 = (E*)wbase;
  R* const red = (R*)(wbase + 2 * S::stage_bytes);                             // [NV][32]
  E* const rowv = (E*)(wbase + 2 * S::stage_bytes + S::red_bytes);             // rt_k[NB2], st_k[NB2]
  uint64_t* const bar = (uint64_t*)(wbase + 2 * S::stage_bytes + S::red_bytes + S::row_bytes);
  const WorkItem w = items[item];
  const int nch = CPR * (w.rb1 - w.rb0);
  if (lane == 0) {
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
    fence_mbar_init();
  }
  __syncwarp();
  const uint64_t pol = policy_evict_first();
  auto issue = [&](int c) {  // lane 0 only: chunk c of the item into stage c & 1
    const RowBlock b = rbs[w.rb0 + c / CPR];
    const int q = c % CPR;
    const int n = __popc(b.mask);
    const size_t off = (size_t)b.pair0 * 2 * NB4 + ((size_t)(q / CPM) * NB4 + (size_t)(q % CPM) * LINES * NB2) * n;
    const uint32_t bytes = (uint32_t)(LINES * NB2 * n * sizeof(E));
    mbar_arrive_expect_tx(&bar[c & 1], bytes);
    bulk_g2s(stage0 + (size_t)(c & 1) * SE, P + off, bytes, &bar[c & 1], pol);
  };
  if (lane == 0) {
    issue(0);
    if (nch > 1) issue(1);
  }
  const int col = w.J * 32 + lane;
  const bool colok = col < nk;
  E rc[NB2], sc[NB2];
#pragma unroll
  for (int i = 0; i < NB2; ++i) {
    rc[i] = colok ? rs[(size_t)col * 2 * NB2 + i] : E();
    sc[i] = colok ? rs[(size_t)col * 2 * NB2 + NB2 + i] : E();
  }
  Acc rX[NB2], rY[NB2];
#pragma unroll
  for (int i = 0; i < NB2; ++i) {
    A::zero(rX[i]);
    A::zero(rY[i]);
  }
  bool any_rev = false;
  bool failed = false;
  const unsigned lt = (1u << lane) - 1u;
#pragma unroll 1
  for (int rbi = 0; rbi < w.rb1 - w.rb0; ++rbi) {
    const RowBlock b = rbs[w.rb0 + rbi];
    const bool active = (b.mask >> lane) & 1u;
    const bool rev = (b.revmask >> lane) & 1u;
    any_rev |= rev;
    const int n = __popc(b.mask);
    const int slot = __popc(b.mask & lt);
    if (lane < 2 * NB2) rowv[lane] = rs[(size_t)b.row * 2 * NB2 + lane];
    __syncwarp();
#pragma unroll 1
    for (int q = 0; q < CPR; ++q) {
      const int c = rbi * CPR + q;
      if (!mbar_wait_bounded(&bar[c & 1], (uint32_t)((c >> 1) & 1), errflag)) {
        failed = true;
        break;
      }
      const E* st = stage0 + (size_t)(c & 1) * SE + slot;
      const int l0 = (q % CPM) * LINES;
      if (active) {
        if (q < CPM) {
          // P1 rows a = l0..: X_k[a] = sum_cc P1[a][cc] rt_col[cc];  Y_col[cc] += st_k[a] conj(P1[a][cc])
#pragma unroll
          for (int r = 0; r < LINES; ++r) {
            const int a = l0 + r;
            const E sra = rowv[NB2 + a];
            Acc f;
            A::zero(f);
#pragma unroll
            for (int cc = 0; cc < NB2; ++cc) {
              const E p1 = st[(r * NB2 + cc) * n];
              A::mac(f, p1, rc[cc]);
              if (rev) A::mac_cx(rY[cc], p1, sra);
            }
            red[(2 * a) * 32 + lane] = A::red_re(f);
            red[(2 * a + 1) * 32 + lane] = A::red_im(f);
          }
        } else {
          // P2 columns cc = l0..: Y_k[cc] = sum_a st_col[a] P2[a][cc];  X_col[a] += conj(P2[a][cc]) rt_k[cc]
#pragma unroll
          for (int r = 0; r < LINES; ++r) {
            const int cc = l0 + r;
            const E rrc = rowv[cc];
            Acc f;
            A::zero(f);
#pragma unroll
            for (int a = 0; a < NB2; ++a) {
              const E p2 = st[(r * NB2 + a) * n];
              A::mac(f, p2, sc[a]);
              if (rev) A::mac_cx(rX[a], p2, rrc);
            }
            red[(2 * NB2 + 2 * cc) * 32 + lane] = A::red_re(f);
            red[(2 * NB2 + 2 * cc + 1) * 32 + lane] = A::red_im(f);
          }
        }
      }
      // the stage buffer is free once every lane has read it: order those reads before the next
      // bulk copy into it (generic -> async proxy), then refill it
      fence_proxy_async();
      __syncwarp();
      if (lane == 0 && c + 2 < nch) issue(c + 2);
    }
    if (failed) break;
    if (active && rev) {
#pragma unroll
      for (int i = 0; i < NB2; ++i) {
        A::renorm(rX[i]);
        A::renorm(rY[i]);
      }
    }
    // the row block is complete: forward reduction over the active lanes
    constexpr int LPV = 32 / NV > 0 ? 32 / NV : 1;
#pragma unroll 1
    for (int v0 = 0; v0 < NV; v0 += 32 / LPV) {
      const int v = v0 + lane / LPV;
      const int part = lane % LPV;
      R s = A::red_zero();
      if (v < NV) {
        const int span = 32 / LPV;
        unsigned m = (b.mask >> (part * span)) & (span == 32 ? 0xffffffffu : ((1u << span) - 1u));
        while (m) {
          const int j = __ffs(m) - 1;
          m &= m - 1;
          A::red_add(s, red[v * 32 + part * span + j]);
        }
      }
#pragma unroll
      for (int mm = 1; mm < LPV; mm <<= 1) A::red_add(s, A::red_shfl_xor(s, mm));
      if (v < NV && part == 0) atomicAdd(acc + (size_t)b.row * 2 * NB2 * 2 + v, A::red_to_double(s));
    }
    __syncwarp();
  }
  if (failed) {  // drain whatever copies are still pending (bounded), then leave
    if (lane == 0) {
      mbar_wait_bounded(&bar[0], 0, nullptr, 1u << 16);
      mbar_wait_bounded(&bar[1], 0, nullptr, 1u << 16);
      mbar_wait_bounded(&bar[0], 1, nullptr, 1u << 16);
      mbar_wait_bounded(&bar[1], 1, nullptr, 1u << 16);
    }
    __syncwarp();
    return;
  }
  if (colok && any_rev) {
    double* dst = acc + (size_t)col * 2 * NB2 * 2;
#pragma unroll
    for (int i = 0; i < NB2; ++i) {
      atomicAdd(dst + 2 * i, A::re_d(rX[i]));
      atomicAdd(dst + 2 * i + 1, A::im_d(rX[i]));
      atomicAdd(dst + 2 * NB2 + 2 * i, A::re_d(rY[i]));
      atomicAdd(dst + 2 * NB2 + 2 * i + 1, A::im_d(rY[i]));
    }
  }
}

}  // namespace dmd
