// Column-block k-pair contraction in Hermitian coordinates (layout in dmd_layout.h).
//
// Coordinates. rt_k = conj(D_k) o rho_k and st_k = conj(D_k) o (1 - rho_k) are Hermitian nb x nb
// matrices when rho_k is (D_k[(i,j)] = exp(i t (e_i - e_j))). A Hermitian matrix v has nb^2 real
// coordinates q: q[(i,i)] = v_ii, and for i < j q[(i,j)] = Re v_ij, q[(j,i)] = Im v_ij, so v = M q
// with M[(ij),(ij)] = 1, M[(ij),(ji)] = i, M[(ji),(ij)] = 1, M[(ji),(ji)] = -i. The host stores
//   Q1 = M^H P1 M      (row-major, like P1)        Q2 = M^T P2 conj(M)   (column-major, like P2)
// and the kernel accumulates the transformed sums X' = M^H X, Y' = M^H Y:
//   X'_k   += Q1 r_c                      Y'_c[j] += sum_a s_k[a] conj(Q1[a][j])
//   Y'_k[j] += sum_a Q2[a][j] s_c[a]      X'_c[a] += sum_j conj(Q2[a][j]) r_k[j]
// (r, s: coordinates of rt, st). Every product is complex x real -- half the multiply-adds of the
// complex form -- and the finish maps X = (M^H)^-1 X' back (k_finish, herm = 1).
// A state that is not exactly Hermitian is split rho = H + i A with H, A Hermitian; the A part's
// coordinates go through a second launch of the same kernel, gated on a device flag that the prep
// kernel raises, whose sums are multiplied by i. The arithmetic is linear in the vectors, so the
// two launches together equal the general complex contraction.
//
// Work decomposition. One warp per work item: a run of row blocks of one column block J. Lane s
// owns column c = 32 J + s: it keeps r_c, s_c in registers and accumulates the reverse (column
// side) sums across all row blocks of the item without cross-lane traffic. For each row block the
// forward sums of the active lanes are reduced through shared memory and added to the row's
// accumulator with FP64 atomics; the reverse sums are flushed once per work item. The P elements
// of a row block are staged through shared memory by bulk copies (TMA unit), double-buffered per
// warp, with bounded waits.
//
// Arithmetic policies:
//   ArithF64 -- complex128 P, FP64 fused multiply-adds (exact FP64 path).
//   ArithDF  -- (hi, lo) FP32 pairs for P and the coordinates; products are error-free transformed
//               (p = xh*yh, e = fma(xh,yh,-p) + xh*yl + xl*yh) and sums use TwoSum on the high
//               parts, so each product carries ~2^-47 relative error and the FP32 pipes (64x the
//               FP64 rate on this part) do the work; the real and the imaginary half of each step
//               are one FP32x2 instruction.
#pragma once
#include "dmd_common.cuh"
#include "dmd_layout.h"
#include "dmd_tma.cuh"

namespace dmd {

// ---------------------------------------------------------------------------------------------
// double-float helpers (no contraction: every operation is an explicit round-to-nearest op)
// ---------------------------------------------------------------------------------------------
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

// (hi, lo) = x * y
__device__ __forceinline__ void df_mul(float& hi, float& lo, float xh, float xl, float yh, float yl) {
  const float p = __fmul_rn(xh, yh);
  float e = __fmaf_rn(xh, yh, -p);
  e = __fmaf_rn(xh, yl, e);
  lo = __fmaf_rn(xl, yh, e);
  hi = p;
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

__device__ __forceinline__ float2 split_df1(double v) {
  const float h = __double2float_rn(v);
  return make_float2(h, __double2float_rn(v - (double)h));
}

// Packed (re, im) double-float arithmetic on the FP32x2 instructions (fma/add/mul .f32x2): both
// halves of every instruction are the same round-to-nearest operation that the scalar helpers above
// perform, so the results are bit-identical to applying those helpers to the real and the imaginary
// part, at half the issued instructions. a - b is fma(b, -1, a), one rounding of the exact difference.
__device__ __forceinline__ float2 f2sub(float2 a, float2 b) { return __ffma2_rn(b, make_float2(-1.f, -1.f), a); }

// packed TwoSum: s + e = a + b exactly, per half
__device__ __forceinline__ void two_sum2(float2 a, float2 b, float2& s, float2& e) {
  s = __fadd2_rn(a, b);
  const float2 bb = f2sub(s, a);
  e = __fadd2_rn(f2sub(a, f2sub(s, bb)), f2sub(b, bb));
}

struct ArithDF {
  // P element: (re_h, im_h, re_l, im_l) -- the high parts and the low parts as FP32x2 pairs
  typedef float4 elem;
  typedef float2 relem;  // real coordinate: (h, l)
  // a coordinate prepared for the products: (h, h, l, l), or (h, -h, l, -l) for conj(x) * v
  typedef float4 pcoord;
  typedef float4 pcoord_cx;
  struct acc {
    float2 h, l;  // (re, im) high parts, (re, im) low parts
  };
  static __device__ __forceinline__ pcoord prep(relem v) { return make_float4(v.x, v.x, v.y, v.y); }
  static __device__ __forceinline__ pcoord_cx prep_cx(relem v) { return make_float4(v.x, -v.x, v.y, -v.y); }
  static __device__ __forceinline__ float2 hi(const float4& x) { return make_float2(x.x, x.y); }
  static __device__ __forceinline__ float2 lo(const float4& x) { return make_float2(x.z, x.w); }
  static __device__ __forceinline__ void zero(acc& a) { a.h = a.l = make_float2(0.f, 0.f); }
  // a += x * v, v prepared: the error-free product (p = xh*vh, e = fma(xh,vh,-p) + xh*vl + xl*vh)
  // added with TwoSum on the high parts
  static __device__ __forceinline__ void pmac(acc& a, const elem& x, const float4& v) {
    const float2 xh = hi(x), xl = lo(x), vh = hi(v), vl = lo(v);
    const float2 p = __fmul2_rn(xh, vh);
    float2 e = __ffma2_rn(xh, vh, make_float2(-p.x, -p.y));
    e = __ffma2_rn(xh, vl, e);
    e = __ffma2_rn(xl, vh, e);
    float2 s, t;
    two_sum2(a.h, p, s, t);
    a.h = s;
    a.l = __fadd2_rn(a.l, __fadd2_rn(t, e));
  }
  static __device__ __forceinline__ void mac(acc& a, const elem& x, const pcoord& v) { pmac(a, x, v); }
  // a += conj(x) * v (v prepared by prep_cx: the imaginary half multiplies by -v)
  static __device__ __forceinline__ void mac_cx(acc& a, const elem& x, const pcoord_cx& v) { pmac(a, x, v); }
  // a = x * v
  static __device__ __forceinline__ void mul(acc& a, const elem& x, const pcoord& v) {
    const float2 xh = hi(x), xl = lo(x), vh = hi(v), vl = lo(v);
    const float2 p = __fmul2_rn(xh, vh);
    float2 e = __ffma2_rn(xh, vh, make_float2(-p.x, -p.y));
    e = __ffma2_rn(xh, vl, e);
    a.l = __ffma2_rn(xl, vh, e);
    a.h = p;
  }
  static __device__ __forceinline__ void renorm(acc& a) {
    const float2 s = __fadd2_rn(a.h, a.l);
    a.l = f2sub(a.l, f2sub(s, a.h));
    a.h = s;
  }
  // forward flush on packed complex entries (re_h, im_h, re_l, im_l), multiplied by i when imag
  static constexpr bool kPackedRed = true;
  static __device__ __forceinline__ float4 red_pack(const acc& a, bool imag) {
    return imag ? make_float4(-a.h.y, a.h.x, -a.l.y, a.l.x) : make_float4(a.h.x, a.h.y, a.l.x, a.l.y);
  }
  // s += b (double-float, per half)
  static __device__ __forceinline__ void red_add4(float4& s, const float4& b) {
    float2 h, t;
    two_sum2(hi(s), hi(b), h, t);
    const float2 l = __fadd2_rn(lo(s), __fadd2_rn(t, lo(b)));
    s = make_float4(h.x, h.y, l.x, l.y);
  }
  // reduction scratch entry: one real (hi, lo)
  typedef float2 red_t;
  static __device__ __forceinline__ float2 red_re(const acc& a) { return make_float2(a.h.x, a.l.x); }
  static __device__ __forceinline__ float2 red_im(const acc& a) { return make_float2(a.h.y, a.l.y); }
  static __device__ __forceinline__ float2 red_neg(float2 v) { return make_float2(-v.x, -v.y); }
  static __device__ __forceinline__ float2 red_zero() { return make_float2(0.f, 0.f); }
  static __device__ __forceinline__ void red_add(float2& s, float2 b) { df_add(s.x, s.y, b.x, b.y); }
  static __device__ __forceinline__ float2 red_shfl_xor(float2 v, int m) {
    return make_float2(__shfl_xor_sync(0xffffffffu, v.x, m), __shfl_xor_sync(0xffffffffu, v.y, m));
  }
  static __device__ __forceinline__ double red_to_double(float2 v) { return (double)v.x + (double)v.y; }
  static __device__ __forceinline__ double re_d(const acc& a) { return (double)a.h.x + (double)a.l.x; }
  static __device__ __forceinline__ double im_d(const acc& a) { return (double)a.h.y + (double)a.l.y; }
  static __device__ __forceinline__ relem from_double(double v) { return split_df1(v); }
};

struct ArithF64 {
  typedef double2 elem;
  typedef double relem;
  typedef double pcoord;
  typedef double pcoord_cx;
  static __device__ __forceinline__ double prep(double v) { return v; }
  static __device__ __forceinline__ double prep_cx(double v) { return v; }
  struct acc {
    double x, y;
  };
  static __device__ __forceinline__ void zero(acc& a) { a.x = a.y = 0.0; }
  static __device__ __forceinline__ void mac(acc& a, const elem& x, const relem& v) {
    a.x = fma(x.x, v, a.x);
    a.y = fma(x.y, v, a.y);
  }
  static __device__ __forceinline__ void mac_cx(acc& a, const elem& x, const relem& v) {
    a.x = fma(x.x, v, a.x);
    a.y = fma(-x.y, v, a.y);
  }
  static __device__ __forceinline__ void mul(acc& a, const elem& x, const relem& v) {
    a.x = x.x * v;
    a.y = x.y * v;
  }
  static __device__ __forceinline__ void renorm(acc&) {}
  static constexpr bool kPackedRed = false;
  typedef double red_t;
  static __device__ __forceinline__ double red_re(const acc& a) { return a.x; }
  static __device__ __forceinline__ double red_im(const acc& a) { return a.y; }
  static __device__ __forceinline__ double red_neg(double v) { return -v; }
  static __device__ __forceinline__ double red_zero() { return 0.0; }
  static __device__ __forceinline__ void red_add(double& s, double b) { s += b; }
  static __device__ __forceinline__ double red_shfl_xor(double v, int m) { return __shfl_xor_sync(0xffffffffu, v, m); }
  static __device__ __forceinline__ double red_to_double(double v) { return v; }
  static __device__ __forceinline__ double re_d(const acc& a) { return a.x; }
  static __device__ __forceinline__ double im_d(const acc& a) { return a.y; }
  static __device__ __forceinline__ relem from_double(double v) { return v; }
};

// Reduced-precision forms: Q stored complex64 (ArithF32) or as bf16 hi + bf16 lo per component
// (ArithBF2, one 32-bit word per component: hi in the upper half, lo in the lower), FP32 products
// and sums, FP64 atomics. They contract only rho - diag(f_ref) (see k_prep_herm).
struct ArithF32 {
  typedef float2 elem;
  typedef float relem;
  typedef float pcoord;
  typedef float pcoord_cx;
  static __device__ __forceinline__ float prep(float v) { return v; }
  static __device__ __forceinline__ float prep_cx(float v) { return v; }
  typedef float2 acc;
  static __device__ __forceinline__ float2 val(const elem& x) { return x; }
  static __device__ __forceinline__ void zero(acc& a) { a.x = a.y = 0.f; }
  static __device__ __forceinline__ void mac(acc& a, const elem& x, const relem& v) {
    a.x = __fmaf_rn(x.x, v, a.x);
    a.y = __fmaf_rn(x.y, v, a.y);
  }
  static __device__ __forceinline__ void mac_cx(acc& a, const elem& x, const relem& v) {
    a.x = __fmaf_rn(x.x, v, a.x);
    a.y = __fmaf_rn(-x.y, v, a.y);
  }
  static __device__ __forceinline__ void mul(acc& a, const elem& x, const relem& v) {
    a.x = __fmul_rn(x.x, v);
    a.y = __fmul_rn(x.y, v);
  }
  static __device__ __forceinline__ void renorm(acc&) {}
  static constexpr bool kPackedRed = false;
  typedef float red_t;
  static __device__ __forceinline__ float red_re(const acc& a) { return a.x; }
  static __device__ __forceinline__ float red_im(const acc& a) { return a.y; }
  static __device__ __forceinline__ float red_neg(float v) { return -v; }
  static __device__ __forceinline__ float red_zero() { return 0.f; }
  static __device__ __forceinline__ void red_add(float& s, float b) { s = __fadd_rn(s, b); }
  static __device__ __forceinline__ float red_shfl_xor(float v, int m) { return __shfl_xor_sync(0xffffffffu, v, m); }
  static __device__ __forceinline__ double red_to_double(float v) { return (double)v; }
  static __device__ __forceinline__ double re_d(const acc& a) { return (double)a.x; }
  static __device__ __forceinline__ double im_d(const acc& a) { return (double)a.y; }
  static __device__ __forceinline__ relem from_double(double v) { return __double2float_rn(v); }
};

__device__ __forceinline__ float bf2_to_float(uint32_t w) {
  return __fadd_rn(__uint_as_float(w & 0xffff0000u), __uint_as_float(w << 16));
}

struct ArithBF2 : ArithF32 {
  typedef uint2 elem;
  static __device__ __forceinline__ float2 val(const elem& x) { return make_float2(bf2_to_float(x.x), bf2_to_float(x.y)); }
  static __device__ __forceinline__ void mac(acc& a, const elem& x, const relem& v) { ArithF32::mac(a, val(x), v); }
  static __device__ __forceinline__ void mac_cx(acc& a, const elem& x, const relem& v) { ArithF32::mac_cx(a, val(x), v); }
  static __device__ __forceinline__ void mul(acc& a, const elem& x, const relem& v) { ArithF32::mul(a, val(x), v); }
};

// ---------------------------------------------------------------------------------------------
// Prep: Hermitian and anti-Hermitian coordinates of rt, st per k (written at pos[k]) and the
// accumulators' start values (zero, or acc0; skipped when acc is null). One thread per (energy rank
// p, element (i, j)) and chunk of qc states, k = inv[p], so that the stores run in position order;
// the thread of (i, j) with i < j writes the coordinates at (i, j) and (j, i). ws = 0 skips the st
// coordinates (the tensor-core form contracts rt only, s = -r there); the tensor-core form (ws = 0,
// FP32 coordinates) also takes its phases and its off-diagonal products in FP32 (the phase argument
// is reduced modulo 2 pi in FP64) and stores FP32 phases in ph. Raises *hflag
// when some rho_k is not exactly Hermitian. rs layout: [nrhs][nk][2][NB2] Hermitian part (r, s), then
// the anti-Hermitian part; the batched form runs one grid row (blockIdx.y) per chunk of states, and
// the phase D_k(i, j) = exp(i t (e_i - e_j)) is computed once per thread for all states of its chunk.
// The first chunk stores D_k in ph ([nk][NB2], read by the finish kernel).
// Deviation form (fref != null, window occupations [nk][NB]): the coordinates are those of
// rho - diag(f) and of (1 - rho) - diag(1 - f) = -(rho - diag(f)); the contraction of diag(f) is
// the constant acc0 (position order), formed once in FP64. Linearized form (lin): the coordinates of
// rho - diag(f_eq) only, with zero st coordinates (the Q2 slot then carries the reverse operator).
// ---------------------------------------------------------------------------------------------
template <typename A, int NB>
__global__ void k_prep_herm(int nk, int nbdm, int bs, const double2* __restrict__ y, const double* __restrict__ ew,
                            const int* __restrict__ inv, TimeArg ta, int phase, typename A::relem* __restrict__ rs,
                            double2* __restrict__ acc, unsigned int* __restrict__ hflag,
                            const double* __restrict__ fref, const double2* __restrict__ acc0, int lin,
                            int nrhs, int qc, double2* __restrict__ ph, int ws) {
  constexpr int NB2 = NB * NB;
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= nk * NB2) return;
  const int q0 = blockIdx.y * qc, q1 = min(nrhs, q0 + qc);
  const size_t cstride = (size_t)nk * 2 * NB2;  // coordinates (and sums) per state
  const size_t sstride = (size_t)nk * nbdm * nbdm;
  const int p = idx / NB2, ab = idx - p * NB2, i = ab / NB, j = ab - i * NB;
  const int k = inv[p];
  const size_t ax = (size_t)p * 2 * NB2 + ab;
  if (acc) {
    const double2 a0 = acc0 ? acc0[ax] : mk2(0.0, 0.0), a1 = acc0 ? acc0[ax + NB2] : mk2(0.0, 0.0);
    for (int q = q0; q < q1; ++q) {
      acc[(size_t)q * cstride + ax] = a0;
      acc[(size_t)q * cstride + ax + NB2] = a1;
    }
  }
  if (i > j) return;
  const double2* yk = y + (size_t)k * nbdm * nbdm;
  constexpr bool F32C = sizeof(typename A::relem) == 4;  // FP32 coordinates
  const bool fast = F32C && ws == 0;
  if (i == j) {
    if (ph && blockIdx.y == 0) {
      if (fast) ((float2*)ph)[(size_t)k * NB2 + ab] = make_float2(1.f, 0.f);
      else ph[(size_t)k * NB2 + ab] = mk2(1.0, 0.0);
    }
    const double fi = fref ? fref[(size_t)k * NB + i] : 0.0;
    for (int q = q0; q < q1; ++q) {
      typename A::relem* rh = rs + (size_t)q * cstride + (size_t)p * 2 * NB2;
      typename A::relem* ra = rs + (size_t)(nrhs + q) * cstride + (size_t)p * 2 * NB2;
      const double2 vij = yk[(size_t)q * sstride + (bs + i) * nbdm + bs + j];
      // H_ii = Re rho_ii, A_ii = Im rho_ii; 1 - rho: (1 - Re rho_ii, -Im rho_ii) (set_oneminusdm)
      if (fref) {
        const double dv = __dsub_rn(vij.x, fi);
        rh[ab] = A::from_double(dv);
        if (ws) rh[NB2 + ab] = A::from_double(lin ? 0.0 : -dv);
      } else {
        rh[ab] = A::from_double(vij.x);
        if (ws) rh[NB2 + ab] = A::from_double(1.0 - vij.x);
      }
      ra[ab] = A::from_double(vij.y);
      if (ws) ra[NB2 + ab] = A::from_double(lin ? 0.0 : 0.0 - vij.y);
      if (vij.y != 0.0) atomicOr(hflag, 1u);
    }
    return;
  }
  const int ji = j * NB + i;
  if constexpr (F32C) {
    if (fast) {
      float2 dc = make_float2(1.f, 0.f);  // conj(D)
      if (phase) {
        const double x = (ew[k * NB + i] - ew[k * NB + j]) * eval_time(ta);
        const double xr = fma(-6.283185307179586, rint(x * 0.15915494309189535), x);
        float sn, cs;
        sincosf((float)xr, &sn, &cs);
        if (ph && blockIdx.y == 0) {
          ((float2*)ph)[(size_t)k * NB2 + ab] = make_float2(cs, sn);
          ((float2*)ph)[(size_t)k * NB2 + ji] = make_float2(cs, -sn);
        }
        dc = make_float2(cs, -sn);
      }
      for (int q = q0; q < q1; ++q) {
        typename A::relem* rh = rs + (size_t)q * cstride + (size_t)p * 2 * NB2;
        typename A::relem* ra = rs + (size_t)(nrhs + q) * cstride + (size_t)p * 2 * NB2;
        const double2 vij = yk[(size_t)q * sstride + (bs + i) * nbdm + bs + j];
        const double2 vji = yk[(size_t)q * sstride + (bs + j) * nbdm + bs + i];
        float2 hf = make_float2(0.5f * ((float)vij.x + (float)vji.x), 0.5f * ((float)vij.y - (float)vji.y));
        float2 af = make_float2(0.f, 0.f);
        if (vij.x != vji.x || vij.y != -vji.y) {  // not exactly Hermitian: the anti-Hermitian pass runs
          atomicOr(hflag, 1u);
          const double2 hij = mk2(__dmul_rn(__dadd_rn(vij.x, vji.x), 0.5), __dmul_rn(__dsub_rn(vij.y, vji.y), 0.5));
          const double2 dif = mk2(__dsub_rn(vij.x, vji.x), __dadd_rn(vij.y, vji.y));
          hf = make_float2((float)hij.x, (float)hij.y);
          af = make_float2((float)__dmul_rn(dif.y, 0.5), (float)__dmul_rn(-dif.x, 0.5));
        }
        const float2 r1 = make_float2(__fmaf_rn(dc.x, hf.x, -dc.y * hf.y), __fmaf_rn(dc.x, hf.y, dc.y * hf.x));
        const float2 r2 = make_float2(__fmaf_rn(dc.x, af.x, -dc.y * af.y), __fmaf_rn(dc.x, af.y, dc.y * af.x));
        rh[ab] = r1.x;
        rh[ji] = r1.y;
        ra[ab] = r2.x;
        ra[ji] = r2.y;
      }
      return;
    }
  }
  double2 d = mk2(1.0, 0.0);
  if (phase) {
    const double2 dk = ccis((ew[k * NB + i] - ew[k * NB + j]) * eval_time(ta));
    if (ph && blockIdx.y == 0) {
      ph[(size_t)k * NB2 + ab] = dk;
      ph[(size_t)k * NB2 + ji] = cconj(dk);
    }
    d = cconj(dk);
  }
  for (int q = q0; q < q1; ++q) {
    typename A::relem* rh = rs + (size_t)q * cstride + (size_t)p * 2 * NB2;
    typename A::relem* ra = rs + (size_t)(nrhs + q) * cstride + (size_t)p * 2 * NB2;
    const double2 vij = yk[(size_t)q * sstride + (bs + i) * nbdm + bs + j];
    const double2 vji = yk[(size_t)q * sstride + (bs + j) * nbdm + bs + i];
    // H_ij = (rho_ij + conj(rho_ji)) / 2, A_ij = (rho_ij - conj(rho_ji)) / (2i); exact for Hermitian rho
    const double2 hij = mk2(__dmul_rn(__dadd_rn(vij.x, vji.x), 0.5), __dmul_rn(__dsub_rn(vij.y, vji.y), 0.5));
    const double2 dif = mk2(__dsub_rn(vij.x, vji.x), __dadd_rn(vij.y, vji.y));  // rho_ij - conj(rho_ji)
    const double2 r1 = cmul_rn(d, hij);                       // conj(D) o H
    rh[ab] = A::from_double(r1.x);
    rh[ji] = A::from_double(r1.y);
    if (ws) {
      rh[NB2 + ab] = A::from_double(lin ? 0.0 : -r1.x);      // conj(D) o (1 - H) off the diagonal
      rh[NB2 + ji] = A::from_double(lin ? 0.0 : -r1.y);
    }
    if (dif.x != 0.0 || dif.y != 0.0) {  // the anti-Hermitian part is read only when hflag is raised
      atomicOr(hflag, 1u);
      const double2 aij = mk2(__dmul_rn(dif.y, 0.5), __dmul_rn(-dif.x, 0.5));
      const double2 r2 = cmul_rn(d, aij);                     // conj(D) o A
      ra[ab] = A::from_double(r2.x);
      ra[ji] = A::from_double(r2.y);
      if (ws) {
        ra[NB2 + ab] = A::from_double(lin ? 0.0 : -r2.x);    // conj(D) o (-A)
        ra[NB2 + ji] = A::from_double(lin ? 0.0 : -r2.y);
      }
    } else {
      ra[ab] = ra[ji] = A::from_double(0.0);
      if (ws) ra[NB2 + ab] = ra[NB2 + ji] = A::from_double(0.0);
    }
  }
}

// Prep of the tensor-core batched form: the same r coordinates and FP32 phases as k_prep_herm's
// FP32 tensor-core path, but one thread per (energy rank p, chunk of qc states) covering all nb^2
// elements, so that every lane of a warp runs the same code (the per-element form leaves the lanes of
// i > j idle and splits diagonal from off-diagonal work) and each state's window block is read and
// its coordinates written as whole vectors.
template <int NB>
__global__ void k_prep_tc(int nk, int nbdm, int bs, const double2* __restrict__ y, const double* __restrict__ ew,
                          const int* __restrict__ inv, TimeArg ta, int phase, float* __restrict__ rs,
                          unsigned int* __restrict__ hflag, const double* __restrict__ fref, int nrhs, int qc,
                          float2* __restrict__ ph) {
  constexpr int NB2 = NB * NB;
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= nk) return;
  const int q0 = blockIdx.y * qc, q1 = min(nrhs, q0 + qc);
  const size_t cstride = (size_t)nk * 2 * NB2;
  const size_t sstride = (size_t)nk * nbdm * nbdm;
  const int k = inv[p];
  float2 dc[NB2];  // conj(D) for i < j
#pragma unroll
  for (int e = 0; e < NB2; ++e) dc[e] = make_float2(1.f, 0.f);
  if (phase) {
    const double t = eval_time(ta);
#pragma unroll
    for (int i = 0; i < NB; ++i)
#pragma unroll
      for (int j = i + 1; j < NB; ++j) {
        const double x = (ew[k * NB + i] - ew[k * NB + j]) * t;
        const double xr = fma(-6.283185307179586, rint(x * 0.15915494309189535), x);
        float sn, cs;
        sincosf((float)xr, &sn, &cs);
        dc[i * NB + j] = make_float2(cs, -sn);
      }
  }
  if (ph && blockIdx.y == 0) {
#pragma unroll
    for (int i = 0; i < NB; ++i)
#pragma unroll
      for (int j = 0; j < NB; ++j) {
        const float2 d = i < j ? dc[i * NB + j] : (i > j ? dc[j * NB + i] : make_float2(1.f, 0.f));
        ph[(size_t)k * NB2 + i * NB + j] = i < j ? make_float2(d.x, -d.y) : d;  // D = conj(conj(D)), D_ji = conj(D_ij)
      }
  }
  double fi[NB];
#pragma unroll
  for (int i = 0; i < NB; ++i) fi[i] = fref ? fref[(size_t)k * NB + i] : 0.0;
  for (int q = q0; q < q1; ++q) {
    const double2* yk = y + (size_t)q * sstride + (size_t)k * nbdm * nbdm;
    double2 v[NB2];
#pragma unroll
    for (int i = 0; i < NB; ++i)
#pragma unroll
      for (int j = 0; j < NB; ++j) v[i * NB + j] = yk[(bs + i) * nbdm + bs + j];
    float r[NB2], a[NB2];
    bool nonherm = false;
#pragma unroll
    for (int i = 0; i < NB; ++i) {
      const double2 vii = v[i * NB + i];
      r[i * NB + i] = __double2float_rn(fref ? __dsub_rn(vii.x, fi[i]) : vii.x);
      a[i * NB + i] = __double2float_rn(vii.y);
      nonherm |= vii.y != 0.0;
    }
#pragma unroll
    for (int i = 0; i < NB; ++i)
#pragma unroll
      for (int j = i + 1; j < NB; ++j) {
        const double2 vij = v[i * NB + j], vji = v[j * NB + i];
        float2 hf = make_float2(0.5f * ((float)vij.x + (float)vji.x), 0.5f * ((float)vij.y - (float)vji.y));
        float2 af = make_float2(0.f, 0.f);
        if (vij.x != vji.x || vij.y != -vji.y) {  // not exactly Hermitian: the anti-Hermitian pass runs
          nonherm = true;
          const double2 hij = mk2(__dmul_rn(__dadd_rn(vij.x, vji.x), 0.5), __dmul_rn(__dsub_rn(vij.y, vji.y), 0.5));
          const double2 dif = mk2(__dsub_rn(vij.x, vji.x), __dadd_rn(vij.y, vji.y));
          hf = make_float2((float)hij.x, (float)hij.y);
          af = make_float2((float)__dmul_rn(dif.y, 0.5), (float)__dmul_rn(-dif.x, 0.5));
        }
        const float2 d = dc[i * NB + j];
        r[i * NB + j] = __fmaf_rn(d.x, hf.x, -d.y * hf.y);
        r[j * NB + i] = __fmaf_rn(d.x, hf.y, d.y * hf.x);
        a[i * NB + j] = __fmaf_rn(d.x, af.x, -d.y * af.y);
        a[j * NB + i] = __fmaf_rn(d.x, af.y, d.y * af.x);
      }
    if (nonherm) atomicOr(hflag, 1u);
    float4* rh = (float4*)(rs + (size_t)q * cstride + (size_t)p * 2 * NB2);
    float4* ra = (float4*)(rs + (size_t)(nrhs + q) * cstride + (size_t)p * 2 * NB2);
#pragma unroll
    for (int e = 0; e < NB2 / 4; ++e) {
      rh[e] = make_float4(r[4 * e], r[4 * e + 1], r[4 * e + 2], r[4 * e + 3]);
      ra[e] = make_float4(a[4 * e], a[4 * e + 1], a[4 * e + 2], a[4 * e + 3]);
    }
  }
}

// ---------------------------------------------------------------------------------------------
// The contraction. P2 is stored column-major, so both halves of a pair are consumed "line by
// line": a Q1 row a gives X'_k[a] and a Q2 column j gives Y'_k[j], while the reverse sums Y'_c
// (indexed by Q1's column) and X'_c (indexed by Q2's row) stay in registers with compile-time
// indices. G = nb^2 / 4 lanes share a pair (1 for nb = 2, 4 for nb = 4): lane (g, s) owns slot s of
// the row block (column W J + s, W = 32 / G) and the quarter [4g, 4g + 4) of every line, so each lane
// handles 4 elements per line and holds 4 coordinates and 8 reverse sums whatever nb is. A row
// block is consumed in chunks of LINES lines that stream through a per-warp ring of NST stages: the
// copy of chunk i + NST is issued as soon as chunk i has been read. Lane r holds the descriptor of
// the item's row block r (items have at most 32), so issuing a copy needs no memory access; the next
// row's coordinates are fetched one row block ahead. The forward partials of every 8 lines are
// reduced over the warp through a shared buffer and added with 16 FP64 atomics. Waits are bounded
// (dmd_tma.cuh); a timeout sets *errflag.
// ---------------------------------------------------------------------------------------------
// FA (forward atomics): each active lane adds its forward partials straight to the row's sums with
// FP64 reductions in L2 instead of reducing them over the warp through shared memory first; the
// per-warp reduction buffer is then not allocated. For the FP64 form, whose bound is the FP64 pipe,
// this moves the cross-lane additions (about one FP64 add per element per pair) off that pipe.
template <typename A, int NB, int LINES, int NST, int RW = 1, bool FA = false>
struct CbTmaSmem {
  static constexpr int NB2 = NB * NB, NB4 = NB2 * NB2;
  static constexpr int G = NB2 / 4, W = 32 / G;  // lanes per pair, slots (columns) per row block
  static constexpr int FL = 8, NV = 2 * FL * RW; // lines per forward flush, reals per flush (all RHS)
  static constexpr int CPM = NB2 / LINES;        // chunks per matrix
  static constexpr int CPR = 2 * CPM;            // chunks per row block
  // packed complex flush entries (one state, one lane per pair)
  static constexpr bool PR = A::kPackedRed && !FA && RW == 1 && G == 1;
  static constexpr size_t stage_bytes = (size_t)LINES * NB2 * W * sizeof(typename A::elem);
  static constexpr size_t red_bytes = FA ? 0 : PR ? (size_t)FL * 32 * 16 : (size_t)NV * 32 * sizeof(typename A::red_t);
  static constexpr size_t row_bytes = (size_t)4 * NB2 * RW * sizeof(typename A::relem);  // r_k, s_k, zeros
  static constexpr size_t warp_bytes = ((NST * stage_bytes + red_bytes + row_bytes + 8 * NST) + 127) / 128 * 128;
  static constexpr size_t cta_bytes = 4 * warp_bytes;
  static_assert(NB2 % 4 == 0 && (2 * NB2) % FL == 0 && FL % LINES == 0, "shape");
  static_assert(!FA || G == 1, "forward atomics: one lane per pair (nb = 2)");
};

// slot of (value v, lane j) in the per-warp reduction buffer: rows rotated by v so that the
// reducing lanes (one value each, all reading entry j of their row) hit distinct banks
__device__ __forceinline__ int rsw(int v, int j) { return v * 32 + ((j + v) & 31); }

// IMAG: the sums are multiplied by i before they are added (anti-Hermitian pass).
// Batched form (RW > 1 or nrhs > 1): nrhs states share P; a warp carries RW of them, so each
// staged element feeds RW products. Warp w of the grid takes RHS group w % ngroups of work item
// w / ngroups (the warps of a block share an item, so its P chunks come from HBM once and from L2
// for the others). Coordinates of state q start at rs + q * rstride, its sums at acc + q * astride.
template <typename A, int NB, int LINES, int NST, int MINB, bool IMAG, int RW = 1, bool FA = false>
__global__ void __launch_bounds__(128, MINB) k_pairs_herm(const WorkItem* __restrict__ items, int nitems,
                                                          const RowBlock* __restrict__ rbs,
                                                          const typename A::elem* __restrict__ P,
                                                          const typename A::relem* __restrict__ rs,
                                                          double* __restrict__ acc, int nk,
                                                          const unsigned int* __restrict__ gate,
                                                          unsigned int* __restrict__ errflag, int nrhs = 1,
                                                          size_t rstride = 0, size_t astride = 0) {
  typedef CbTmaSmem<A, NB, LINES, NST, RW, FA> S;
  constexpr int NB2 = S::NB2, NB4 = S::NB4, G = S::G, W = S::W, FL = S::FL, NV = S::NV;
  constexpr int CPM = S::CPM, CPR = S::CPR;
  constexpr size_t SE = S::stage_bytes / sizeof(typename A::elem);  // elements per stage
  constexpr unsigned FULL = 0xffffffffu;
  typedef typename A::elem E;
  typedef typename A::relem V;
  typedef typename A::acc Acc;
  typedef typename A::red_t R;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  if (gate && *gate == 0u) return;  // anti-Hermitian pass with nothing to do
  const int wib = threadIdx.x >> 5;
  const int lane = threadIdx.x & 31;
  const int ngroups = (nrhs + RW - 1) / RW;
  const int wg = blockIdx.x * 4 + wib;
  const int item = wg / ngroups;
  const int q0 = (wg % ngroups) * RW;  // first state of this warp
  if (item >= nitems) return;
  const int nq = nrhs - q0 < RW ? nrhs - q0 : RW;  // states carried (the last group may be short)
  const int qg = lane / W, sl = lane % W;          // quarter, slot
  const int q4 = 4 * qg;
  unsigned char* wbase = smem_raw + (size_t)wib * S::warp_bytes;
  E* const stage0 = (E*)wbase;
  R* const red = (R*)(wbase + NST * S::stage_bytes);                  // [NV][32]
  V* const rowv = (V*)(wbase + NST * S::stage_bytes + S::red_bytes);  // [RW][r_k, s_k], then zeros
  uint64_t* const bar = (uint64_t*)(wbase + NST * S::stage_bytes + S::red_bytes + S::row_bytes);
  const WorkItem w = items[item];
  const int nrb = w.rb1 - w.rb0;  // <= kMaxRowBlocksPerItem = 32
  RowBlock mine;                  // lane r: the item's row block r
  mine.row = 0;
  mine.mask = 0;
  mine.revmask = 0;
  mine.pair0 = 0;
  if (lane < nrb) mine = rbs[w.rb0 + lane];
  const int nch = CPR * nrb;
  if (lane == 0) {
#pragma unroll
    for (int s = 0; s < NST; ++s) mbar_init(&bar[s], 1);
    fence_mbar_init();
  }
  __syncwarp();
  const uint64_t pol = policy_evict_first();
  // chunk c of the item into stage c % NST; called by the whole warp, lane 0 issues
  auto issue = [&](int c) {
    const int rbi = c / CPR;
    const uint32_t p0 = __shfl_sync(FULL, mine.pair0, rbi);
    const uint32_t m = __shfl_sync(FULL, mine.mask, rbi);
    if (lane == 0) {
      const int q = c % CPR;
      const int n = __popc(m);
      const size_t off = (size_t)p0 * 2 * NB4 + ((size_t)(q / CPM) * NB4 + (size_t)(q % CPM) * LINES * NB2) * n;
      const uint32_t bytes = (uint32_t)(LINES * NB2 * n * sizeof(E));
      const int s = c % NST;
      mbar_arrive_expect_tx(&bar[s], bytes);
      bulk_g2s(stage0 + (size_t)s * SE, P + off, bytes, &bar[s], pol);
    }
  };
#pragma unroll
  for (int c = 0; c < NST; ++c)
    if (c < nch) issue(c);
  constexpr int RV = 2 * NB2 * RW;  // row coordinates of all carried states
  for (int i = lane; i < RV; i += 32) rowv[RV + i] = V();
  const int col = w.J * W + sl;
  const bool colok = col < nk;
  typename A::pcoord rc[4][RW], sc[4][RW];  // r_col, s_col on this lane's quarter, per state
#pragma unroll
  for (int u = 0; u < RW; ++u)
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const bool ok = colok && u < nq;
      const V* rq = rs + (size_t)(q0 + u) * rstride + (size_t)col * 2 * NB2;
      rc[i][u] = A::prep(ok ? rq[q4 + i] : V());
      sc[i][u] = A::prep(ok ? rq[NB2 + q4 + i] : V());
    }
  Acc rX[4][RW], rY[4][RW];
#pragma unroll
  for (int u = 0; u < RW; ++u)
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      A::zero(rX[i][u]);
      A::zero(rY[i][u]);
    }
  // coordinates of the first row: element i of state u at rowv[u * 2 NB2 + i]
  auto row_coord = [&](int row, int i) -> V {
    const int u = i / (2 * NB2), e = i % (2 * NB2);
    return u < nq ? rs[(size_t)(q0 + u) * rstride + (size_t)row * 2 * NB2 + e] : V();
  };
  constexpr int RPL = (RV + 31) / 32;  // row coordinates per lane
  V rnext[RPL];
  {
    const int r0 = __shfl_sync(FULL, mine.row, 0);
#pragma unroll
    for (int t = 0; t < RPL; ++t) {
      const int i = lane + 32 * t;
      rnext[t] = (i < RV && nrb > 0) ? row_coord(r0, i) : V();
    }
  }
  bool any_rev = false;
  int cfail = -1;
  const unsigned lt = (1u << sl) - 1u;
#pragma unroll 1
  for (int rbi = 0; rbi < nrb; ++rbi) {
    const int brow = __shfl_sync(FULL, mine.row, rbi);
    const unsigned bmask = __shfl_sync(FULL, mine.mask, rbi);
    const unsigned brev = __shfl_sync(FULL, mine.revmask, rbi);
    const int nrow = __shfl_sync(FULL, mine.row, rbi + 1 < nrb ? rbi + 1 : rbi);
    const bool active = (bmask >> sl) & 1u;
    // a lane whose pair has no reverse term reads zero row coordinates: its reverse sums receive
    // exact zeros and the inner loops carry no branch
    const bool rev = (brev >> sl) & 1u;
    any_rev |= rev;
    const int n = __popc(bmask);
    const int slot = __popc(bmask & lt);
    unsigned lm = 0;  // active lanes of the warp
#pragma unroll
    for (int gg = 0; gg < G; ++gg) lm |= bmask << (gg * W);
#pragma unroll
    for (int t = 0; t < RPL; ++t) {
      const int i = lane + 32 * t;
      if (i < RV) {
        rowv[i] = rnext[t];
        if (rbi + 1 < nrb) rnext[t] = row_coord(nrow, i);
      }
    }
    __syncwarp();
    const V* rv = rowv + (rev ? 0 : RV);
#pragma unroll 1
    for (int q = 0; q < CPR; ++q) {
      const int c = rbi * CPR + q;
      const int s = c % NST;
      if (!__all_sync(FULL, mbar_wait_bounded(&bar[s], (uint32_t)((c / NST) & 1), errflag))) {
        cfail = c;
        break;
      }
      const E* st = stage0 + (size_t)s * SE + slot;
      const int l0 = (q % CPM) * LINES;
      if (active) {
        if (q < CPM) {
          // Q1 rows a: X'_k[a] = sum_j Q1[a][j] r_c[j];  Y'_c[j] += s_k[a] conj(Q1[a][j])
#pragma unroll
          for (int r = 0; r < LINES; ++r) {
            const int a = l0 + r;
            Acc f[RW];
            typename A::pcoord_cx sa[RW];
#pragma unroll
            for (int u = 0; u < RW; ++u) sa[u] = A::prep_cx(rv[u * 2 * NB2 + NB2 + a]);
#pragma unroll
            for (int i = 0; i < 4; ++i) {
              const E p1 = st[(r * NB2 + q4 + i) * n];
#pragma unroll
              for (int u = 0; u < RW; ++u) {
                if (i == 0) A::mul(f[u], p1, rc[i][u]);
                else A::mac(f[u], p1, rc[i][u]);
                A::mac_cx(rY[i][u], p1, sa[u]);
              }
            }
            if constexpr (FA) {
              double* dst = acc + (size_t)brow * 4 * NB2 + 2 * (q * LINES + r);
#pragma unroll
              for (int u = 0; u < RW; ++u) {
                if (u < nq) {
                  atomicAdd(dst + (size_t)(q0 + u) * astride, IMAG ? -A::im_d(f[u]) : A::re_d(f[u]));
                  atomicAdd(dst + (size_t)(q0 + u) * astride + 1, IMAG ? A::re_d(f[u]) : A::im_d(f[u]));
                }
              }
            } else if constexpr (S::PR) {
              reinterpret_cast<float4*>(red)[rsw((q * LINES + r) % FL, lane)] = A::red_pack(f[0], IMAG);
            } else {
              const int v = 2 * ((q * LINES + r) % FL);
#pragma unroll
              for (int u = 0; u < RW; ++u) {
                red[rsw(v * RW + 2 * u, lane)] = IMAG ? A::red_neg(A::red_im(f[u])) : A::red_re(f[u]);
                red[rsw(v * RW + 2 * u + 1, lane)] = IMAG ? A::red_re(f[u]) : A::red_im(f[u]);
              }
            }
          }
        } else {
          // Q2 columns j: Y'_k[j] = sum_a Q2[a][j] s_c[a];  X'_c[a] += conj(Q2[a][j]) r_k[j]
#pragma unroll
          for (int r = 0; r < LINES; ++r) {
            const int j = l0 + r;
            Acc f[RW];
            typename A::pcoord_cx rj[RW];
#pragma unroll
            for (int u = 0; u < RW; ++u) rj[u] = A::prep_cx(rv[u * 2 * NB2 + j]);
#pragma unroll
            for (int i = 0; i < 4; ++i) {
              const E p2 = st[(r * NB2 + q4 + i) * n];
#pragma unroll
              for (int u = 0; u < RW; ++u) {
                if (i == 0) A::mul(f[u], p2, sc[i][u]);
                else A::mac(f[u], p2, sc[i][u]);
                A::mac_cx(rX[i][u], p2, rj[u]);
              }
            }
            if constexpr (FA) {
              double* dst = acc + (size_t)brow * 4 * NB2 + 2 * (q * LINES + r);
#pragma unroll
              for (int u = 0; u < RW; ++u) {
                if (u < nq) {
                  atomicAdd(dst + (size_t)(q0 + u) * astride, IMAG ? -A::im_d(f[u]) : A::re_d(f[u]));
                  atomicAdd(dst + (size_t)(q0 + u) * astride + 1, IMAG ? A::re_d(f[u]) : A::im_d(f[u]));
                }
              }
            } else if constexpr (S::PR) {
              reinterpret_cast<float4*>(red)[rsw((q * LINES + r) % FL, lane)] = A::red_pack(f[0], IMAG);
            } else {
              const int v = 2 * ((q * LINES + r) % FL);
#pragma unroll
              for (int u = 0; u < RW; ++u) {
                red[rsw(v * RW + 2 * u, lane)] = IMAG ? A::red_neg(A::red_im(f[u])) : A::red_re(f[u]);
                red[rsw(v * RW + 2 * u + 1, lane)] = IMAG ? A::red_re(f[u]) : A::red_im(f[u]);
              }
            }
          }
        }
      }
      // the stage is free once every lane has read it: order those reads before the next bulk copy
      // into it (generic -> async proxy), then refill it
      fence_proxy_async();
      __syncwarp();
      if (c + NST < nch) issue(c + NST);
      if constexpr (S::PR) {
        if (((q + 1) * LINES) % FL == 0) {
          // packed entries: lane (part, v) sums line v over the active lanes [8 part, 8 part + 8) (the
          // 8 lanes of a quarter warp read 8 lines of one source lane: distinct banks), the four parts
          // are added with two shuffles, and lanes 0-15 add line (lane & 7)'s real (part 0) or
          // imaginary (part 1) sum to the row
          const int L0 = (q + 1) * LINES - FL;
          const int v = lane & 7, part = lane >> 3;
          const float4* red4 = reinterpret_cast<const float4*>(red);
          float4 sum = make_float4(0.f, 0.f, 0.f, 0.f);
          unsigned m = (lm >> (part * 8)) & 0xffu;
          while (m) {
            const int jj = __ffs(m) - 1;
            m &= m - 1;
            A::red_add4(sum, red4[rsw(v, part * 8 + jj)]);
        }
#pragma unroll
        for (int mm = 8; mm < 32; mm <<= 1) {
          const float4 o = make_float4(__shfl_xor_sync(FULL, sum.x, mm), __shfl_xor_sync(FULL, sum.y, mm),
                                       __shfl_xor_sync(FULL, sum.z, mm), __shfl_xor_sync(FULL, sum.w, mm));
          A::red_add4(sum, o);
        }
        if (lane < 16)
          atomicAdd(acc + (size_t)q0 * astride + (size_t)brow * 4 * NB2 + 2 * L0 + 2 * v + part,
                    part == 0 ? (double)sum.x + (double)sum.z : (double)sum.y + (double)sum.w);
        __syncwarp();
        }
      } else if (!FA && ((q + 1) * LINES) % FL == 0) {
        // lines [L0, L0 + FL) of this row block are complete: reduce over the active lanes and add
        // to the row's sums (line L is real pair 2L, 2L + 1 of [X'(NB2) | Y'(NB2)]); buffer value
        // v * RW + 2u + ri holds line v / 2 (of the flush), part ri, state u
        const int L0 = (q + 1) * LINES - FL;
        constexpr int LPV = 32 / NV > 0 ? 32 / NV : 1;
#pragma unroll 1
        for (int v0 = 0; v0 < NV; v0 += 32 / LPV) {
          const int v = v0 + lane / LPV;
          const int part = lane % LPV;
          R sum = A::red_zero();
          if (v < NV) {
            const int span = 32 / LPV;
            unsigned m = (lm >> (part * span)) & (span == 32 ? 0xffffffffu : ((1u << span) - 1u));
            while (m) {
              const int jj = __ffs(m) - 1;
              m &= m - 1;
              A::red_add(sum, red[rsw(v, part * span + jj)]);
            }
          }
#pragma unroll
          for (int mm = 1; mm < LPV; mm <<= 1) A::red_add(sum, A::red_shfl_xor(sum, mm));
          if (v < NV && part == 0) {
            const int line2 = v / (2 * RW), u = (v / 2) % RW, ri = v & 1;
            if (u < nq)
              atomicAdd(acc + (size_t)(q0 + u) * astride + (size_t)brow * 4 * NB2 + 2 * L0 + 2 * line2 + ri,
                        A::red_to_double(sum));
          }
        }
        __syncwarp();
      }
    }
    if (cfail >= 0) break;
    // keep the low parts of the reverse sums small (each took NB2 products in this row block)
#pragma unroll
    for (int u = 0; u < RW; ++u)
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        A::renorm(rX[i][u]);
        A::renorm(rY[i][u]);
      }
  }
  if (cfail >= 0) {  // drain the copies still in flight (bounded), then leave
    if (lane == 0) {
      const int clast = (cfail + NST < nch ? cfail + NST : nch) - 1;
      for (int c = cfail; c <= clast; ++c) mbar_wait_bounded(&bar[c % NST], (uint32_t)((c / NST) & 1), nullptr, 1u << 16);
    }
    __syncwarp();
    return;
  }
  if (colok && any_rev) {
#pragma unroll
    for (int u = 0; u < RW; ++u) {
      if (u >= nq) break;
      double* dst = acc + (size_t)(q0 + u) * astride + (size_t)col * 4 * NB2;
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        const double xr = A::re_d(rX[i][u]), xi = A::im_d(rX[i][u]), yr = A::re_d(rY[i][u]), yi = A::im_d(rY[i][u]);
        atomicAdd(dst + 2 * (q4 + i), IMAG ? -xi : xr);
        atomicAdd(dst + 2 * (q4 + i) + 1, IMAG ? xr : xi);
        atomicAdd(dst + 2 * NB2 + 2 * (q4 + i), IMAG ? -yi : yr);
        atomicAdd(dst + 2 * NB2 + 2 * (q4 + i) + 1, IMAG ? yr : yi);
      }
    }
  }
}

}  // namespace dmd
