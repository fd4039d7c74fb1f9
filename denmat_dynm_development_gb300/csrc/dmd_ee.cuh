// e-e scattering operators rebuilt from the density matrix (eeMode = Pee_update, static screening):
// elecelec_model::calc_P (ElecElec_Model.h:186-262) for every stored k-pair, with the screened
// Coulomb interaction of coulomb_model::vq (Coulomb_Model.h:632-660) and the screening density of
// coulomb_model::init (Coulomb_Model.h:533-569).
//
// For a pair (k1, k2) and every k3 with k4 = k1 + k3 - k2 on the k-point set and some band
// combination inside the energy-conservation window, the Lindblad operator
//   A[(a,b),(c,d)] = delta(e1a - e2b + e3c - e4d) * mee,  mee = o12[a][b] o34[c][d]
//   (exchange: (o12[a][b] o34[c][d] - o14[a][d] o32[c][b]) / 2), o_ij = U_i^dag U_j, o12 and o14
//   times vq(k1 - k2), vq(k1 - k4)
// enters P1ee[(i1,i2),(i3,i4)] += sum_(i6,i8) (dm1_k3 A[(i1,i3)] dm_k4)[i6][i8] conj(A[(i2,i4)][i6,i8])
// and P2ee[(i1,i2),(i3,i4)] += sum_(i6,i8) (dm_k3 A[(i3,i1)] dm1_k4)[i6][i8] conj(A[(i4,i2)][i6,i8]),
// with A[(a,b)] read as an nb x nb matrix over (c, d); at set-up dm, dm1 are replaced by the
// occupations (calc_A1f / calc_A1fbar).
//
// GPU layout of the work: one warp per pair. Phase 1: the 32 lanes test 32 k3 at a time (k4 by
// integer mesh arithmetic and a dense mesh table, the energy window by every band combination in
// FP32 with a margin above its rounding) and append the candidates to a warp buffer. Phase 2: groups of G = 2 nb^2 lanes take one candidate each
// (4 groups for nb = 2, one for nb = 4); lane (w, r), r = (i1, i3), forms the real (w = 0) or
// imaginary (w = 1) part of the overlaps' entry r and half w of the columns of row r of A in shared
// memory, then its own A1rho (w = 0) or A1rhobar (w = 1) row, and accumulates P1ee or P2ee over
// (i2, i4) in registers. The groups' partial sums are added with shuffles at the end. The
// candidate search, the overlaps, delta and A are FP64; the two contractions (A1rho and the
// accumulation, 90 % of the multiply-adds) are FP64 for FP64 handles and double-float (FP32 pairs,
// ~2^-47 per product, renormalised after every work item) otherwise: GB300's FP32 pipes run them at
// several times the FP64 rate.
#pragma once
#include "dmd_common.cuh"
#include "dmd_kernels.cuh"
#include "dmd_pairs_cb.cuh"

namespace dmd {

enum { EE_UNSCREENED = 0, EE_DEBYE = 1, EE_BECHSTEDT = 2, EE_RPA = 3 };

// screening constants (Coulomb_Model.h:423-424, 555-569), computed on the device from nfree
struct EeScreen {
  double prefac_vq, prefac_vq_bare, qscr2_debye, fac0, fac2, fac4, nfree, pad;
};

struct EeArgs {
  int nk, npair, nbw;
  int kmesh[3];
  double GGT[9];
  double ethr, prefac_exp, prefac;   // energy window; -1/(4 degauss^2); prefac_gauss / nk_full (x2 with exchange)
  int formula, antisym;
  const int2* kk;                    // [npair] stored (k1, k2)
  const double* kvec;                // [nk][3] fractional
  const int4* kidx;                  // [nk] mesh indices (kIndexMap::ikvec3)
  const int* kmap;                   // [n0 n1 n2] mesh index -> k or -1
  const double2* U;                  // [nk][nbw][nb]
  const double* ew;                  // [nk][nb] window energies
  const float* ewf;                  // [nk][nb] window energies minus their minimum, FP32 (candidate test)
  float thr32;                       // ethr plus a margin above the FP32 rounding of that test
  const double2* dm;                 // [nk][nb^2] window density matrix (Schrodinger picture), or null
  const double2* dm1;                // [nk][nb^2] 1 - dm
  const float4* dmf;                 // the same as double-floats (re_h, im_h, re_l, im_l)
  const float4* dm1f;
  const double* f;                   // [nk][nb] occupations when dm is null
  const EeScreen* scr;
  const double* vqtab;               // [n0 n1 n2] static RPA vq by the q mesh index (EE_RPA)
  double2* Pee;                      // [npair][2][nb^4]: P1ee, P2ee (prefactor included)
  // plasmon-pole screening (dynamic): vq(q, w) per matrix element from A(q), E^2(q) by q mesh index
  int dynamic, two_freqs;
  double smearing;
  const double2* Aq;
  const double2* Eq2;
};

// wrap to [-0.5, 0.5) (comm/kmap.h:6-15) and |q|^2 in the reciprocal metric (comm/matrix3.h:119-121)
__device__ __forceinline__ double ee_q2(const EeArgs& a, double q0, double q1, double q2) {
  double v[3] = {q0, q1, q2};
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    v[d] -= floor(0.5 + v[d]);
    if (fabs(v[d] - 0.5) < 1e-6) v[d] = -0.5;
  }
  const double* m = a.GGT;
  return v[0] * v[0] * m[0] + v[1] * v[1] * m[4] + v[2] * v[2] * m[8] +
         2 * (v[0] * v[1] * m[1] + v[0] * v[2] * m[2] + v[1] * v[2] * m[5]);
}

// mesh index of u - v; both lie in [0, n), so the difference lies in (-n, n)
__device__ __forceinline__ size_t ee_qmesh(const int* kmesh, int4 u, int4 v) {
  int m0 = u.x - v.x, m1 = u.y - v.y, m2 = u.z - v.z;
  m0 += m0 < 0 ? kmesh[0] : 0;
  m1 += m1 < 0 ? kmesh[1] : 0;
  m2 += m2 < 0 ? kmesh[2] : 0;
  return ((size_t)m0 * kmesh[1] + m1) * kmesh[2] + m2;
}

// coulomb_model::vq, static branches (Coulomb_Model.h:632-666), q = k_i - k_j
__device__ __forceinline__ double ee_vq(const EeArgs& a, const EeScreen& s, int ki, int kj) {
  const double* x = a.kvec + 3 * ki;
  const double* y = a.kvec + 3 * kj;
  const double q2 = ee_q2(a, x[0] - y[0], x[1] - y[1], x[2] - y[2]);
  if (a.formula == EE_RPA) return q2 < 1e-20 ? 0.0 : a.vqtab[ee_qmesh(a.kmesh, a.kidx[ki], a.kidx[kj])];
  if (a.formula == EE_UNSCREENED) return q2 < 1e-20 ? 0.0 : s.prefac_vq / q2;
  if (a.formula == EE_DEBYE) return s.prefac_vq / (s.qscr2_debye + q2);
  if (q2 < 1e-20) return 0.0;
  const double epsq = 1 + 1. / (s.fac0 + s.fac2 * q2 + s.fac4 * q2 * q2);
  return s.prefac_vq_bare / epsq / q2;
}

// a / b as scalar.h computes it: complex(a.x b.x + a.y b.y, a.y b.x - a.x b.y) times 1 / b.norm()
__device__ __forceinline__ double2 ee_cdiv(double2 a, double2 b) {
  const double r = 1.0 / (b.x * b.x + b.y * b.y);
  return mk2((a.x * b.x + a.y * b.y) * r, (a.y * b.x - a.x * b.y) * r);
}

// coulomb_model::vq(q, w) with plasmon-pole screening (Coulomb_Model.h:659-687), q by its |q|^2 and
// mesh index: the static value at w = 0, else (prefac_vq + A / (cw^2 - E^2)) / |q|^2 with
// cw = |w| + i smearing, conjugated for w < 0
__device__ __forceinline__ double2 ee_vq_dyn(const EeArgs& a, const EeScreen& s, double q2, size_t m, double w) {
  if (q2 < 1e-20) return mk2(0, 0);
  if (w == 0) return mk2(a.vqtab[m], 0);
  const double cx = fabs(w), cy = a.smearing;
  const double2 E = a.Eq2[m];
  const double2 t = ee_cdiv(a.Aq[m], mk2(cx * cx - cy * cy - E.x, cy * cx + cx * cy - E.y));
  const double rq = 1.0 / q2;
  return mk2((t.x + s.prefac_vq) * rq, (w < 0 ? -t.y : t.y) * rq);
}

// the interaction factor of one matrix element (ElecElec_Model.h:96-110, 124-135): vq at the mean
// energy transfer, or with the two-frequency option sqrt(|vq(wa)| |vq(wb)|) cis(mean phase)
__device__ __forceinline__ double2 ee_vq_elem(const EeArgs& a, const EeScreen& s, double q2, size_t m, double wa,
                                              double wb, double wmean) {
  if (!a.two_freqs) return ee_vq_dyn(a, s, q2, m, wmean);
  const double2 va = ee_vq_dyn(a, s, q2, m, wa), vb = ee_vq_dyn(a, s, q2, m, wb);
  const double vabs = sqrt(sqrt(va.x * va.x + va.y * va.y) * sqrt(vb.x * vb.x + vb.y * vb.y));
  double sn, cs;
  sincos(0.5 * (atan2(va.y, va.x) + atan2(vb.y, vb.x)), &sn, &cs);
  return mk2(cs * vabs, sn * vabs);
}

// element (c, d) of U_ki^dag U_kj (elecelec_model::calc_ovlp, ElecElec_Model.h:72-80)
template <int NB>
__device__ __forceinline__ double2 ee_ovlp(const EeArgs& a, int ki, int kj, int c, int d) {
  const double2* ui = a.U + (size_t)ki * a.nbw * NB;
  const double2* uj = a.U + (size_t)kj * a.nbw * NB;
  double2 s = mk2(0, 0);
  for (int w = 0; w < a.nbw; ++w) s = cfma_conja(ui[w * NB + c], uj[w * NB + d], s);
  return s;
}

// one part of ee_ovlp: the real (part 0) or imaginary (part 1) FMA chain of cfma_conja, with the
// same operations in the same order, chosen by operand selection so that lanes with different
// parts do not diverge
template <int NB>
__device__ __forceinline__ double ee_ovlp_part(const EeArgs& a, int ki, int kj, int c, int d, int part) {
  const double2* ui = a.U + (size_t)ki * a.nbw * NB;
  const double2* uj = a.U + (size_t)kj * a.nbw * NB;
  double s = 0;
  for (int w = 0; w < a.nbw; ++w) {
    const double2 x = ui[w * NB + c], y = uj[w * NB + d];
    // real: x.x y.x + (x.y y.y + s); imaginary: x.x y.y + (-x.y y.x + s)
    s = fma(x.x, part ? y.y : y.x, fma(part ? -x.y : x.y, part ? y.x : y.y, s));
  }
  return s;
}

// static RPA screening (Coulomb_Model.h:690-736): one thread per ordered pair (i, j) of k-points adds
// sum_(b1,b2) dfde |<i b1|j b2>|^2 to the accumulator of the mesh index of q = k_i - k_j (FP64
// atomics), with dfde = (f_j - f_i) / (e_i - e_j), or (1 - f) f / T at degenerate energies
// With eppa > 0 (Godby-Needs plasmon pole, Coulomb_Model.h:794-819) the sums at w = i eppa as well:
// dfde = (f_j - f_i) / (e_i - e_j - i eppa) into qacc1 (complex).
template <int NB>
__global__ void k_ee_rpa_sum(EeArgs a, double T, const double* __restrict__ f, double* __restrict__ qacc,
                             unsigned int* __restrict__ qhit, double eppa = 0.0, double* __restrict__ qacc1 = nullptr) {
  const long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (idx >= (long long)a.nk * a.nk) return;
  const int i = (int)(idx / a.nk), j = (int)(idx % a.nk);
  const int4 vi = a.kidx[i], vj = a.kidx[j];
  // the k-point of this mesh index as the table keeps it (a duplicate index is served by its first k)
  if (a.kmap[((size_t)vj.x * a.kmesh[1] + vj.y) * a.kmesh[2] + vj.z] != j) return;
  double g = 0;
  double2 g1 = mk2(0, 0);
#pragma unroll
  for (int b1 = 0; b1 < NB; ++b1)
#pragma unroll
    for (int b2 = 0; b2 < NB; ++b2) {
      const double de = a.ew[(size_t)i * NB + b1] - a.ew[(size_t)j * NB + b2];
      double dfde;
      if (fabs(de) < 1e-8) {
        const double favg = 0.5 * (f[(size_t)i * NB + b1] + f[(size_t)j * NB + b2]);
        dfde = (1 - favg) * favg / T;
      } else {
        dfde = (f[(size_t)j * NB + b2] - f[(size_t)i * NB + b1]) / de;
      }
      const double2 o = ee_ovlp<NB>(a, i, j, b1, b2);
      const double n2 = o.x * o.x + o.y * o.y;
      g += dfde * n2;
      if (qacc1) {
        const double2 d1 = ee_cdiv(mk2(f[(size_t)j * NB + b2] - f[(size_t)i * NB + b1], 0), mk2(de, -eppa));
        g1.x += d1.x * n2;
        g1.y += d1.y * n2;
      }
    }
  const size_t m = ee_qmesh(a.kmesh, vi, vj);
  atomicAdd(&qacc[m], g);
  if (qacc1) {
    atomicAdd(&qacc1[2 * m], g1.x);
    atomicAdd(&qacc1[2 * m + 1], g1.y);
  }
  qhit[m] = 1u;
}

// vq = prefac_vq / (|q|^2 + qscr2) for every q mesh index that occurs (Coulomb_Model.h:819-826);
// |q|^2 from the mesh index wrapped to [-0.5, 0.5)
// With ppa (Aq set): the plasmon-pole terms of calc_vq_RPA (Coulomb_Model.h:855-874), eps^-1(w) =
// 1 + A / (w^2 - E^2): Hybertsen-Louie (qacc1 null) A = prefac_vq wp2, E^2 = wp2 (1 + |q|^2 / qscr2);
// Godby-Needs from eps^-1 at 0 and at i eppa: E^2 = wp2 (1 - epspinv) / (epspinv - eps0inv),
// A = prefac_vq (1 - eps0inv) E^2; wp2 = eppa^2, zero at Gamma.
__global__ void k_ee_rpa_table(EeArgs a, double prefac_vq, double nk_full, const double* __restrict__ qacc,
                               const unsigned int* __restrict__ qhit, double* __restrict__ vqtab,
                               double eppa = 0.0, const double* __restrict__ qacc1 = nullptr,
                               double2* __restrict__ Aq = nullptr, double2* __restrict__ Eq2 = nullptr) {
  const size_t n = (size_t)a.kmesh[0] * a.kmesh[1] * a.kmesh[2];
  const size_t m = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (m >= n) return;
  if (Aq) {
    Aq[m] = mk2(0, 0);
    Eq2[m] = mk2(0, 0);
  }
  if (!qhit[m]) {
    vqtab[m] = 0.0;
    return;
  }
  const int m2 = (int)(m % a.kmesh[2]), m1 = (int)((m / a.kmesh[2]) % a.kmesh[1]), m0 = (int)(m / ((size_t)a.kmesh[1] * a.kmesh[2]));
  const double q2 = ee_q2(a, (double)m0 / a.kmesh[0], (double)m1 / a.kmesh[1], (double)m2 / a.kmesh[2]);
  const double qs = prefac_vq / nk_full * qacc[m];
  vqtab[m] = q2 < 1e-20 ? 0.0 : prefac_vq / (q2 + qs);
  if (!Aq || q2 < 1e-20) return;
  const double wp2 = eppa * eppa;
  if (!qacc1) {  // Hybertsen-Louie
    const double2 t = ee_cdiv(mk2(q2, 0), mk2(qs, 0));
    Aq[m] = mk2(prefac_vq * wp2, 0);
    Eq2[m] = mk2((t.x + 1) * wp2, t.y * wp2);
  } else {  // Godby-Needs
    const double sc = prefac_vq / nk_full, rq = 1.0 / q2;
    const double2 qs1 = mk2(sc * qacc1[2 * m], sc * qacc1[2 * m + 1]);
    const double2 e0 = ee_cdiv(mk2(1, 0), mk2(qs * rq + 1, 0));
    const double2 ep = ee_cdiv(mk2(1, 0), mk2(qs1.x * rq + 1, qs1.y * rq));
    const double2 E = ee_cdiv(mk2((-ep.x + 1) * wp2, -ep.y * wp2), mk2(ep.x - e0.x, ep.y - e0.y));
    const double2 c = mk2((-e0.x + 1) * prefac_vq, -e0.y * prefac_vq);
    Eq2[m] = E;
    Aq[m] = mk2(c.x * E.x - c.y * E.y, c.x * E.y + c.y * E.x);
  }
}

// the window density matrix in the Schrodinger picture and 1 - rho from the state y (one thread per
// (k, i, j) of the window): electronphonon::reset_scatt's window copy (ElectronPhonon.cpp:19-28)
// and add_scatt_contrib's conversion (ElectronPhonon.cpp:56-66)
__device__ __forceinline__ float4 split_dfc(double2 v) {  // (re_h, im_h, re_l, im_l)
  const float2 a = split_df1(v.x), b = split_df1(v.y);
  return make_float4(a.x, b.x, a.y, b.y);
}

template <int NB>
__global__ void k_ee_dm(int nk, int nbdm, int bs, const double2* __restrict__ y, const double* __restrict__ ew,
                        TimeArg ta, int interaction, double2* __restrict__ dm, double2* __restrict__ dm1,
                        float4* __restrict__ dmf, float4* __restrict__ dm1f) {
  constexpr int NB2 = NB * NB;
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= nk * NB2) return;
  const int k = idx / NB2, e = idx % NB2, i = e / NB, j = e % NB;
  const int lo_i = i < j ? i : j, hi_j = i < j ? j : i;
  double2 v = y[(size_t)k * nbdm * nbdm + (bs + lo_i) * nbdm + bs + hi_j];  // the upper element
  if (interaction && lo_i != hi_j) {
    const double t = eval_time(ta);
    const double* ek = ew + (size_t)k * NB;
    v = cmul_rn(v, ccis((ek[hi_j] - ek[lo_i]) * t));
  }
  double2 d, d1;
  if (i == j) {  // zhemm reads the diagonal as real (BLAS ZHEMM)
    d = mk2(v.x, 0.0);
    d1 = mk2(1.0 - v.x, 0.0);
  } else {
    d = i < j ? v : cconj(v);  // lower = conj(upper)
    d1 = mk2(-d.x, -d.y);
  }
  dm[idx] = d;
  dm1[idx] = d1;
  dmf[idx] = split_dfc(d);
  dm1f[idx] = split_dfc(d1);
}

// 1/n! for n = 8 .. 0 as double-floats (hi, lo)
#define EE_DF_CONST(v) {(float)(v), (float)((v) - (double)(float)(v))}
__constant__ float2 c_ee_inv_fact[9] = {
    EE_DF_CONST(1.0 / 40320.0), EE_DF_CONST(1.0 / 5040.0), EE_DF_CONST(1.0 / 720.0),
    EE_DF_CONST(1.0 / 120.0),   EE_DF_CONST(1.0 / 24.0),   EE_DF_CONST(1.0 / 6.0),
    EE_DF_CONST(0.5),           EE_DF_CONST(1.0),          EE_DF_CONST(1.0)};
#undef EE_DF_CONST

// exp(x) for x <= 0 as a double-float: Cody-Waite reduction x = k ln2 + r in FP64 (ln2 in two
// parts), |r| <= ln2/2, then exp(r) from its Taylor series to degree 12 by Horner's rule, the terms
// of degree 12 .. 9 in FP32 and the rest in double-float (truncation and FP32 rounding together
// below 2.5e-16 relative), and the scaling by 2^k. The bound holds for x >= -55: the low part lies
// up to ~2^-50 below the high part, and once 2^k scales it under FP32's smallest normal (k below
// about -80) it rounds to the subnormal grid, whose spacing 2^-149 is then no longer negligible
// against the result. Below x = -55 the FP64 value is split instead.
// The two parts of ln2 are the published split of fdlibm's e_exp.c (ln2HI[0], ln2LO[0], Sun
// Microsystems, 1993): a 32-bit high part whose products with integers k are exact, and the rest.
__device__ __forceinline__ float2 df_exp_neg(double x) {
  if (x < -55.0) return split_df1(exp(x));
  const double k = rint(x * 1.4426950408889634);
  double r = fma(-k, 6.93147180369123816490e-01, x);  // ln2 high part (trailing bits zero)
  r = fma(-k, 1.90821492927058770002e-10, r);         // ln2 - high part
  const float2 rr = split_df1(r);
  // the terms of degree 12 .. 9 in FP32: their sum is below 2.8e-6 r^9 and r^9 below 7.3e-5, so its
  // FP32 rounding stays under 1e-16 of the result
  float ph = 1.0f / 479001600.0f, pl = 0.f;
  ph = fmaf(ph, rr.x, 1.0f / 39916800.0f);
  ph = fmaf(ph, rr.x, 1.0f / 3628800.0f);
  ph = fmaf(ph, rr.x, 1.0f / 362880.0f);
  // the terms of degree 8 .. 0 by Horner's rule in double-float; the loop stays rolled (with the
  // coefficients in constant memory) to keep the kernel's code within the instruction cache
#pragma unroll 1
  for (int n = 0; n < 9; ++n) {
    float h, l;
    df_mul(h, l, ph, pl, rr.x, rr.y);
    df_renorm(h, l);
    const float2 cn = c_ee_inv_fact[n];
    df_add(h, l, cn.x, cn.y);
    ph = h;
    pl = l;
  }
  df_renorm(ph, pl);
  const int ki = (int)k;
  return make_float2(ldexpf(ph, ki), ldexpf(pl, ki));
}

// complex arithmetic of the two contractions: FP64, or double-float on the FP32 pipes
struct EeF64 {
  static constexpr bool kDF = false;
  typedef double2 c;
  static __device__ __forceinline__ c zero() { return mk2(0, 0); }
  static __device__ __forceinline__ c from(double2 v) { return v; }
  static __device__ __forceinline__ void set_part(c& dst, int part, double v) {  // from(), one part
    reinterpret_cast<double*>(&dst)[part] = v;
  }
  static __device__ __forceinline__ c load(const double2* d, const float4*, size_t i) { return d[i]; }
  static __device__ __forceinline__ void mac(c& acc, c x, c y) { acc = cfma(x, y, acc); }  // acc += x y
  static __device__ __forceinline__ void mac_conj(c& acc, c x, c y) {                      // acc += x conj(y)
    acc = mk2(fma(x.x, y.x, fma(x.y, y.y, acc.x)), fma(x.y, y.x, fma(-x.x, y.y, acc.y)));
  }
  static __device__ __forceinline__ c scale(c x, double s) { return mk2(x.x * s, x.y * s); }
  static __device__ __forceinline__ void renorm(c&) {}
  static __device__ __forceinline__ double2 value(c v) { return v; }
};

// Double-float complex arithmetic with the real and imaginary halves as FP32x2 pairs
// (re_h, im_h, re_l, im_l), each step one packed instruction (ArithDF): a complex product is two
// packed error-free multiply-adds, x y = y o (Re x, Re x) + (-Im y, Re y) o (Im x, Im x) and
// x conj(y) = x o (Re y, Re y) + (Im x, -Re x) o (Im y, Im y).
struct EeDF {
  static constexpr bool kDF = true;
  typedef float4 c;  // (re_h, im_h, re_l, im_l)
  typedef ArithDF::acc A;
  static __device__ __forceinline__ A un(const c& v) { return A{make_float2(v.x, v.y), make_float2(v.z, v.w)}; }
  static __device__ __forceinline__ c pk(const A& a) { return make_float4(a.h.x, a.h.y, a.l.x, a.l.y); }
  static __device__ __forceinline__ float4 bre(const c& v) { return make_float4(v.x, v.x, v.z, v.z); }
  static __device__ __forceinline__ float4 bim(const c& v) { return make_float4(v.y, v.y, v.w, v.w); }
  static __device__ __forceinline__ c zero() { return make_float4(0.f, 0.f, 0.f, 0.f); }
  static __device__ __forceinline__ c from(double2 v) { return split_dfc(v); }
  static __device__ __forceinline__ void set_part(c& dst, int part, double v) {  // from(), one part
    const float2 f = split_df1(v);
    reinterpret_cast<float*>(&dst)[part] = f.x;
    reinterpret_cast<float*>(&dst)[2 + part] = f.y;
  }
  static __device__ __forceinline__ c load(const double2*, const float4* f, size_t i) { return f[i]; }
  static __device__ __forceinline__ void mac(c& a, c x, c y) {  // a += x y
    A t = un(a);
    ArithDF::pmac(t, y, bre(x));
    ArithDF::pmac(t, make_float4(-y.y, y.x, -y.w, y.z), bim(x));
    a = pk(t);
  }
  static __device__ __forceinline__ void mac_conj(c& a, c x, c y) {  // a += x conj(y)
    A t = un(a);
    ArithDF::pmac(t, x, bre(y));
    ArithDF::pmac(t, make_float4(x.y, -x.x, x.w, -x.z), bim(y));
    a = pk(t);
  }
  static __device__ __forceinline__ c scale(c x, double s) {
    const float2 v = split_df1(s);
    A r;
    ArithDF::mul(r, x, make_float4(v.x, v.x, v.y, v.y));
    return pk(r);
  }
  static __device__ __forceinline__ void renorm(c& a) {
    A t = un(a);
    ArithDF::renorm(t);
    a = pk(t);
  }
  static __device__ __forceinline__ double2 value(c v) { return mk2((double)v.x + (double)v.z, (double)v.y + (double)v.w); }
  static __device__ __forceinline__ c mul(c x, c y) {  // x y
    A r;
    ArithDF::mul(r, y, bre(x));
    ArithDF::pmac(r, make_float4(-y.y, y.x, -y.w, y.z), bim(x));
    ArithDF::renorm(r);
    return pk(r);
  }
  static __device__ __forceinline__ c scale_df(c x, float2 s) {
    A r;
    ArithDF::mul(r, x, make_float4(s.x, s.x, s.y, s.y));
    ArithDF::renorm(r);
    return pk(r);
  }
  // a += b (double-float, per half)
  static __device__ __forceinline__ void add(c& a, const c& b) { ArithDF::red_add4(a, b); }
};

// screening density and constants (one block): with update, nfree = sum over k and window bands of
// the electron (or, below nv, hole) occupations / (nk_full cell_size) (Coulomb_Model.h:533-553)
__global__ void k_ee_screen(int nk, int nb, int nv, const double2* __restrict__ dm, int update, double nfree0,
                            double nk_full, double cell_size, double eps, double T, double meff,
                            EeScreen* __restrict__ out) {
  __shared__ double part[256];
  double n = 0;
  if (update)
    for (int i = threadIdx.x; i < nk * nb; i += blockDim.x) {
      const int k = i / nb, b = i % nb;
      const double ft = dm[(size_t)k * nb * nb + b * nb + b].x;
      n += b < nv ? 1 - ft : ft;
    }
  part[threadIdx.x] = n;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if ((int)threadIdx.x < s) part[threadIdx.x] += part[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    const double nf = update ? part[0] / (nk_full * cell_size) : nfree0;
    EeScreen c;
    c.prefac_vq = 4 * M_PI / eps / cell_size;
    c.prefac_vq_bare = 4 * M_PI / cell_size;
    const double kF = pow(3 * M_PI * M_PI * nf, 1. / 3.);
    const double kF2 = kF * kF;
    const double EF = kF2 / 2. / meff;
    const double qTF2 = 6 * M_PI * nf / eps / EF;
    c.fac0 = 1. / (eps - 1);
    c.fac2 = 1. / qTF2;
    c.fac4 = 3. / 4. / kF2 / qTF2;
    c.qscr2_debye = 4 * M_PI * nf / eps / T;
    c.nfree = nf;
    c.pad = 0;
    *out = c;
  }
}

template <int NB, typename V>
struct EeSmem {
  static constexpr int NB2 = NB * NB, NB4 = NB2 * NB2, G = 2 * NB2, NG = 32 / G;
  typename V::c o12[NB2];  // the overlaps in the contraction's arithmetic
  typename V::c o34[NG][NB2], o14[NG][NB2], o32[NG][NB2];
  typename V::c A[NG][NB4];
  int2 cand[64];
};

// warps (pairs) per CTA: nb = 4 keeps 2 so that the per-lane scratch fits the static shared memory
__host__ __device__ constexpr int ee_warps_per_cta(int nb) { return nb == 4 ? 2 : 4; }

// DYN: plasmon-pole screening (a.dynamic); a separate instantiation so that the static kernel keeps
// its registers and occupancy
template <int NB, typename V = EeF64, bool DYN = false>
__global__ void __launch_bounds__(32 * ee_warps_per_cta(NB), (NB == 2 && V::kDF) ? 7 : 1) k_ee_pairs(EeArgs a) {
  typedef EeSmem<NB, V> S;
  typedef typename V::c C;
  constexpr int WPC = ee_warps_per_cta(NB);
  constexpr int NB2 = S::NB2, NB4 = S::NB4, G = S::G, NG = S::NG;
  __shared__ S smem_all[WPC];
  __shared__ typename V::c scratch[NB == 4 ? WPC : 1][NB == 4 ? 32 : 1][NB == 4 ? 2 * NB * NB : 1];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  S& sm = smem_all[warp];
  const int p = blockIdx.x * WPC + warp;
  if (p >= a.npair) return;
  const int k1 = a.kk[p].x, k2 = a.kk[p].y;
  const unsigned FULL = 0xffffffffu;
  const int grp = lane / G, role = lane % G, w = role / NB2, r = role % NB2, i1 = r / NB, i3 = r % NB;
  double2* out = a.Pee + (size_t)p * 2 * NB4;
  if (k1 == k2 && !a.antisym) {  // ElecElec_Model.h:191-194
    for (int e = lane; e < 2 * NB4; e += 32) out[e] = mk2(0, 0);
    return;
  }
  const EeScreen scr = *a.scr;
  // plasmon-pole screening: the overlaps stay unscaled and each matrix element takes vq(q, w) (its
  // |q|^2 and mesh index for q = k1 - k2 here, k1 - k4 per candidate)
  const double q2_12 = DYN ? ee_q2(a, a.kvec[3 * k1] - a.kvec[3 * k2], a.kvec[3 * k1 + 1] - a.kvec[3 * k2 + 1],
                                         a.kvec[3 * k1 + 2] - a.kvec[3 * k2 + 2])
                                 : 0.0;
  const size_t m_12 = DYN ? ee_qmesh(a.kmesh, a.kidx[k1], a.kidx[k2]) : 0;
  if (lane < NB2) {  // o12 = vq(k1 - k2) U_k1^dag U_k2
    const double vq = DYN ? 1.0 : ee_vq(a, scr, k1, k2);
    const double2 o = ee_ovlp<NB>(a, k1, k2, lane / NB, lane % NB);
    sm.o12[lane] = V::from(mk2(vq * o.x, vq * o.y));
  }
  C acc[NB2];
#pragma unroll
  for (int e = 0; e < NB2; ++e) acc[e] = V::zero();
  const int4 i1v = a.kidx[k1], i2v = a.kidx[k2];
  float x12[NB2];  // e1a - e2b of this pair for the FP32 candidate test
#pragma unroll
  for (int i = 0; i < NB; ++i)
#pragma unroll
    for (int j = 0; j < NB; ++j) x12[i * NB + j] = a.ewf[(size_t)k1 * NB + i] - a.ewf[(size_t)k2 * NB + j];
  const double* e1 = a.ew + (size_t)k1 * NB;
  const double* e2 = a.ew + (size_t)k2 * NB;
  int ncand = 0;
  for (int c0 = 0; c0 < a.nk; c0 += 32) {
    // phase 1: candidates k3 of this chunk
    const int k3 = c0 + lane;
    int k4 = -1;
    if (k3 < a.nk && !(a.antisym && k1 == k2 && k2 == k3)) {
      const int4 i3v = a.kidx[k3];
      // the mesh indices lie in [0, n), so i1 + i3 - i2 lies in (-n, 2n): one fold per axis
      int m0 = i1v.x + i3v.x - i2v.x, m1 = i1v.y + i3v.y - i2v.y, m2 = i1v.z + i3v.z - i2v.z;
      m0 += m0 < 0 ? a.kmesh[0] : (m0 >= a.kmesh[0] ? -a.kmesh[0] : 0);
      m1 += m1 < 0 ? a.kmesh[1] : (m1 >= a.kmesh[1] ? -a.kmesh[1] : 0);
      m2 += m2 < 0 ? a.kmesh[2] : (m2 >= a.kmesh[2] ? -a.kmesh[2] : 0);
      k4 = a.kmap[((size_t)m0 * a.kmesh[1] + m1) * a.kmesh[2] + m2];
      if (k4 >= 0) {  // some band combination inside the window, with a margin (exact FP64 test in phase 2)
        bool hit = false;
#pragma unroll
        for (int c = 0; c < NB; ++c)
#pragma unroll
          for (int d = 0; d < NB; ++d) {
            const float y = a.ewf[(size_t)k3 * NB + c] - a.ewf[(size_t)k4 * NB + d];
#pragma unroll
            for (int q = 0; q < NB2; ++q) hit |= fabsf(x12[q] + y) < a.thr32;
          }
        if (!hit) k4 = -1;
      }
    }
    const unsigned ball = __ballot_sync(FULL, k4 >= 0);
    if (k4 >= 0) sm.cand[ncand + __popc(ball & ((1u << lane) - 1))] = make_int2(k3, k4);
    ncand += __popc(ball);
    __syncwarp();
    const bool last = c0 + 32 >= a.nk;
    if (ncand < 32 && !last) continue;
    // phase 2: process min(ncand, 32) candidates (all of them after the last chunk)
    const int take = last ? ncand : 32;
    for (int s0 = 0; s0 < take; s0 += NG) {
      const int s = s0 + grp;
      const bool act = s < take;
      int ka = 0, kb = 0;
      if (act) {
        ka = sm.cand[s].x;
        kb = sm.cand[s].y;
        // overlaps of this candidate: lane (w, r) forms the real (w = 0) or imaginary (w = 1) part of
        // entry r of o34 (and of o14, o32 with the exchange term)
        const int c = r / NB, d = r % NB;
        V::set_part(sm.o34[grp][r], w, ee_ovlp_part<NB>(a, ka, kb, c, d, w));
        if (a.antisym) {
          const double vq = DYN ? 1.0 : ee_vq(a, scr, k1, kb);
          V::set_part(sm.o14[grp][r], w, vq * ee_ovlp_part<NB>(a, k1, kb, c, d, w));
          V::set_part(sm.o32[grp][r], w, ee_ovlp_part<NB>(a, ka, k2, c, d, w));
        }
      }
      __syncwarp();
      if (act) {  // row r = (i1, i3) of A, columns cd of half w (calc_delta, calc_mee[_ex], calc_A)
        const double* e3 = a.ew + (size_t)ka * NB;
        const double* e4 = a.ew + (size_t)kb * NB;
        const C m12 = sm.o12[i1 * NB + i3];
        double q2_14 = 0.0;
        size_t m_14 = 0;
        if (DYN && a.antisym) {
          q2_14 = ee_q2(a, a.kvec[3 * k1] - a.kvec[3 * kb], a.kvec[3 * k1 + 1] - a.kvec[3 * kb + 1],
                        a.kvec[3 * k1 + 2] - a.kvec[3 * kb + 2]);
          m_14 = ee_qmesh(a.kmesh, a.kidx[k1], a.kidx[kb]);
        }
        constexpr int HALF = NB2 / 2;  // both halves of the group share the row's elements
#pragma unroll 1
        for (int h = 0; h < HALF; ++h) {  // rolled: one copy of the exp in the code
          const int cd = w * HALF + h, c = cd / NB, d = cd % NB;
          const double de = e1[i1] - e2[i3] + e3[c] - e4[d];  // the window test stays FP64
          C v = V::zero();
          if (fabs(de) < a.ethr) {
            // plasmon pole: mee *= vq(k1 - k2, w) (calc_mee) and, with the exchange term, mee *=
            // vq(k1 - k4, w_ex) (calc_mee_ex scales the direct term), the exchange term unscreened
            double2 f12 = mk2(1, 0), f14 = mk2(1, 0);
            if constexpr (DYN) {
              f12 = ee_vq_elem(a, scr, q2_12, m_12, e1[i1] - e2[i3], e4[d] - e3[c], 0.5 * (e1[i1] - e2[i3] + e4[d] - e3[c]));
              if (a.antisym)
                f14 = ee_vq_elem(a, scr, q2_14, m_14, e1[i1] - e4[d], e2[i3] - e3[c], 0.5 * (e1[i1] - e4[d] + e2[i3] - e3[c]));
            }
            if constexpr (V::kDF) {
              C mee = V::mul(m12, sm.o34[grp][cd]);
              if constexpr (DYN) {
                mee = V::mul(mee, V::from(f12));
                if (a.antisym) mee = V::mul(mee, V::from(f14));
              }
              if (a.antisym) {
                const C mex = V::mul(sm.o14[grp][i1 * NB + d], sm.o32[grp][c * NB + i3]);
                mee = make_float4(0.5f * mee.x, 0.5f * mee.y, 0.5f * mee.z, 0.5f * mee.w);  // exact halves
                V::add(mee, make_float4(-0.5f * mex.x, -0.5f * mex.y, -0.5f * mex.z, -0.5f * mex.w));
              }
              v = V::scale_df(mee, df_exp_neg(a.prefac_exp * (de * de)));
            } else {
              double2 mee = cmul_rn(m12, sm.o34[grp][cd]);
              if constexpr (DYN) {
                mee = cmul_rn(mee, f12);
                if (a.antisym) mee = cmul_rn(mee, f14);
              }
              if (a.antisym) {
                const double2 mex = cmul_rn(sm.o14[grp][i1 * NB + d], sm.o32[grp][c * NB + i3]);
                mee = mk2(-0.5 * mex.x + 0.5 * mee.x, -0.5 * mex.y + 0.5 * mee.y);
              }
              v = cscale_rn(exp(a.prefac_exp * (de * de)), mee);
            }
          }
          sm.A[grp][r * NB2 + cd] = v;
        }
      }
      __syncwarp();
      if (act) {
        // X = dm1_k3 A[(i1,i3)] dm_k4 (w = 0) or dm_k3 A[(i3,i1)] dm1_k4 (w = 1)
        const C* Ar = &sm.A[grp][(w == 0 ? r : i3 * NB + i1) * NB2];
        const size_t lo = (size_t)ka * NB2, ro = (size_t)kb * NB2;
        const double2* Ld = w == 0 ? a.dm1 : a.dm;
        const float4* Lf = w == 0 ? a.dm1f : a.dmf;
        const double2* Rd = w == 0 ? a.dm : a.dm1;
        const float4* Rf = w == 0 ? a.dmf : a.dm1f;
        if constexpr (NB == 2) {
          C X[NB2];
          if (a.dm) {
            C T[NB2];
#pragma unroll
            for (int i = 0; i < NB; ++i)
#pragma unroll
              for (int j = 0; j < NB; ++j) {
                C t = V::zero();
#pragma unroll
                for (int m = 0; m < NB; ++m) V::mac(t, Ar[i * NB + m], V::load(Rd, Rf, ro + m * NB + j));
                T[i * NB + j] = t;
              }
#pragma unroll
            for (int i = 0; i < NB; ++i)
#pragma unroll
              for (int j = 0; j < NB; ++j) {
                C t = V::zero();
#pragma unroll
                for (int m = 0; m < NB; ++m) V::mac(t, V::load(Ld, Lf, lo + i * NB + m), T[m * NB + j]);
                X[i * NB + j] = t;
              }
          } else {
            const double* f3 = a.f + (size_t)ka * NB;
            const double* f4 = a.f + (size_t)kb * NB;
#pragma unroll
            for (int i = 0; i < NB; ++i)
#pragma unroll
              for (int j = 0; j < NB; ++j) {
                const double sl = w == 0 ? 1 - f3[i] : f3[i], sr = w == 0 ? f4[j] : 1 - f4[j];
                X[i * NB + j] = V::scale(V::scale(Ar[i * NB + j], sl), sr);
              }
          }
          // acc[(i2,i4)] += sum_(i6,i8) X[i6,i8] conj(A[(i2,i4) or (i4,i2)][i6,i8])
#pragma unroll
          for (int i2 = 0; i2 < NB; ++i2)
#pragma unroll
            for (int i4 = 0; i4 < NB; ++i4) {
              const C* B = &sm.A[grp][(w == 0 ? i2 * NB + i4 : i4 * NB + i2) * NB2];
              C t = acc[i2 * NB + i4];
#pragma unroll
              for (int q = 0; q < NB2; ++q) V::mac_conj(t, X[q], B[q]);
              V::renorm(t);
              acc[i2 * NB + i4] = t;
            }
        } else {
          // nb = 4: the same with rolled outer loops and T, X in this lane's shared scratch, so the
          // code stays within the instruction cache
          C* Ts = scratch[warp][lane];
          C* Xs = Ts + NB2;
          if (a.dm) {
#pragma unroll 1
            for (int i = 0; i < NB; ++i)
#pragma unroll
              for (int j = 0; j < NB; ++j) {
                C t = V::zero();
#pragma unroll
                for (int m = 0; m < NB; ++m) V::mac(t, Ar[i * NB + m], V::load(Rd, Rf, ro + m * NB + j));
                Ts[i * NB + j] = t;
              }
#pragma unroll 1
            for (int i = 0; i < NB; ++i)
#pragma unroll
              for (int j = 0; j < NB; ++j) {
                C t = V::zero();
#pragma unroll
                for (int m = 0; m < NB; ++m) V::mac(t, V::load(Ld, Lf, lo + i * NB + m), Ts[m * NB + j]);
                Xs[i * NB + j] = t;
              }
          } else {
            const double* f3 = a.f + (size_t)ka * NB;
            const double* f4 = a.f + (size_t)kb * NB;
#pragma unroll 1
            for (int i = 0; i < NB; ++i)
#pragma unroll
              for (int j = 0; j < NB; ++j) {
                const double sl = w == 0 ? 1 - f3[i] : f3[i], sr = w == 0 ? f4[j] : 1 - f4[j];
                Xs[i * NB + j] = V::scale(V::scale(Ar[i * NB + j], sl), sr);
              }
          }
#pragma unroll 1
          for (int q = 0; q < NB2; ++q) {
            const C xq = Xs[q];
#pragma unroll
            for (int i2 = 0; i2 < NB; ++i2)
#pragma unroll
              for (int i4 = 0; i4 < NB; ++i4)
                V::mac_conj(acc[i2 * NB + i4], xq, sm.A[grp][(w == 0 ? i2 * NB + i4 : i4 * NB + i2) * NB2 + q]);
          }
#pragma unroll
          for (int e = 0; e < NB2; ++e) V::renorm(acc[e]);
        }
      }
      __syncwarp();
    }
    // keep the candidates not taken
    const int rest = ncand - take;
    int2 keep = make_int2(0, 0);
    if (lane < rest) keep = sm.cand[take + lane];
    __syncwarp();
    if (lane < rest) sm.cand[lane] = keep;
    ncand = rest;
    __syncwarp();
  }
  // add the groups' partial sums (lanes with the same role), in FP64
  double2 accd[NB2];
#pragma unroll
  for (int e = 0; e < NB2; ++e) accd[e] = V::value(acc[e]);
#pragma unroll
  for (int off = G; off < 32; off <<= 1)
#pragma unroll
    for (int e = 0; e < NB2; ++e) {
      accd[e].x += __shfl_xor_sync(FULL, accd[e].x, off);
      accd[e].y += __shfl_xor_sync(FULL, accd[e].y, off);
    }
  if (grp == 0) {
#pragma unroll
    for (int i2 = 0; i2 < NB; ++i2)
#pragma unroll
      for (int i4 = 0; i4 < NB; ++i4) {
        const double2 v = accd[i2 * NB + i4];
        out[w * NB4 + ((i1 * NB + i2) * NB + i3) * NB + i4] = mk2(a.prefac * v.x, a.prefac * v.y);
      }
  }
}

// The e-e source of the linearized operators besides P_ee (elecelec_model::calc_P3P4 and calc_P5P6,
// ElecElec_Model_linear.cpp:3-112), at the occupations f (the f_eq of the linearization), for every
// stored pair (k1, ka), FP64:
//   P3 / P4[(i1,i2),(ia,ib)] = sum_(k3, i3, i4) A[(i1,i4),(i3,ia)] w conj(A[(i2,i4),(i3,ib)]), A of
//     (k1, k4, k3, ka) with k4 = k1 + k3 - ka, w = (1 - f3) f4 (P3) or f3 (1 - f4) (P4);
//   P5 / P6[(i1,i2),(ia,ib)] = sum_(k3, i3, i4) A[(i1,i3),(ib,i4)] w conj(A[(i2,i3),(ia,i4)]), A of
//     (k1, k3, ka, k4) with k4 = k1 + ka - k3, w = f3 f4 (P5) or (1 - f3)(1 - f4) (P6);
// A(q1, q2, q3, q4)[(a,b),(c,d)] = delta(e_q1 a - e_q2 b + e_q3 c - e_q4 d) vq(q1 - q2) o(q1,q2)[a][b]
// o(q3,q4)[c][d] (the exchange form with the exchange term), as calc_A (ElecElec_Model.h:144-162).
// With the exchange term P3, P4 stay zero (the reference skips them). A set-up computation: one block
// per pair; its first warp tests 32 k3 at a time for a k4 on the set and a band combination in the
// window (the exact FP64 test), keeping the candidates in k3 order; then all threads build A of
// each candidate in shared memory and thread (i1,i2,ia,ib) accumulates its four outputs in k3 order.
__device__ __forceinline__ double2 ee_cmul(double2 a, double2 b) {
  return mk2(fma(a.x, b.x, -a.y * b.y), fma(a.x, b.y, a.y * b.x));
}
__device__ __forceinline__ double2 ee_cfma_conjb(double2 a, double2 b, double2 c) {  // c + a conj(b)
  return mk2(fma(a.x, b.x, fma(a.y, b.y, c.x)), fma(a.y, b.x, fma(-a.x, b.y, c.y)));
}

template <int NB>
__global__ void __launch_bounds__(NB == 4 ? 256 : 32) k_ee_p36(EeArgs a, const double* __restrict__ f,
                                                              double2* __restrict__ P3, double2* __restrict__ P4,
                                                              double2* __restrict__ P5, double2* __restrict__ P6) {
  constexpr int NB2 = NB * NB, NB4 = NB2 * NB2;
  __shared__ double2 sA[NB4];
  __shared__ double2 so12[NB2], so34[NB2], so14[NB2], so32[NB2];
  __shared__ int cand3[32], cand4[32];
  __shared__ int ncand;
  const int p = blockIdx.x;
  if (p >= a.npair) return;
  const int t = threadIdx.x;
  const int k1 = a.kk[p].x, ka = a.kk[p].y;
  const EeScreen scr = *a.scr;
  const unsigned FULL = 0xffffffffu;
  const int i1 = t / (NB * NB2), i2 = (t / NB2) % NB, ia = (t / NB) % NB, ib = t % NB;  // output (i1,i2),(ia,ib)
  for (int phase = 0; phase < 2; ++phase) {
    double2 x = mk2(0, 0), y = mk2(0, 0);
    if (!(phase == 0 && a.antisym)) {
      for (int c0 = 0; c0 < a.nk; c0 += 32) {
        if (t < 32) {
          const int k3 = c0 + t;
          int k4 = -1;
          bool ok = k3 < a.nk;
          if (ok && phase == 0) ok = !(ka == k3 && !a.antisym) && !(a.antisym && ka == k3 && k1 == ka);
          if (ok && phase == 1) ok = !(k1 == k3 && !a.antisym) && !(a.antisym && k1 == k3 && ka == k3);
          if (ok) {  // k4 = k1 + k3 - ka (phase 0) or k1 + ka - k3 (phase 1) by mesh index arithmetic
            const int4 u = a.kidx[k1], v = a.kidx[phase ? ka : k3], w = a.kidx[phase ? k3 : ka];
            int m[3] = {u.x + v.x - w.x, u.y + v.y - w.y, u.z + v.z - w.z};
            for (int d = 0; d < 3; ++d) m[d] += m[d] < 0 ? a.kmesh[d] : (m[d] >= a.kmesh[d] ? -a.kmesh[d] : 0);
            k4 = a.kmap[((size_t)m[0] * a.kmesh[1] + m[1]) * a.kmesh[2] + m[2]];
            ok = k4 >= 0;
          }
          if (ok) {  // calc_delta's window test over every band combination
            const int q1 = k1, q2 = phase ? k3 : k4, q3 = phase ? ka : k3, q4 = phase ? k4 : ka;
            bool hit = false;
            for (int c = 0; c < NB4; ++c) {
              const double de = a.ew[(size_t)q1 * NB + c / (NB * NB2)] - a.ew[(size_t)q2 * NB + (c / NB2) % NB] +
                                a.ew[(size_t)q3 * NB + (c / NB) % NB] - a.ew[(size_t)q4 * NB + c % NB];
              hit |= fabs(de) < a.ethr;
            }
            ok = hit;
          }
          const unsigned ball = __ballot_sync(FULL, ok);
          if (ok) {
            const int pos = __popc(ball & ((1u << t) - 1));
            cand3[pos] = k3;
            cand4[pos] = k4;
          }
          if (t == 0) ncand = __popc(ball);
        }
        __syncthreads();
        const int nc = ncand;
        for (int ci = 0; ci < nc; ++ci) {
          const int k3 = cand3[ci], k4 = cand4[ci];
          const int q1 = k1, q2 = phase ? k3 : k4, q3 = phase ? ka : k3, q4 = phase ? k4 : ka;
          if (t < NB2) {  // calc_ovlps with the first overlap times vq
            const double vq = ee_vq(a, scr, q1, q2);
            const double2 o = ee_ovlp<NB>(a, q1, q2, t / NB, t % NB);
            so12[t] = mk2(vq * o.x, vq * o.y);
            so34[t] = ee_ovlp<NB>(a, q3, q4, t / NB, t % NB);
            if (a.antisym) {
              const double vx = ee_vq(a, scr, q1, q4);
              const double2 ox = ee_ovlp<NB>(a, q1, q4, t / NB, t % NB);
              so14[t] = mk2(vx * ox.x, vx * ox.y);
              so32[t] = ee_ovlp<NB>(a, q3, q2, t / NB, t % NB);
            }
          }
          __syncthreads();
          if (t < NB4) {  // A[(c1,c2),(c3,c4)] = delta mee (calc_delta, calc_mee[_ex], calc_A)
            const int c1 = t / (NB * NB2), c2 = (t / NB2) % NB, c3 = (t / NB) % NB, c4 = t % NB;
            const double de = a.ew[(size_t)q1 * NB + c1] - a.ew[(size_t)q2 * NB + c2] + a.ew[(size_t)q3 * NB + c3] -
                              a.ew[(size_t)q4 * NB + c4];
            double2 mee = ee_cmul(so12[c1 * NB + c2], so34[c3 * NB + c4]);
            if (a.antisym) {
              const double2 mex = ee_cmul(so14[c1 * NB + c4], so32[c3 * NB + c2]);
              mee = mk2(0.5 * mee.x - 0.5 * mex.x, 0.5 * mee.y - 0.5 * mex.y);
            }
            const double dl = fabs(de) < a.ethr ? exp(a.prefac_exp * de * de) : 0.0;
            sA[t] = mk2(dl * mee.x, dl * mee.y);
          }
          __syncthreads();
          if (t < NB4) {
            const double* f3 = f + (size_t)k3 * NB;
            const double* f4 = f + (size_t)k4 * NB;
            if (phase == 0) {
              for (int i4 = 0; i4 < NB; ++i4)
                for (int i3 = 0; i3 < NB; ++i3) {
                  const double2 A1 = sA[((i1 * NB + i4) * NB + i3) * NB + ia];
                  const double2 A2 = sA[((i2 * NB + i4) * NB + i3) * NB + ib];
                  const double w3 = (1 - f3[i3]) * f4[i4], w4 = f3[i3] * (1 - f4[i4]);
                  x = ee_cfma_conjb(mk2(w3 * A1.x, w3 * A1.y), A2, x);
                  y = ee_cfma_conjb(mk2(w4 * A1.x, w4 * A1.y), A2, y);
                }
            } else {
              for (int i3 = 0; i3 < NB; ++i3)
                for (int i4 = 0; i4 < NB; ++i4) {
                  const double2 A1 = sA[((i1 * NB + i3) * NB + ib) * NB + i4];
                  const double2 A2 = sA[((i2 * NB + i3) * NB + ia) * NB + i4];
                  const double w5 = f3[i3] * f4[i4], w6 = (1 - f3[i3]) * (1 - f4[i4]);
                  x = ee_cfma_conjb(mk2(w5 * A1.x, w5 * A1.y), A2, x);
                  y = ee_cfma_conjb(mk2(w6 * A1.x, w6 * A1.y), A2, y);
                }
            }
          }
          __syncthreads();
        }
        __syncthreads();  // every thread has read ncand before the next chunk's test overwrites it
      }
    }
    if (t < NB4) {
      double2* ox = (phase ? P5 : P3) + (size_t)p * NB4 + t;
      double2* oy = (phase ? P6 : P4) + (size_t)p * NB4 + t;
      *ox = mk2(a.prefac * x.x, a.prefac * x.y);
      *oy = mk2(a.prefac * y.x, a.prefac * y.y);
    }
    __syncthreads();
  }
}

}  // namespace dmd
