// Per-evaluation kernels of the Lindblad right-hand side: phase/prep, finish (+coherent term and
// stepper fusion), observables and stepper combinations. The k-pair contraction kernels live in
// dmd_pairs.cuh.
//
// Algebra (exact rewrite of evolve_eph.cpp:34-166). With D_k[(i,j)] = exp(i t (e_k,i - e_k,j)) the
// reference's P(t) phase factorises: P1(t)[a][b] = P1[a][b] D_k[a] conj(D_k'[b]) and
// P2(t)[a][b] = P2[a][b] D_k[b] conj(D_k'[a]). Hence, with rt_k = conj(D_k) o rho_k and
// st_k = conj(D_k) o (1 - rho_k),
//   Pdm_k  = D_k o X_k,  X_k  = sum_pairs P1 rt_k'        + [k' side] conj(P2) rt_k
//   dm1P_k = D_k o Y_k,  Y_k  = sum_pairs st_k'^T P2      + [k' side] st_k^T conj(P1)
// and the pair loop needs no trigonometry. The finish applies D_k, forms
// c = (1-rho_k) Pdm_k - dm1P_k rho_k with Hermitian operands read from their upper triangles
// (zhemm, comm/mymatrix.cpp:73-76) and returns (prefac/2) (c + c^dagger) (evolve_eph.cpp:140-152).
#pragma once
#include "dmd_common.cuh"

namespace dmd {

// time of an evaluation: either a plain value or derived on the device from a step counter so that
// captured graphs need no parameter updates. stage: 0 -> t, 1/2 -> t + h/2, 3 -> t + h.
struct TimeArg {
  double t;               // used when tref == nullptr
  const double* tref;     // [t0, h]
  const long long* step;  // completed steps since t0
  int stage;
};

__device__ __forceinline__ double eval_time(const TimeArg& ta) {
  if (!ta.tref) return ta.t;
  const double t0 = ta.tref[0], h = ta.tref[1];
  const double t = t0 + (double)(*ta.step) * h;
  if (ta.stage == 0) return t;
  if (ta.stage == 3) return t + h;
  return t + 0.5 * h;
}

// rt_k, st_k (window, phase removed) and zeroed X/Y accumulators. One thread per (k, element); the
// phase D_k(i, j) is stored in ph ([nk][NB2]) for the finish kernel.
template <int NB>
__global__ void k_prep(int nk, int nbdm, int bs, const double2* __restrict__ y, const double* __restrict__ ew,
                       TimeArg ta, int phase, double2* __restrict__ rs, double2* __restrict__ acc,
                       double2* __restrict__ ph) {
  constexpr int NB2 = NB * NB;
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= nk * NB2) return;
  const int k = idx / NB2, ab = idx - k * NB2, i = ab / NB, j = ab - i * NB;
  const double2 r = y[(size_t)k * nbdm * nbdm + (bs + i) * nbdm + bs + j];
  // set_oneminusdm (DenMat.cpp:249-261): 1 - dm on the diagonal, -dm elsewhere
  const double2 s = (i == j) ? mk2(1.0 - r.x, 0.0 - r.y) : mk2(-r.x, -r.y);
  double2 rt = r, st = s;
  if (phase) {
    const double t = eval_time(ta);
    const double2 d = ccis((ew[k * NB + i] - ew[k * NB + j]) * t);
    ph[(size_t)k * NB2 + ab] = d;
    rt = cmul_rn(cconj(d), r);
    st = cmul_rn(cconj(d), s);
  }
  rs[(size_t)k * 2 * NB2 + ab] = rt;
  rs[(size_t)k * 2 * NB2 + NB2 + ab] = st;
  acc[(size_t)k * 2 * NB2 + ab] = mk2(0.0, 0.0);
  acc[(size_t)k * 2 * NB2 + NB2 + ab] = mk2(0.0, 0.0);
}

// Hermitian operand read from the upper triangle with a real diagonal (BLAS zhemm semantics)
__device__ __forceinline__ double2 herm_up(const double2* A, int n, int i, int l) {
  if (i == l) return mk2(A[i * n + i].x, 0.0);
  return (i < l) ? A[i * n + l] : cconj(A[l * n + i]);
}

struct FinishArgs {
  int nk, nbdm, bs;
  double prefac;       // prefac_eph
  int picture;         // 0 interaction, 1 schrodinger
  int phase;           // alg.expt in the interaction picture
  const double* ew;    // [nk][NB]
  const double* edm;   // [nk][nbdm]
  const double2* H;    // [nk][nbdm^2] or null
  const double2* eq;   // [nk][NB2] or null
  const double2* y;    // state the RHS is evaluated on
  const double2* acc;  // [nk][2][NB2], indexed by pos[k] when pos is set
  const double2* ph;   // D_k(i, j) = exp(i t (e_i - e_j)) of this evaluation [nk][NB2] (prep kernels)
  // split finish (k_finish<.., DEV = true): acc holds the FP32 contraction of rho - F only,
  // F = diag(fref), and the phases are FP32 (ph32)
  const double* fref;  // [nk][NB]
  const float2* x0y0;  // X0, Y0 = contraction of F, back-transformed [nk][2][NB2] (null: zero)
  const float2* v0;    // (prefac/2)(C0 + C0^dagger), C0 = (1 - F) X0 - Y0 F, [nk][NB2] (null: zero)
  const float2* ph32;  // D_k(i, j) in FP32 [nk][NB2]
  const int* pos;      // k -> accumulator row (column-block layout) or null
  int herm;            // accumulators hold X' = M^H X, Y' = M^H Y (Hermitian coordinates)
  int nrhs;            // batched form: states evaluated together (blockIdx.y), 1 otherwise
  size_t sstride;      // state elements per state (nk * nbdm^2)
  size_t astride;      // accumulator elements (double2) per state
  int lin;             // linearized: the scattering term is (prefac/2)(D o X + h.c.) (evolve_eph_linear.cpp:44-51)
  unsigned int* hflag; // non-Hermitian-state flag of the prep kernel, cleared here (or null)
  int want_eph, want_coh;
  // output: plain RHS
  double2* out;
  // RK4 stage fusion (mode 1)
  int mode;            // 0: out = f; 1: RK4 stage; 2: Euler
  int stage;
  const double* tref;  // [t0, h] for RK4/Euler
  long long* step;
  double2* K;          // [4][nk*nbdm^2]
  double2* ybase;      // y_n
  double2* ytmp;       // next stage input
  TimeArg ta;
};

__device__ __forceinline__ float2 f2(double2 v) { return make_float2((float)v.x, (float)v.y); }
__device__ __forceinline__ float2 fmul(float2 a, float2 b) {
  return make_float2(__fmaf_rn(a.x, b.x, -a.y * b.y), __fmaf_rn(a.x, b.y, a.y * b.x));
}
__device__ __forceinline__ float2 ffma(float2 a, float2 b, float2 c) {  // c + a*b
  return make_float2(__fmaf_rn(a.x, b.x, __fmaf_rn(-a.y, b.y, c.x)), __fmaf_rn(a.x, b.y, __fmaf_rn(a.y, b.x, c.y)));
}

// One thread per k: scattering finish + coherent term, then the stepper's update for this k.
// ND > 0: the density matrix has ND = nbdm = NB bands (compile time, arrays in registers); ND = 0:
// nbdm is read at run time.
// DEV (batched reduced-precision form): with rho = F + delta, F = diag(f_ref),
//   c = D o C0 + (1 - F)(D o Xd) - (D o Yd) F - delta (D o (X0 + Xd)) - (D o (Y0 + Yd)) delta
// (Hermitian operands from their upper triangles, F diagonal, C0 = (1 - F) X0 - Y0 F), so
// (prefac/2)(c + c^dagger) = D o V0 + (prefac/2)(c1 + c1^dagger). The per-k constant V0 is formed
// in FP64 on the host (where (1 - F) X0 and Y0 F cancel) and stored rounded to FP32; the terms of
// first and second order in delta (c1) are FP32; the state update stays FP64.
template <int NB, int ND = 0, bool DEV = false>
__global__ void k_finish(FinishArgs a) {
  constexpr int NB2 = NB * NB;
  constexpr int NDA = ND > 0 ? ND : DMD_MAX_NBDM;  // array extent
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  const int q = blockIdx.y;  // state of the batch
  if (a.hflag && k == 0 && q == 0) *a.hflag = 0u;  // every pair launch of this evaluation has completed
  if (k >= a.nk) return;
  const int nd = ND > 0 ? ND : a.nbdm, nd2 = nd * nd;
  const int bs = (ND == NB) ? 0 : a.bs;  // the window is the whole density matrix
  const double t = eval_time(a.ta);
  const size_t qs = (size_t)q * a.sstride;
  const double2* yk = a.y + qs + (size_t)k * nd2;
  double2 f[NDA * NDA];
#pragma unroll
  for (int i = 0; i < nd2; ++i) f[i] = mk2(0.0, 0.0);

  // coherent term: -i [H(t), rho] (DenMat.cpp:29-55)
  if (a.want_coh) {
    const double* ek = a.edm + (size_t)k * nd;
    if (a.H) {
      double2 Ht[NDA * NDA];
      const double2* Hk = a.H + (size_t)k * nd2;
#pragma unroll
      for (int i = 0; i < nd; ++i)
#pragma unroll
        for (int j = 0; j < nd; ++j)
          Ht[i * nd + j] = (a.picture == 0 && i != j) ? cmul_rn(Hk[i * nd + j], ccis((ek[i] - ek[j]) * t)) : Hk[i * nd + j];
      double2 c1[NDA * NDA];
#pragma unroll
      for (int i = 0; i < nd; ++i)
#pragma unroll
        for (int j = 0; j < nd; ++j) {  // dm * H (zhemm Right, beta = 0)
          double2 s = mk2(0.0, 0.0);
#pragma unroll
          for (int l = 0; l < nd; ++l) s = cadd_rn(s, cmul_rn(yk[i * nd + l], herm_up(Ht, nd, l, j)));
          c1[i * nd + j] = cmul_rn(mk2(1.0, 0.0), s);
        }
#pragma unroll
      for (int i = 0; i < nd; ++i)
#pragma unroll
        for (int j = 0; j < nd; ++j) {  // H * dm - (dm * H)   (zhemm Left, beta = -1)
          double2 s = mk2(0.0, 0.0);
#pragma unroll
          for (int l = 0; l < nd; ++l) s = cadd_rn(s, cmul_rn(herm_up(Ht, nd, i, l), yk[l * nd + j]));
          const double2 o = cadd_rn(cmul_rn(mk2(1.0, 0.0), s), cmul_rn(mk2(-1.0, 0.0), c1[i * nd + j]));
          f[i * nd + j] = cadd_rn(mk2(0.0, 0.0), cmul_rn(o, mk2(0.0, -1.0)));
        }
    } else if (a.picture == 1) {  // commutator_mat_diag(C, e, dm, nb, -i)
#pragma unroll
      for (int i = 0; i < nd; ++i)
#pragma unroll
        for (int j = 0; j < nd; ++j) {
          const double2 d = yk[i * nd + j];
          const double2 c = mk2(-__dmul_rn(d.x, ek[j]), -__dmul_rn(d.y, ek[j]));
          f[i * nd + j] = cadd_rn(mk2(0.0, 0.0), cmul_rn(cadd_rn(c, cmul_rn(mk2(ek[i], 0.0), d)), mk2(0.0, -1.0)));
        }
    }
  }

  // scattering finish on the window (evolve_eph.cpp:140-162, evolve_driver :21-32)
  if (DEV && a.want_eph) {
    // the sums (and for nb = 2 the per-k constants) as 16-byte loads (every block starts on a
    // 16-byte boundary); for nb = 4 the constants stay element loads, which keeps it free of spills
    constexpr bool PRE = NB == 2;
    const float4* Xs4 =
        (const float4*)((const float2*)a.acc + (size_t)q * a.astride + (size_t)(a.pos ? a.pos[k] : k) * 2 * NB2);
    float2 X[NB2], Y[NB2], X0[PRE ? NB2 : 1], Y0[PRE ? NB2 : 1], Dk[PRE ? NB2 : 1], V0[PRE ? NB2 : 1];
#pragma unroll
    for (int i = 0; i < NB2 / 2; ++i) {
      const float4 x = Xs4[i], yv = Xs4[NB2 / 2 + i];
      X[2 * i] = make_float2(x.x, x.y);
      X[2 * i + 1] = make_float2(x.z, x.w);
      Y[2 * i] = make_float2(yv.x, yv.y);
      Y[2 * i + 1] = make_float2(yv.z, yv.w);
      if constexpr (!PRE) continue;
      const float4 x0 = a.x0y0 ? ((const float4*)(a.x0y0 + (size_t)k * 2 * NB2))[i] : make_float4(0.f, 0.f, 0.f, 0.f);
      const float4 y0 =
          a.x0y0 ? ((const float4*)(a.x0y0 + (size_t)k * 2 * NB2))[NB2 / 2 + i] : make_float4(0.f, 0.f, 0.f, 0.f);
      X0[2 * i] = make_float2(x0.x, x0.y);
      X0[2 * i + 1] = make_float2(x0.z, x0.w);
      Y0[2 * i] = make_float2(y0.x, y0.y);
      Y0[2 * i + 1] = make_float2(y0.z, y0.w);
      const float4 d = a.phase ? ((const float4*)(a.ph32 + (size_t)k * NB2))[i] : make_float4(1.f, 0.f, 1.f, 0.f);
      Dk[2 * i] = make_float2(d.x, d.y);
      Dk[2 * i + 1] = make_float2(d.z, d.w);
      const float4 v = a.v0 ? ((const float4*)(a.v0 + (size_t)k * NB2))[i] : make_float4(0.f, 0.f, 0.f, 0.f);
      V0[2 * i] = make_float2(v.x, v.y);
      V0[2 * i + 1] = make_float2(v.z, v.w);
    }
    if (a.herm) {  // X = (M^H)^-1 X'
#pragma unroll
      for (int i = 0; i < NB; ++i)
#pragma unroll
        for (int j = i + 1; j < NB; ++j) {
          const float2 xu = X[i * NB + j], xl = X[j * NB + i], yu = Y[i * NB + j], yl = Y[j * NB + i];
          X[i * NB + j] = make_float2(0.5f * (xu.x - xl.y), 0.5f * (xu.y + xl.x));
          X[j * NB + i] = make_float2(0.5f * (xu.x + xl.y), 0.5f * (xu.y - xl.x));
          Y[i * NB + j] = make_float2(0.5f * (yu.x - yl.y), 0.5f * (yu.y + yl.x));
          Y[j * NB + i] = make_float2(0.5f * (yu.x + yl.y), 0.5f * (yu.y - yl.x));
        }
    }
    const double* fk = a.fref + (size_t)k * NB;
    float ff[NB];
    float2 dh[NB2], D[NB2], PXd[NB2], PXt[NB2], PYd[NB2], PYt[NB2];
#pragma unroll
    for (int i = 0; i < NB; ++i) ff[i] = (float)fk[i];
#pragma unroll
    for (int i = 0; i < NB; ++i)
#pragma unroll
      for (int j = 0; j < NB; ++j) {
        const int e = i * NB + j;
        // herm_up(rho - F): upper triangle, real diagonal (the diagonal difference in FP64)
        if (i == j) dh[e] = make_float2((float)__dsub_rn(yk[(bs + i) * nd + bs + i].x, fk[i]), 0.f);
        else if (i < j) dh[e] = f2(yk[(bs + i) * nd + bs + j]);
        else dh[e] = make_float2(dh[j * NB + i].x, -dh[j * NB + i].y);
        float2 x0, y0;
        if constexpr (PRE) {
          D[e] = (a.phase && i != j) ? Dk[e] : make_float2(1.f, 0.f);
          x0 = X0[e];
          y0 = Y0[e];
        } else {
          D[e] = (a.phase && i != j) ? a.ph32[(size_t)k * NB2 + e] : make_float2(1.f, 0.f);
          x0 = a.x0y0 ? a.x0y0[(size_t)k * 2 * NB2 + e] : make_float2(0.f, 0.f);
          y0 = a.x0y0 ? a.x0y0[(size_t)k * 2 * NB2 + NB2 + e] : make_float2(0.f, 0.f);
        }
        PXd[e] = fmul(D[e], X[e]);
        PYd[e] = fmul(D[e], Y[e]);
        PXt[e] = ffma(D[e], x0, PXd[e]);
        PYt[e] = ffma(D[e], y0, PYd[e]);
      }
    float2 c[NB2];
#pragma unroll
    for (int i = 0; i < NB; ++i)
#pragma unroll
      for (int j = 0; j < NB; ++j) {
        const int e = i * NB + j;
        if (a.lin) {
          c[e] = PXd[e];
        } else {
          float2 s = make_float2((1.f - ff[i]) * PXd[e].x - ff[j] * PYd[e].x, (1.f - ff[i]) * PXd[e].y - ff[j] * PYd[e].y);
#pragma unroll
          for (int l = 0; l < NB; ++l) {
            const float2 d1 = dh[i * NB + l], d2 = dh[l * NB + j];
            s = ffma(make_float2(-d1.x, -d1.y), PXt[l * NB + j], s);
            s = ffma(make_float2(-PYt[i * NB + l].x, -PYt[i * NB + l].y), d2, s);
          }
          c[e] = s;
        }
      }
    const float pf = (float)(a.prefac * 0.5);
#pragma unroll
    for (int i = 0; i < NB; ++i)
#pragma unroll
      for (int j = i; j < NB; ++j) {
        const float2 c1 = c[i * NB + j], c2 = c[j * NB + i];
        float2 vf = make_float2(pf * (c1.x + c2.x), pf * (c1.y - c2.y));
        if (a.v0) {  // + D o V0
          if constexpr (PRE) vf = ffma(D[i * NB + j], V0[i * NB + j], vf);
          else vf = ffma(D[i * NB + j], a.v0[(size_t)k * NB2 + i * NB + j], vf);
        }
        const double2 v = mk2((double)vf.x, (double)vf.y);
#pragma unroll
        for (int w = 0; w < (i == j ? 1 : 2); ++w) {
          const int ii = w ? j : i, jj = w ? i : j;
          double2 u = w ? cconj(v) : v;
          if (a.eq) {
            const double2 qv = a.eq[(size_t)k * NB2 + ii * NB + jj];
            if (ii == jj || a.picture == 1) u = csub_rn(u, qv);
            else {
              float2 d = make_float2(1.f, 0.f);
              if (a.phase) {
                if constexpr (PRE) d = Dk[ii * NB + jj];
                else d = a.ph32[(size_t)k * NB2 + ii * NB + jj];
              }
              u = csub_rn(u, cmul_rn(qv, mk2((double)d.x, (double)d.y)));
            }
          }
          double2& o = f[(bs + ii) * nd + bs + jj];
          o = a.want_coh ? cadd_rn(o, u) : u;
        }
      }
  } else if (a.want_eph) {
    const double* ew = a.ew + (size_t)k * NB;
    const double2* Xs = a.acc + (size_t)q * a.astride + (size_t)(a.pos ? a.pos[k] : k) * 2 * NB2;
    double2 X[NB2], Y[NB2];
#pragma unroll
    for (int i = 0; i < NB2; ++i) {
      X[i] = Xs[i];
      Y[i] = Xs[NB2 + i];
    }
    if (a.herm) {  // X = (M^H)^-1 X': X_ij = (X'_ij + i X'_ji) / 2, X_ji = (X'_ij - i X'_ji) / 2 for i < j
#pragma unroll
      for (int i = 0; i < NB; ++i)
#pragma unroll
        for (int j = i + 1; j < NB; ++j) {
          const double2 xu = X[i * NB + j], xl = X[j * NB + i], yu = Y[i * NB + j], yl = Y[j * NB + i];
          X[i * NB + j] = mk2(0.5 * (xu.x - xl.y), 0.5 * (xu.y + xl.x));
          X[j * NB + i] = mk2(0.5 * (xu.x + xl.y), 0.5 * (xu.y - xl.x));
          Y[i * NB + j] = mk2(0.5 * (yu.x - yl.y), 0.5 * (yu.y + yl.x));
          Y[j * NB + i] = mk2(0.5 * (yu.x + yl.y), 0.5 * (yu.y - yl.x));
        }
    }
    double2 rw[NB2], sw[NB2], Pdm[NB2], dmP[NB2];
#pragma unroll
    for (int i = 0; i < NB; ++i)
#pragma unroll
      for (int j = 0; j < NB; ++j) {
        const double2 r = yk[(bs + i) * nd + bs + j];
        rw[i * NB + j] = r;
        sw[i * NB + j] = (i == j) ? mk2(1.0 - r.x, 0.0 - r.y) : mk2(-r.x, -r.y);
        if (a.phase && i != j) {  // D_k(i, i) = 1
          const double2 d = a.ph ? a.ph[(size_t)k * NB2 + i * NB + j] : ccis((ew[i] - ew[j]) * t);
          Pdm[i * NB + j] = cmul_rn(d, X[i * NB + j]);
          dmP[i * NB + j] = cmul_rn(d, Y[i * NB + j]);
        } else {
          Pdm[i * NB + j] = X[i * NB + j];
          dmP[i * NB + j] = Y[i * NB + j];
        }
      }
    double2 c[NB2];
    if (a.lin) {
#pragma unroll
      for (int i = 0; i < NB2; ++i) c[i] = Pdm[i];
    } else {
      // c = (1 - dm) Pdm - dm1P dm (zhemm Left alpha 1 beta 0, then zhemm Right alpha -1 beta 1):
      // the Hermitian operands are read from their upper triangles; complex multiply-adds on the FMA
      // pipe (the unit scalings alpha = 1, -1 are exact and not multiplied out)
#pragma unroll
      for (int i = 0; i < NB; ++i)
#pragma unroll
        for (int j = 0; j < NB; ++j) {
          double2 s = mk2(0.0, 0.0);
#pragma unroll
          for (int l = 0; l < NB; ++l) s = cfma(herm_up(sw, NB, i, l), Pdm[l * NB + j], s);
#pragma unroll
          for (int l = 0; l < NB; ++l) {
            const double2 m = dmP[i * NB + l];
            s = cfma(mk2(-m.x, -m.y), herm_up(rw, NB, l, j), s);
          }
          c[i * NB + j] = s;
        }
    }
    const double pf = a.prefac * 0.5;
#pragma unroll
    for (int i = 0; i < NB; ++i)
#pragma unroll
      for (int j = i; j < NB; ++j) {
        // (prefac/2)(c + c^dagger); the (j, i) element is the exact conjugate of the (i, j) one
        const double2 v = cscale_rn(pf, cadd_rn(c[i * NB + j], cconj(c[j * NB + i])));
#pragma unroll
        for (int w = 0; w < (i == j ? 1 : 2); ++w) {
          const int ii = w ? j : i, jj = w ? i : j;
          double2 u = w ? cconj(v) : v;
          if (a.eq) {
            const double2 q = a.eq[(size_t)k * NB2 + ii * NB + jj];
            if (ii == jj || a.picture == 1) u = csub_rn(u, q);
            else u = csub_rn(u, cmul_rn(q, a.ph ? a.ph[(size_t)k * NB2 + ii * NB + jj] : ccis((ew[ii] - ew[jj]) * t)));
          }
          double2& o = f[(bs + ii) * nd + bs + jj];
          o = cadd_rn(o, u);
        }
      }
  }

  const size_t base = qs + (size_t)k * nd2;
  if (a.mode == 0) {
#pragma unroll
    for (int i = 0; i < nd2; ++i) a.out[base + i] = f[i];
    return;
  }
  const size_t n = a.sstride * a.nrhs;  // stage stride: the whole batch
  if (a.mode == 1) {
    const double h = a.tref[1], hh = 0.5 * h, h6 = h / 6.0;
    double2* Ks = a.K + (size_t)a.stage * n;
#pragma unroll
    for (int i = 0; i < nd2; ++i) {
      const double2 yb = a.ybase[base + i];
      Ks[base + i] = f[i];
      if (a.stage == 0) a.ytmp[base + i] = cadd_rn(yb, cscale_rn(hh, f[i]));
      else if (a.stage == 1) a.ytmp[base + i] = cadd_rn(yb, cscale_rn(hh, f[i]));
      else if (a.stage == 2) a.ytmp[base + i] = cadd_rn(yb, cscale_rn(h, f[i]));
      else {
        const double2 k1 = a.K[base + i], k2 = a.K[n + base + i], k3 = a.K[2 * n + base + i];
        // y + h/6 * (k1 + 2 k2 + 2 k3 + k4), evaluated left to right
        const double sx = __dadd_rn(__dadd_rn(__dadd_rn(k1.x, __dmul_rn(2.0, k2.x)), __dmul_rn(2.0, k3.x)), f[i].x);
        const double sy = __dadd_rn(__dadd_rn(__dadd_rn(k1.y, __dmul_rn(2.0, k2.y)), __dmul_rn(2.0, k3.y)), f[i].y);
        a.ybase[base + i] = mk2(__dadd_rn(yb.x, __dmul_rn(h6, sx)), __dadd_rn(yb.y, __dmul_rn(h6, sy)));
      }
    }
    return;
  }
  if (a.mode == 2) {  // update_dm_euler: dm += 0.5*dt*(ddmdt + ddmdt^dagger)
    const double h = a.tref[1];
    const double hf = 0.5 * h;
#pragma unroll
    for (int i = 0; i < nd; ++i)
#pragma unroll
      for (int j = 0; j < nd; ++j) {
        const double2 v = cscale_rn(hf, cadd_rn(f[i * nd + j], cconj(f[j * nd + i])));
        a.ybase[base + i * nd + j] = cadd_rn(a.ybase[base + i * nd + j], v);
      }
  }
}

// The split finish of k_finish<NB, NB, true> with NB threads per (k, state): thread i computes row i
// of the result and the operands the rows share (the column terms D o (X + X0) and rho - F) go
// through shared memory. Each thread then holds a row instead of the whole NB x NB block, which for
// nb = 4 takes k_finish from 251 registers per thread (8 warps per SM) to a third of that. Same
// arithmetic element by element, so the result equals k_finish's; the (j, i) element of the
// Hermitian sum is formed from the (j, i) operands, which gives the exact conjugate of (i, j).
// Blocks of 128 threads: 32 (k, state) groups of NB = 4 threads, blockIdx.y the state.
template <int NB>
__global__ void __launch_bounds__(128) k_finish_rows(FinishArgs a) {
  constexpr int NB2 = NB * NB, GPB = 128 / NB;  // groups per block
  __shared__ float2 sPX[GPB][NB2], sdh[GPB][NB2], sc[GPB][NB2];
  __shared__ double2 sf[GPB][NB2];  // H(t), then the result's transpose (Euler)
  const int g = threadIdx.x / NB, i = threadIdx.x % NB;
  const int k = blockIdx.x * GPB + g;
  const int q = blockIdx.y;
  if (a.hflag && k == 0 && q == 0 && i == 0) *a.hflag = 0u;
  const bool live = k < a.nk;  // dead groups still reach the warp barriers
  const int kk = live ? k : 0;
  const double t = eval_time(a.ta);
  const size_t qs = (size_t)q * a.sstride;
  const double2* yk = a.y + qs + (size_t)kk * NB2;
  const unsigned gm = ((1u << NB) - 1u) << ((threadIdx.x & 31) / NB * NB);  // this group's lanes
  double2 f[NB];
#pragma unroll
  for (int j = 0; j < NB; ++j) f[j] = mk2(0.0, 0.0);

  // coherent term, row i (as k_finish)
  if (a.want_coh) {
    const double* ek = a.edm + (size_t)kk * NB;
    if (a.H) {
      const double2* Hk = a.H + (size_t)kk * NB2;
#pragma unroll
      for (int j = 0; j < NB; ++j)  // row i of H(t) into shared memory
        sf[g][i * NB + j] =
            (a.picture == 0 && i != j) ? cmul_rn(Hk[i * NB + j], ccis((ek[i] - ek[j]) * t)) : Hk[i * NB + j];
      __syncwarp(gm);
      auto hup = [&](int r, int c) {  // read with zhemm's upper-triangle semantics
        if (r == c) return mk2(sf[g][r * NB + r].x, 0.0);
        return r < c ? sf[g][r * NB + c] : cconj(sf[g][c * NB + r]);
      };
#pragma unroll
      for (int j = 0; j < NB; ++j) {
        double2 s1 = mk2(0.0, 0.0), s2 = mk2(0.0, 0.0);
#pragma unroll
        for (int l = 0; l < NB; ++l) s1 = cadd_rn(s1, cmul_rn(yk[i * NB + l], hup(l, j)));
        const double2 c1 = cmul_rn(mk2(1.0, 0.0), s1);
#pragma unroll
        for (int l = 0; l < NB; ++l) s2 = cadd_rn(s2, cmul_rn(hup(i, l), yk[l * NB + j]));
        const double2 o = cadd_rn(cmul_rn(mk2(1.0, 0.0), s2), cmul_rn(mk2(-1.0, 0.0), c1));
        f[j] = cadd_rn(mk2(0.0, 0.0), cmul_rn(o, mk2(0.0, -1.0)));
      }
      __syncwarp(gm);  // sf is reused below
    } else if (a.picture == 1) {
#pragma unroll
      for (int j = 0; j < NB; ++j) {
        const double2 d = yk[i * NB + j];
        const double2 c = mk2(-__dmul_rn(d.x, ek[j]), -__dmul_rn(d.y, ek[j]));
        f[j] = cadd_rn(mk2(0.0, 0.0), cmul_rn(cadd_rn(c, cmul_rn(mk2(ek[i], 0.0), d)), mk2(0.0, -1.0)));
      }
    }
  }

  if (a.want_eph) {
    const float2* Xs = (const float2*)a.acc + (size_t)q * a.astride + (size_t)(a.pos ? a.pos[kk] : kk) * 2 * NB2;
    const double* fk = a.fref + (size_t)kk * NB;
    float2 PXd[NB], PYd[NB], PYt[NB], D[NB];
#pragma unroll
    for (int j = 0; j < NB; ++j) {
      const int e = i * NB + j;
      // X = (M^H)^-1 X' element (i, j) from X'(i, j) and X'(j, i)
      float2 x = Xs[e], yv = Xs[NB2 + e];
      if (a.herm && i != j) {
        const int lo = i < j ? i : j, hi = i < j ? j : i;
        const float2 xu = Xs[lo * NB + hi], xl = Xs[hi * NB + lo], yu = Xs[NB2 + lo * NB + hi],
                     yl = Xs[NB2 + hi * NB + lo];
        if (i < j) {
          x = make_float2(0.5f * (xu.x - xl.y), 0.5f * (xu.y + xl.x));
          yv = make_float2(0.5f * (yu.x - yl.y), 0.5f * (yu.y + yl.x));
        } else {
          x = make_float2(0.5f * (xu.x + xl.y), 0.5f * (xu.y - xl.x));
          yv = make_float2(0.5f * (yu.x + yl.y), 0.5f * (yu.y - yl.x));
        }
      }
      D[j] = (a.phase && i != j) ? a.ph32[(size_t)kk * NB2 + e] : make_float2(1.f, 0.f);
      const float2 x0 = a.x0y0 ? a.x0y0[(size_t)kk * 2 * NB2 + e] : make_float2(0.f, 0.f);
      const float2 y0 = a.x0y0 ? a.x0y0[(size_t)kk * 2 * NB2 + NB2 + e] : make_float2(0.f, 0.f);
      PXd[j] = fmul(D[j], x);
      PYd[j] = fmul(D[j], yv);
      sPX[g][e] = ffma(D[j], x0, PXd[j]);
      PYt[j] = ffma(D[j], y0, PYd[j]);
      // herm_up(rho - F) (the diagonal difference in FP64)
      float2 dh;
      if (i == j) dh = make_float2((float)__dsub_rn(yk[i * NB + i].x, fk[i]), 0.f);
      else if (i < j) dh = f2(yk[i * NB + j]);
      else {
        const float2 u = f2(yk[j * NB + i]);
        dh = make_float2(u.x, -u.y);
      }
      sdh[g][e] = dh;
    }
    __syncwarp(gm);
    const float fi = (float)fk[i];
#pragma unroll
    for (int j = 0; j < NB; ++j) {
      float2 c;
      if (a.lin) {
        c = PXd[j];
      } else {
        const float fj = (float)fk[j];
        c = make_float2((1.f - fi) * PXd[j].x - fj * PYd[j].x, (1.f - fi) * PXd[j].y - fj * PYd[j].y);
#pragma unroll
        for (int l = 0; l < NB; ++l) {
          const float2 d1 = sdh[g][i * NB + l], d2 = sdh[g][l * NB + j];
          c = ffma(make_float2(-d1.x, -d1.y), sPX[g][l * NB + j], c);
          c = ffma(make_float2(-PYt[l].x, -PYt[l].y), d2, c);
        }
      }
      sc[g][i * NB + j] = c;
    }
    __syncwarp(gm);
    const float pf = (float)(a.prefac * 0.5);
#pragma unroll
    for (int j = 0; j < NB; ++j) {
      const float2 c1 = sc[g][i * NB + j], c2 = sc[g][j * NB + i];
      float2 vf = make_float2(pf * (c1.x + c2.x), pf * (c1.y - c2.y));
      if (a.v0) vf = ffma(D[j], a.v0[(size_t)kk * NB2 + i * NB + j], vf);  // + D o V0
      double2 u = mk2((double)vf.x, (double)vf.y);
      if (a.eq) {
        const double2 qv = a.eq[(size_t)kk * NB2 + i * NB + j];
        if (i == j || a.picture == 1) u = csub_rn(u, qv);
        else u = csub_rn(u, cmul_rn(qv, mk2((double)D[j].x, (double)D[j].y)));
      }
      f[j] = a.want_coh ? cadd_rn(f[j], u) : u;
    }
  }

  if (!live) return;
  const size_t base = qs + (size_t)k * NB2 + (size_t)i * NB;
  if (a.mode == 0) {
#pragma unroll
    for (int j = 0; j < NB; ++j) a.out[base + j] = f[j];
    return;
  }
  const size_t n = a.sstride * a.nrhs;
  if (a.mode == 1) {
    const double h = a.tref[1], hh = 0.5 * h, h6 = h / 6.0;
    double2* Ks = a.K + (size_t)a.stage * n;
#pragma unroll
    for (int j = 0; j < NB; ++j) {
      const double2 yb = a.ybase[base + j];
      Ks[base + j] = f[j];
      if (a.stage == 0) a.ytmp[base + j] = cadd_rn(yb, cscale_rn(hh, f[j]));
      else if (a.stage == 1) a.ytmp[base + j] = cadd_rn(yb, cscale_rn(hh, f[j]));
      else if (a.stage == 2) a.ytmp[base + j] = cadd_rn(yb, cscale_rn(h, f[j]));
      else {
        const double2 k1 = a.K[base + j], k2 = a.K[n + base + j], k3 = a.K[2 * n + base + j];
        const double sx = __dadd_rn(__dadd_rn(__dadd_rn(k1.x, __dmul_rn(2.0, k2.x)), __dmul_rn(2.0, k3.x)), f[j].x);
        const double sy = __dadd_rn(__dadd_rn(__dadd_rn(k1.y, __dmul_rn(2.0, k2.y)), __dmul_rn(2.0, k3.y)), f[j].y);
        a.ybase[base + j] = mk2(__dadd_rn(yb.x, __dmul_rn(h6, sx)), __dadd_rn(yb.y, __dmul_rn(h6, sy)));
      }
    }
    return;
  }
  if (a.mode == 2) {  // update_dm_euler: dm += 0.5 dt (ddmdt + ddmdt^dagger); f^T through shared memory
#pragma unroll
    for (int j = 0; j < NB; ++j) sf[g][i * NB + j] = f[j];
    __syncwarp(gm);
    const double hf = 0.5 * a.tref[1];
#pragma unroll
    for (int j = 0; j < NB; ++j) {
      const double2 v = cscale_rn(hf, cadd_rn(f[j], cconj(sf[g][j * NB + i])));
      a.ybase[base + j] = cadd_rn(a.ybase[base + j], v);
    }
  }
}

// advance the device step counter after the last kernel of a step
__global__ void k_step_inc(long long* step) {
  if (threadIdx.x == 0 && blockIdx.x == 0) *step += 1;
}

// out = base + h * (c0 K0 + c1 K1 + ...), left to right; premul: (c0*h)*K0 form of the first stage
__global__ void k_rk_comb(size_t n, const double* __restrict__ base, const double* __restrict__ K, size_t kstride,
                          int nk_terms, const int* __restrict__ kidx, const double* __restrict__ coef, double h,
                          int premul, double* __restrict__ out) {
  const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  if (premul) {  // y + c*h*k
    out[i] = __dadd_rn(base[i], __dmul_rn(__dmul_rn(coef[0], h), K[kidx[0] * kstride + i]));
    return;
  }
  double s = __dmul_rn(coef[0], K[kidx[0] * kstride + i]);
  for (int j = 1; j < nk_terms; ++j) s = __dadd_rn(s, __dmul_rn(coef[j], K[kidx[j] * kstride + i]));
  out[i] = __dadd_rn(base[i], __dmul_rn(h, s));
}

// yerr = h * (e1 K1 + e3 K3 + ...) and per-block max of |yerr| / (eps_rel * |y| + eps_abs)
__global__ void k_rk_err(size_t n, const double* __restrict__ y, const double* __restrict__ K, size_t kstride,
                         int nk_terms, const int* __restrict__ kidx, const double* __restrict__ coef, double h,
                         double eps_abs, double eps_rel, double* __restrict__ blockmax) {
  __shared__ double sm[256];
  const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  double r = 2.2250738585072014e-308;
  if (i < n) {
    double s = __dmul_rn(coef[0], K[kidx[0] * kstride + i]);
    for (int j = 1; j < nk_terms; ++j) s = __dadd_rn(s, __dmul_rn(coef[j], K[kidx[j] * kstride + i]));
    const double yerr = __dmul_rn(h, s);
    const double D0 = __dadd_rn(__dmul_rn(eps_rel, __dadd_rn(fabs(y[i]), 0.0)), eps_abs);
    r = fabs(yerr) / fabs(D0);
  }
  sm[threadIdx.x] = r;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) sm[threadIdx.x] = fmax(sm[threadIdx.x], sm[threadIdx.x + s]);
    __syncthreads();
  }
  if (threadIdx.x == 0) blockmax[blockIdx.x] = sm[0];
}

// observable totals (observable.h:356-366), per-block partial sums; block b covers k in a stripe
__global__ void k_measure(int nk, int nbdm, int bs, int be, const double2* __restrict__ obs, const double* __restrict__ f,
                          const double* __restrict__ edm, double t, int picture, const double2* __restrict__ y,
                          double* __restrict__ part, size_t ystride = 0) {
  __shared__ double s1[256], s2[256];
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  y += (size_t)blockIdx.y * ystride;        // state of the batch
  part += (size_t)blockIdx.y * gridDim.x * 2;
  double ob = 0.0, oba = 0.0;
  if (k < nk) {
    const int nd = nbdm;
    for (int i = bs; i < be; ++i) {
      double o1 = 0.0, o2 = 0.0;
      for (int b = 0; b < nd; ++b) {
        const double2 okib = obs[(size_t)k * nd * nd + i * nd + b];
        const double2 okt = (i == b || picture == 1) ? okib : cmul_rn(okib, ccis((edm[k * nd + i] - edm[k * nd + b]) * t));
        double2 dkbi = y[(size_t)k * nd * nd + b * nd + i];
        if (i == b) dkbi = mk2(__dsub_rn(dkbi.x, f[k * nd + i]), dkbi.y);
        o1 = __dadd_rn(o1, cmul_rn(okt, dkbi).x);
        o2 = __dadd_rn(o2, cmul_rn(okib, dkbi).x);
      }
      ob = __dadd_rn(ob, o1);
      oba = __dadd_rn(oba, o2);
    }
  }
  s1[threadIdx.x] = ob;
  s2[threadIdx.x] = oba;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) {
      s1[threadIdx.x] += s1[threadIdx.x + s];
      s2[threadIdx.x] += s2[threadIdx.x + s];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    part[2 * blockIdx.x] = s1[0];
    part[2 * blockIdx.x + 1] = s2[0];
  }
}

// non-finite scan of the state
__global__ void k_nan_scan(size_t n, const double* __restrict__ y, int* __restrict__ flag) {
  const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i < n && !isfinite(y[i])) atomicOr(flag, 1);
}

}  // namespace dmd
