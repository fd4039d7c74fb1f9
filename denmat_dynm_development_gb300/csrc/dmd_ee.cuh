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
// integer mesh arithmetic and a dense mesh table, energy window by per-k band ranges) and append
// the candidates to a warp buffer. Phase 2: groups of G = 2 nb^2 lanes take one candidate each
// (4 groups for nb = 2, one for nb = 4); lane (w, r), r = (i1, i3), builds one row of A into shared
// memory, then forms its own A1rho (w = 0) or A1rhobar (w = 1) row and accumulates P1ee or P2ee
// over (i2, i4) in registers. The groups' partial sums are added with shuffles at the end. FP64
// throughout (FMA in the contractions).
#pragma once
#include "dmd_common.cuh"
#include "dmd_kernels.cuh"

namespace dmd {

enum { EE_UNSCREENED = 0, EE_DEBYE = 1, EE_BECHSTEDT = 2 };

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
  const double2* erng;               // [nk] (min, max) of the window energies
  const double2* dm;                 // [nk][nb^2] window density matrix (Schrodinger picture), or null
  const double2* dm1;                // [nk][nb^2] 1 - dm
  const double* f;                   // [nk][nb] occupations when dm is null
  const EeScreen* scr;
  double2* Pee;                      // [npair][2][nb^4]: P1ee, P2ee (prefactor included)
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

// coulomb_model::vq, static branches (Coulomb_Model.h:632-660), q = k_i - k_j
__device__ __forceinline__ double ee_vq(const EeArgs& a, const EeScreen& s, int ki, int kj) {
  const double* x = a.kvec + 3 * ki;
  const double* y = a.kvec + 3 * kj;
  const double q2 = ee_q2(a, x[0] - y[0], x[1] - y[1], x[2] - y[2]);
  if (a.formula == EE_UNSCREENED) return q2 < 1e-20 ? 0.0 : s.prefac_vq / q2;
  if (a.formula == EE_DEBYE) return s.prefac_vq / (s.qscr2_debye + q2);
  if (q2 < 1e-20) return 0.0;
  const double epsq = 1 + 1. / (s.fac0 + s.fac2 * q2 + s.fac4 * q2 * q2);
  return s.prefac_vq_bare / epsq / q2;
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

// the window density matrix in the Schrodinger picture and 1 - rho from the state y (one thread per
// (k, i, j) of the window): electronphonon::reset_scatt's window copy (ElectronPhonon.cpp:19-28)
// and add_scatt_contrib's conversion (ElectronPhonon.cpp:56-66)
template <int NB>
__global__ void k_ee_dm(int nk, int nbdm, int bs, const double2* __restrict__ y, const double* __restrict__ ew,
                        TimeArg ta, int interaction, double2* __restrict__ dm, double2* __restrict__ dm1) {
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
  if (i == j) {  // zhemm reads the diagonal as real (BLAS ZHEMM)
    dm[idx] = mk2(v.x, 0.0);
    dm1[idx] = mk2(1.0 - v.x, 0.0);
  } else {
    const double2 u = i < j ? v : cconj(v);  // lower = conj(upper)
    dm[idx] = u;
    dm1[idx] = mk2(-u.x, -u.y);
  }
}

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

template <int NB>
struct EeSmem {
  static constexpr int NB2 = NB * NB, NB4 = NB2 * NB2, G = 2 * NB2, NG = 32 / G;
  double2 o12[NB2];
  double2 o34[NG][NB2], o14[NG][NB2], o32[NG][NB2];
  double2 A[NG][NB4];
  int2 cand[64];
};

template <int NB>
__global__ void __launch_bounds__(128) k_ee_pairs(EeArgs a) {
  typedef EeSmem<NB> S;
  constexpr int NB2 = S::NB2, NB4 = S::NB4, G = S::G, NG = S::NG;
  __shared__ S smem_all[4];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  S& sm = smem_all[warp];
  const int p = blockIdx.x * 4 + warp;
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
  if (lane < NB2) {  // o12 = vq(k1 - k2) U_k1^dag U_k2
    const double vq = ee_vq(a, scr, k1, k2);
    const double2 o = ee_ovlp<NB>(a, k1, k2, lane / NB, lane % NB);
    sm.o12[lane] = mk2(vq * o.x, vq * o.y);
  }
  double2 acc[NB2];
#pragma unroll
  for (int e = 0; e < NB2; ++e) acc[e] = mk2(0, 0);
  const int4 i1v = a.kidx[k1], i2v = a.kidx[k2];
  const double2 r1 = a.erng[k1], r2 = a.erng[k2];
  const double* e1 = a.ew + (size_t)k1 * NB;
  const double* e2 = a.ew + (size_t)k2 * NB;
  int ncand = 0;
  for (int c0 = 0; c0 < a.nk; c0 += 32) {
    // phase 1: candidates k3 of this chunk
    const int k3 = c0 + lane;
    int k4 = -1;
    if (k3 < a.nk && !(a.antisym && k1 == k2 && k2 == k3)) {
      const int4 i3v = a.kidx[k3];
      int m0 = (i1v.x + i3v.x - i2v.x) % a.kmesh[0], m1 = (i1v.y + i3v.y - i2v.y) % a.kmesh[1],
          m2 = (i1v.z + i3v.z - i2v.z) % a.kmesh[2];
      m0 += m0 < 0 ? a.kmesh[0] : 0;
      m1 += m1 < 0 ? a.kmesh[1] : 0;
      m2 += m2 < 0 ? a.kmesh[2] : 0;
      k4 = a.kmap[((size_t)m0 * a.kmesh[1] + m1) * a.kmesh[2] + m2];
      if (k4 >= 0) {  // some band combination may be inside the window (exact test in phase 2)
        const double2 r3 = a.erng[k3], r4 = a.erng[k4];
        const double lo = r1.x - r2.y + r3.x - r4.y, hi = r1.y - r2.x + r3.y - r4.x;
        const double tol = 1e-12 * (fabs(lo) + fabs(hi)) + 1e-300;
        if (!(lo < a.ethr + tol && hi > -a.ethr - tol)) k4 = -1;
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
        // overlaps of this candidate: lanes w = 0 build o34 (and o14), lanes w = 1 o32
        const int c = r / NB, d = r % NB;
        if (w == 0) {
          sm.o34[grp][r] = ee_ovlp<NB>(a, ka, kb, c, d);
          if (a.antisym) {
            const double vq = ee_vq(a, scr, k1, kb);
            const double2 o = ee_ovlp<NB>(a, k1, kb, c, d);
            sm.o14[grp][r] = mk2(vq * o.x, vq * o.y);
          }
        } else if (a.antisym) {
          sm.o32[grp][r] = ee_ovlp<NB>(a, ka, k2, c, d);
        }
      }
      __syncwarp();
      if (act && w == 0) {  // row r = (i1, i3) of A (calc_delta, calc_mee[_ex], calc_A)
        const double* e3 = a.ew + (size_t)ka * NB;
        const double* e4 = a.ew + (size_t)kb * NB;
        const double2 m12 = sm.o12[i1 * NB + i3];
#pragma unroll
        for (int cd = 0; cd < NB2; ++cd) {
          const int c = cd / NB, d = cd % NB;
          const double de = e1[i1] - e2[i3] + e3[c] - e4[d];
          double2 v = mk2(0, 0);
          if (fabs(de) < a.ethr) {
            double2 mee = cmul_rn(m12, sm.o34[grp][cd]);
            if (a.antisym) {
              const double2 mex = cmul_rn(sm.o14[grp][i1 * NB + d], sm.o32[grp][c * NB + i3]);
              mee = mk2(-0.5 * mex.x + 0.5 * mee.x, -0.5 * mex.y + 0.5 * mee.y);
            }
            v = cscale_rn(exp(a.prefac_exp * (de * de)), mee);
          }
          sm.A[grp][r * NB2 + cd] = v;
        }
      }
      __syncwarp();
      if (act) {
        // X = dm1_k3 A[(i1,i3)] dm_k4 (w = 0) or dm_k3 A[(i3,i1)] dm1_k4 (w = 1)
        const double2* Ar = &sm.A[grp][(w == 0 ? r : i3 * NB + i1) * NB2];
        double2 X[NB2];
        if (a.dm) {
          const double2* L = (w == 0 ? a.dm1 : a.dm) + (size_t)ka * NB2;
          const double2* R = (w == 0 ? a.dm : a.dm1) + (size_t)kb * NB2;
          double2 T[NB2];
#pragma unroll
          for (int i = 0; i < NB; ++i)
#pragma unroll
            for (int j = 0; j < NB; ++j) {
              double2 t = mk2(0, 0);
#pragma unroll
              for (int m = 0; m < NB; ++m) t = cfma(Ar[i * NB + m], R[m * NB + j], t);
              T[i * NB + j] = t;
            }
#pragma unroll
          for (int i = 0; i < NB; ++i)
#pragma unroll
            for (int j = 0; j < NB; ++j) {
              double2 t = mk2(0, 0);
#pragma unroll
              for (int m = 0; m < NB; ++m) t = cfma(L[i * NB + m], T[m * NB + j], t);
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
              X[i * NB + j] = cscale_rn(sr, cscale_rn(sl, Ar[i * NB + j]));
            }
        }
        // acc[(i2,i4)] += sum_(i6,i8) X[i6,i8] conj(A[(i2,i4) or (i4,i2)][i6,i8])
#pragma unroll
        for (int i2 = 0; i2 < NB; ++i2)
#pragma unroll
          for (int i4 = 0; i4 < NB; ++i4) {
            const double2* B = &sm.A[grp][(w == 0 ? i2 * NB + i4 : i4 * NB + i2) * NB2];
            double2 t = acc[i2 * NB + i4];
#pragma unroll
            for (int q = 0; q < NB2; ++q) {
              const double2 b = B[q];
              t = mk2(fma(X[q].x, b.x, fma(X[q].y, b.y, t.x)), fma(X[q].y, b.x, fma(-X[q].x, b.y, t.y)));
            }
            acc[i2 * NB + i4] = t;
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
  // add the groups' partial sums (lanes with the same role)
#pragma unroll
  for (int off = G; off < 32; off <<= 1)
#pragma unroll
    for (int e = 0; e < NB2; ++e) {
      acc[e].x += __shfl_xor_sync(FULL, acc[e].x, off);
      acc[e].y += __shfl_xor_sync(FULL, acc[e].y, off);
    }
  if (grp == 0) {
#pragma unroll
    for (int i2 = 0; i2 < NB; ++i2)
#pragma unroll
      for (int i4 = 0; i4 < NB; ++i4) {
        const double2 v = acc[i2 * NB + i4];
        out[w * NB4 + ((i1 * NB + i2) * NB + i3) * NB + i4] = mk2(a.prefac * v.x, a.prefac * v.y);
      }
  }
}

}  // namespace dmd
