// Adjoint (reverse-mode) kernels of the Lindblad right-hand side, FP64.
//
// With the real inner product <A, B> = Re sum conj(A) B over all entries, the vector-Jacobian
// product of f at a state u for a cotangent v (same layout as the state) is formed in three steps,
// all written for complex n x n blocks (n = nb^2 for the pair operators):
//
//   local (per k):  cbar = (prefac/2)(v + v^H) on the e-ph window;
//                   c = (1 - rho) Pdm - dm1P rho, Pdm = D o X, dm1P = D o Y  (forward sums at u)
//                   Xbar = conj(D) o ((1 - rho)^H cbar),  Ybar = conj(D) o (-cbar rho^H)
//                   rho_bar = -cbar Pdm^H - dm1P^H cbar   (+ the coherent term's adjoint)
//   pairs:          the transposed contraction of the forward pair loop (evolve_eph.cpp:49-106):
//                   rt_bar[k'] += P1^H Xbar[k],  st_bar[k'] += conj(P2) Ybar[k]  and, for k < k',
//                   rt_bar[k] += P2^T Xbar[k'],  st_bar[k] += P1 Ybar[k'];
//                   and the gradient with respect to the stored operators,
//                   G1 += conj(Xbar[k]) rt[k']^T + conj(st[k]) Ybar[k']^T,
//                   G2 += st[k'] conj(Ybar[k])^T + Xbar[k'] conj(rt[k])^T   (dJ = Re sum(dP o G))
//   combine:        rho_bar += D o rt_bar - D o st_bar   (rt = conj(D) o rho, st = conj(D) o (1 - rho))
//
// The forward finish reads rho and 1 - rho through their upper triangles (zhemm); on Hermitian
// states, where the trajectory lives, that map equals the plain-product map used here, so the
// gradients with respect to the operators (and the initial state's Hermitian part) are exact.
#pragma once
#include "dmd_common.cuh"
#include "dmd_kernels.cuh"
#include "dmd_pairs_cb.cuh"
#include "dmd_tma.cuh"

namespace dmd {

struct AdjLocalArgs {
  int nk, nbdm, bs, picture, phase, herm, lin, want_coh;
  double prefac, t;
  const double2* u;     // state the RHS was evaluated on [k][nbdm^2]
  const double2* vbar;  // cotangent of the RHS [k][nbdm^2]
  const double2* acc;   // forward sums X', Y' at u ([.][2][NB2], by pos[k] when pos is set)
  const int* pos;
  const double2* ph;    // phases D_k of this evaluation (or null)
  const double* ew;     // [nk][NB]
  const double* edm;    // [nk][nbdm]
  const double2* H;     // coherent H_k (or null)
  double2* Xb;          // [k][NB2]
  double2* Yb;
  double2* rt;          // forward coordinates conj(D) o rho, conj(D) o (1 - rho) [k][NB2]
  double2* st;
  double2* ubar;        // [k][nbdm^2]: coherent adjoint + local e-ph adjoint
  double2* rtb;         // transposed-contraction sums [k][NB2], zeroed here for the pair pass (or null)
  double2* stb;
  float4* dfv;          // double-float forms (x, S(x)) of Xb, Yb, rt, st for k_adj_pairs_df (or null)
  size_t nk2;           // nk NB2
};

__device__ __forceinline__ double2 cmulc(double2 a, double2 b) {  // conj(a) * b
  return mk2(a.x * b.x + a.y * b.y, a.x * b.y - a.y * b.x);
}
__device__ __forceinline__ double2 cadd(double2 a, double2 b) { return mk2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ double2 csub(double2 a, double2 b) { return mk2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ double2 cmul(double2 a, double2 b) {
  return mk2(fma(a.x, b.x, -a.y * b.y), fma(a.x, b.y, a.y * b.x));
}

// a complex as a double-float (re_h, im_h, re_l, im_l)
__device__ __forceinline__ float4 dfc_split(double re, double im) {
  const float rh = __double2float_rn(re), ih = __double2float_rn(im);
  return make_float4(rh, ih, __double2float_rn(__dsub_rn(re, (double)rh)), __double2float_rn(__dsub_rn(im, (double)ih)));
}

template <int NB>
__global__ void k_adj_local(AdjLocalArgs a) {
  constexpr int NB2 = NB * NB;
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= a.nk) return;
  const int nd = a.nbdm, nd2 = nd * nd;
  const double2* yk = a.u + (size_t)k * nd2;
  const double2* vk = a.vbar + (size_t)k * nd2;
  double2* ub = a.ubar + (size_t)k * nd2;
  if (a.rtb)
    for (int e = 0; e < NB2; ++e) {
      a.rtb[(size_t)k * NB2 + e] = mk2(0.0, 0.0);
      a.stb[(size_t)k * NB2 + e] = mk2(0.0, 0.0);
    }
  for (int e = 0; e < nd2; ++e) ub[e] = mk2(0.0, 0.0);
  // coherent term -i[H(t), rho]: adjoint i(H v - v H) (H Hermitian, read from its upper triangle)
  if (a.want_coh) {
    const double* ek = a.edm + (size_t)k * nd;
    if (a.H) {
      const double2* Hk = a.H + (size_t)k * nd2;
      for (int i = 0; i < nd; ++i)
        for (int j = 0; j < nd; ++j) {
          double2 s = mk2(0.0, 0.0);
          for (int l = 0; l < nd; ++l) {
            // Ht(i, l) and Ht(l, j) of the forward: upper triangle, interaction-picture phase
            double2 hil, hlj;
            {
              const int r = i < l ? i : l, c = i < l ? l : i;
              double2 hv = (r == c) ? mk2(Hk[r * nd + r].x, 0.0) : Hk[r * nd + c];
              if (a.picture == 0 && r != c) hv = cmul(hv, ccis((ek[r] - ek[c]) * a.t));
              hil = (i <= l) ? hv : cconj(hv);
            }
            {
              const int r = l < j ? l : j, c = l < j ? j : l;
              double2 hv = (r == c) ? mk2(Hk[r * nd + r].x, 0.0) : Hk[r * nd + c];
              if (a.picture == 0 && r != c) hv = cmul(hv, ccis((ek[r] - ek[c]) * a.t));
              hlj = (l <= j) ? hv : cconj(hv);
            }
            s = cadd(s, csub(cmul(hil, vk[l * nd + j]), cmul(vk[i * nd + l], hlj)));
          }
          ub[i * nd + j] = mk2(-s.y, s.x);  // i * s
        }
    } else if (a.picture == 1) {  // -i[E, rho]: adjoint i (e_i - e_j) v_ij
      for (int i = 0; i < nd; ++i)
        for (int j = 0; j < nd; ++j) {
          const double w = ek[i] - ek[j];
          const double2 v = vk[i * nd + j];
          ub[i * nd + j] = mk2(-w * v.y, w * v.x);
        }
    }
  }
  // e-ph window
  const double2* Xs = a.acc + (size_t)(a.pos ? a.pos[k] : k) * 2 * NB2;
  double2 X[NB2], Y[NB2];
  for (int e = 0; e < NB2; ++e) {
    X[e] = Xs[e];
    Y[e] = Xs[NB2 + e];
  }
  if (a.herm) {  // X = (M^H)^-1 X'
    for (int i = 0; i < NB; ++i)
      for (int j = i + 1; j < NB; ++j) {
        const double2 xu = X[i * NB + j], xl = X[j * NB + i], yu = Y[i * NB + j], yl = Y[j * NB + i];
        X[i * NB + j] = mk2(0.5 * (xu.x - xl.y), 0.5 * (xu.y + xl.x));
        X[j * NB + i] = mk2(0.5 * (xu.x + xl.y), 0.5 * (xu.y - xl.x));
        Y[i * NB + j] = mk2(0.5 * (yu.x - yl.y), 0.5 * (yu.y + yl.x));
        Y[j * NB + i] = mk2(0.5 * (yu.x + yl.y), 0.5 * (yu.y - yl.x));
      }
  }
  const double* ew = a.ew + (size_t)k * NB;
  const double pf = 0.5 * a.prefac;
  double2 D[NB2], r[NB2], om[NB2], cb[NB2], Pdm[NB2], dmP[NB2];
  for (int i = 0; i < NB; ++i)
    for (int j = 0; j < NB; ++j) {
      const int e = i * NB + j;
      D[e] = mk2(1.0, 0.0);
      if (a.phase && i != j) D[e] = a.ph ? a.ph[(size_t)k * NB2 + e] : ccis((ew[i] - ew[j]) * a.t);
      r[e] = yk[(a.bs + i) * nd + a.bs + j];
      om[e] = (i == j) ? mk2(1.0 - r[e].x, -r[e].y) : mk2(-r[e].x, -r[e].y);
      const double2 v1 = vk[(a.bs + i) * nd + a.bs + j], v2 = vk[(a.bs + j) * nd + a.bs + i];
      cb[e] = mk2(pf * (v1.x + v2.x), pf * (v1.y - v2.y));
      Pdm[e] = cmul(D[e], X[e]);
      dmP[e] = cmul(D[e], Y[e]);
    }
  double2* Xbk = a.Xb + (size_t)k * NB2;
  double2* Ybk = a.Yb + (size_t)k * NB2;
  for (int i = 0; i < NB; ++i)
    for (int j = 0; j < NB; ++j) {
      const int e = i * NB + j;
      double2 pb = mk2(0.0, 0.0), db = mk2(0.0, 0.0), rb = mk2(0.0, 0.0);
      if (a.lin) {
        pb = cb[e];
      } else {
        for (int l = 0; l < NB; ++l) {
          pb = cadd(pb, cmulc(om[l * NB + i], cb[l * NB + j]));               // (1 - rho)^H cbar
          db = csub(db, cmul(cb[i * NB + l], cconj(r[j * NB + l])));          // -cbar rho^H
          rb = csub(rb, cmul(cb[i * NB + l], cconj(Pdm[j * NB + l])));        // -cbar Pdm^H
          rb = csub(rb, cmulc(dmP[l * NB + i], cb[l * NB + j]));              // -dm1P^H cbar
        }
      }
      Xbk[e] = cmulc(D[e], pb);
      Ybk[e] = cmulc(D[e], db);
      a.rt[(size_t)k * NB2 + e] = cmulc(D[e], r[e]);
      a.st[(size_t)k * NB2 + e] = cmulc(D[e], om[e]);
      if (a.dfv) {  // (x, S(x)), S(x) = (Im x, -Re x), of the four vectors
        const double2 v4[4] = {Xbk[e], Ybk[e], a.rt[(size_t)k * NB2 + e], a.st[(size_t)k * NB2 + e]};
        for (int v = 0; v < 4; ++v) {
          float4* o = a.dfv + 2 * ((size_t)v * a.nk2 + (size_t)k * NB2 + e);
          o[0] = dfc_split(v4[v].x, v4[v].y);
          o[1] = dfc_split(v4[v].y, -v4[v].x);
        }
      }
      double2& o = ub[(a.bs + i) * nd + a.bs + j];
      o = cadd(o, rb);
    }
}

// Transposed pair contraction and the operator gradient. One thread per (pair, index b).
template <int NB>
__global__ void k_adj_pairs(long long npair, const int2* __restrict__ kk, const double2* __restrict__ P,
                            const double2* __restrict__ Xb, const double2* __restrict__ Yb,
                            const double2* __restrict__ rt, const double2* __restrict__ st, double* __restrict__ rtb,
                            double* __restrict__ stb, double2* __restrict__ G) {
  constexpr int NB2 = NB * NB, NB4 = NB2 * NB2;
  const long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (idx >= npair * NB2) return;
  const long long p = idx / NB2;
  const int b = (int)(idx - p * NB2);
  const int2 kp2 = kk[p];
  const int k = kp2.x, kq = kp2.y;
  const double2* P1 = P + (size_t)p * 2 * NB4;
  const double2* P2 = P1 + NB4;
  double2* G1 = G + (size_t)p * 2 * NB4;
  double2* G2 = G1 + NB4;
  const double2* Xk = Xb + (size_t)k * NB2;
  const double2* Yk = Yb + (size_t)k * NB2;
  const double2* rtq = rt + (size_t)kq * NB2;
  const double2* stq = st + (size_t)kq * NB2;
  double2 a1 = mk2(0.0, 0.0), a2 = mk2(0.0, 0.0);
  for (int a = 0; a < NB2; ++a) {
    a1 = cadd(a1, cmulc(P1[a * NB2 + b], Xk[a]));  // P1^H Xbar[k]
    a2 = cadd(a2, cmulc(P2[b * NB2 + a], Yk[a]));  // conj(P2) Ybar[k]
  }
  atomicAdd(&rtb[((size_t)kq * NB2 + b) * 2], a1.x);
  atomicAdd(&rtb[((size_t)kq * NB2 + b) * 2 + 1], a1.y);
  atomicAdd(&stb[((size_t)kq * NB2 + b) * 2], a2.x);
  atomicAdd(&stb[((size_t)kq * NB2 + b) * 2 + 1], a2.y);
  const bool rev = k < kq;
  const double2* Xq = Xb + (size_t)kq * NB2;
  const double2* Yq = Yb + (size_t)kq * NB2;
  const double2* rtk = rt + (size_t)k * NB2;
  const double2* stk = st + (size_t)k * NB2;
  for (int a = 0; a < NB2; ++a) {
    double2 g1 = cmulc(Xk[a], rtq[b]);                      // conj(Xbar[k][a]) rt[k'][b]
    double2 g2 = cmulc(Yk[b], stq[a]);                      // st[k'][a] conj(Ybar[k][b])
    if (rev) {
      g1 = cadd(g1, cmulc(stk[a], Yq[b]));                  // conj(st[k][a]) Ybar[k'][b]
      g2 = cadd(g2, cmulc(rtk[b], Xq[a]));                  // Xbar[k'][a] conj(rt[k][b])
    }
    G1[a * NB2 + b] = cadd(G1[a * NB2 + b], g1);
    G2[a * NB2 + b] = cadd(G2[a * NB2 + b], g2);
  }
  if (rev) {
    double2 a3 = mk2(0.0, 0.0), a4 = mk2(0.0, 0.0);
    for (int a = 0; a < NB2; ++a) {
      a3 = cadd(a3, cmul(P2[a * NB2 + b], Xq[a]));          // P2^T Xbar[k']
      a4 = cadd(a4, cmul(P1[b * NB2 + a], Yq[a]));          // P1 Ybar[k']
    }
    atomicAdd(&rtb[((size_t)k * NB2 + b) * 2], a3.x);
    atomicAdd(&rtb[((size_t)k * NB2 + b) * 2 + 1], a3.y);
    atomicAdd(&stb[((size_t)k * NB2 + b) * 2], a4.x);
    atomicAdd(&stb[((size_t)k * NB2 + b) * 2 + 1], a4.y);
  }
}

// ---------------------------------------------------------------------------------------------
// Double-float form of the transposed pair contraction and of the operator gradient (handles whose
// forward sums are double-float): the same sums as k_adj_pairs with every product error-free
// transformed on the FP32 pipes (ArithDF's packed (re, im) steps, ~2^-44 relative) instead of on the
// FP64 pipe; the gradient G is kept as double-float (re_h, im_h, re_l, im_l) per element,
// renormalised after every update, and converted to FP64 once at the end (k_df_to_f64).
// A complex product is two packed multiply-adds: with S(x) = (Im x, -Re x),
//   conj(p) x = x o (Re p, Re p) + S(x) o (Im p, Im p),   p x = x o (Re p, Re p) - S(x) o (Im p, Im p),
//   conj(x) y = y o (Re x, Re x) + S(y) o (Im x, Im x).
// ---------------------------------------------------------------------------------------------
// broadcast of the real / imaginary part of a double-float complex (re_h, im_h, re_l, im_l)
__device__ __forceinline__ float4 df_bre(const float4& x) { return make_float4(x.x, x.x, x.z, x.z); }
__device__ __forceinline__ float4 df_bim(const float4& x) { return make_float4(x.y, x.y, x.w, x.w); }
__device__ __forceinline__ float4 df_bimn(const float4& x) { return make_float4(-x.y, -x.y, -x.w, -x.w); }

// pair operators [pair][P1 | P2][nb^4] (complex128) -> double-float copy, one thread per element
__global__ void k_p_to_df(size_t n, const double2* __restrict__ P, float4* __restrict__ out) {
  const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i < n) out[i] = dfc_split(P[i].x, P[i].y);
}

// double-float complex (re_h, im_h, re_l, im_l) -> complex128 in place (its conjugate when conj)
__global__ void k_df_to_f64(size_t n, float4* __restrict__ g, int conj) {
  const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float4 v = g[i];
  const double im = (double)v.y + (double)v.w;
  reinterpret_cast<double2*>(g)[i] = mk2((double)v.x + (double)v.z, conj ? -im : im);
}

// out[j][e] = G[j][m][e] for the n = cnt nb4 elements of a chunk of pairs (G: [pair][2][nb4])
__global__ void k_gather_half(size_t n, size_t nb4, const double2* __restrict__ G, int m, double2* __restrict__ out) {
  const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const size_t j = i / nb4, e = i - j * nb4;
  out[i] = G[(j * 2 + m) * nb4 + e];
}

// g = conj(g) in place
__global__ void k_conj(size_t n, double2* __restrict__ g) {
  const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i < n) g[i].y = -g[i].y;
}

// One thread per (pair, index b), as k_adj_pairs. dfv: k_adj_local's double-float forms; P: double-float pair
// operators; G: double-float gradient [pair][G1 | G2][nb^4].
template <int NB>
__global__ void __launch_bounds__(128) k_adj_pairs_df(long long npair, const int2* __restrict__ kk,
                                                      const float4* __restrict__ P, const float4* __restrict__ dfv,
                                                      size_t nk2, double* __restrict__ rtb, double* __restrict__ stb,
                                                      float4* __restrict__ G) {
  constexpr int NB2 = NB * NB, NB4 = NB2 * NB2;
  typedef ArithDF D;
  const long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (idx >= npair * NB2) return;
  const long long p = idx / NB2;
  const int b = (int)(idx - p * NB2);
  const int2 kp2 = kk[p];
  const int k = kp2.x, kq = kp2.y;
  const float4* P1 = P + (size_t)p * 2 * NB4;
  const float4* P2 = P1 + NB4;
  float4* G1 = G + (size_t)p * 2 * NB4;
  float4* G2 = G1 + NB4;
  // element e of vector v at k: (x, S(x)) at dfv[2 ((v nk + k) NB2 + e)]
  auto vx = [&](int v, int kk_, int e) -> const float4* { return dfv + 2 * ((size_t)v * nk2 + (size_t)kk_ * NB2 + e); };
  D::acc a1, a2;
  D::zero(a1);
  D::zero(a2);
#pragma unroll
  for (int a = 0; a < NB2; ++a) {
    const float4 x = P1[a * NB2 + b];  // conj(P1[a][b]) Xbar[k][a]
    const float4* X = vx(0, k, a);
    D::pmac(a1, X[0], df_bre(x));
    D::pmac(a1, X[1], df_bim(x));
    const float4 y = P2[b * NB2 + a];  // conj(P2[b][a]) Ybar[k][a]
    const float4* Y = vx(1, k, a);
    D::pmac(a2, Y[0], df_bre(y));
    D::pmac(a2, Y[1], df_bim(y));
  }
  double* ro = rtb + ((size_t)kq * NB2 + b) * 2;
  double* so = stb + ((size_t)kq * NB2 + b) * 2;
  atomicAdd(ro, D::re_d(a1));
  atomicAdd(ro + 1, D::im_d(a1));
  atomicAdd(so, D::re_d(a2));
  atomicAdd(so + 1, D::im_d(a2));
  const bool rev = k < kq;
  // G1[a][b] += conj(Xbar[k][a]) rt[k'][b] (+ conj(st[k][a]) Ybar[k'][b]);
  // G2[a][b] += conj(Ybar[k][b]) st[k'][a] (+ conj(rt[k][b]) Xbar[k'][a])
  const float4* rq = vx(2, kq, b);
  const float4* Yq = vx(1, kq, b);
  const float4 Ykb = vx(1, k, b)[0];
  const float4 rkb = vx(2, k, b)[0];
#pragma unroll
  for (int a = 0; a < NB2; ++a) {
    float4 g = G1[a * NB2 + b];
    D::acc c = {make_float2(g.x, g.y), make_float2(g.z, g.w)};
    const float4 Xka = vx(0, k, a)[0];
    D::pmac(c, rq[0], df_bre(Xka));
    D::pmac(c, rq[1], df_bim(Xka));
    if (rev) {
      const float4 ska = vx(3, k, a)[0];
      D::pmac(c, Yq[0], df_bre(ska));
      D::pmac(c, Yq[1], df_bim(ska));
    }
    D::renorm(c);
    G1[a * NB2 + b] = make_float4(c.h.x, c.h.y, c.l.x, c.l.y);
    g = G2[a * NB2 + b];
    c = {make_float2(g.x, g.y), make_float2(g.z, g.w)};
    const float4* sq = vx(3, kq, a);
    D::pmac(c, sq[0], df_bre(Ykb));
    D::pmac(c, sq[1], df_bim(Ykb));
    if (rev) {
      const float4* Xq = vx(0, kq, a);
      D::pmac(c, Xq[0], df_bre(rkb));
      D::pmac(c, Xq[1], df_bim(rkb));
    }
    D::renorm(c);
    G2[a * NB2 + b] = make_float4(c.h.x, c.h.y, c.l.x, c.l.y);
  }
  if (rev) {
    D::acc a3, a4;
    D::zero(a3);
    D::zero(a4);
#pragma unroll
    for (int a = 0; a < NB2; ++a) {
      const float4 x = P2[a * NB2 + b];  // P2[a][b] Xbar[k'][a]
      const float4* X = vx(0, kq, a);
      D::pmac(a3, X[0], df_bre(x));
      D::pmac(a3, X[1], df_bimn(x));
      const float4 y = P1[b * NB2 + a];  // P1[b][a] Ybar[k'][a]
      const float4* Y = vx(1, kq, a);
      D::pmac(a4, Y[0], df_bre(y));
      D::pmac(a4, Y[1], df_bimn(y));
    }
    double* r2 = rtb + ((size_t)k * NB2 + b) * 2;
    double* s2 = stb + ((size_t)k * NB2 + b) * 2;
    atomicAdd(r2, D::re_d(a3));
    atomicAdd(r2 + 1, D::im_d(a3));
    atomicAdd(s2, D::re_d(a4));
    atomicAdd(s2 + 1, D::im_d(a4));
  }
}

// nb = 4: one warp per pair, a pair's double-float operators (8 KB) and gradient (8 KB) staged in
// shared memory by bulk copies (TMA unit) in a 2-stage ring per warp, the per-k vectors of both
// k-points in shared memory. The same sums as k_adj_pairs_df: lanes 0-15 form conj(P1)^T Xbar[k] and
// conj(P2) Ybar[k] for b = lane, lanes 16-31 P2^T Xbar[k'] and P1 Ybar[k'] for b = lane - 16 (k < k'),
// reading rows with a per-lane rotation so that the 16 lanes hit distinct banks; then every lane
// updates 8 elements of G1 and 8 of G2 and stores them to global memory (coalesced). A warp takes a
// contiguous run of pairs. Waits are bounded; a timeout sets *errflag and the warp drains its copies.
template <int NST_, int W_ = 4>
struct AdjBulkSmem {
  static constexpr int NB = 4, NB2 = 16, NB4 = 256;
  static constexpr int NST = NST_;  // ring stages per warp
  static constexpr size_t half_bytes = (size_t)2 * NB4 * 16;           // P1 | P2 (or G1 | G2)
  static constexpr size_t stage_bytes = 2 * half_bytes;                 // operators, then gradient
  static constexpr size_t vec_bytes = (size_t)8 * NB2 * 2 * 16;         // 8 vectors x 16 x (x, S(x))
  static constexpr size_t warp_bytes = (NST * stage_bytes + vec_bytes + 8 * NST + 127) / 128 * 128;
  static constexpr int warps = W_;  // warps (pairs in flight) per CTA
  static constexpr size_t cta_bytes = warps * warp_bytes;
};

template <int NST_, int W_>
__global__ void __launch_bounds__(32 * W_, 2) k_adj_pairs_bulk4(long long npair, const int2* __restrict__ kk,
                                                                  const float4* __restrict__ P,
                                                                  const float4* __restrict__ dfv, size_t nk2,
                                                                  double* __restrict__ rtb, double* __restrict__ stb,
                                                                  float4* __restrict__ G,
                                                                  unsigned int* __restrict__ errflag) {
  typedef AdjBulkSmem<NST_, W_> S;
  typedef ArithDF D;
  constexpr int NB2 = S::NB2, NB4 = S::NB4, NST = S::NST;
  constexpr unsigned FULL = 0xffffffffu;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  const int wib = threadIdx.x >> 5, lane = threadIdx.x & 31;
  unsigned char* wbase = smem_raw + (size_t)wib * S::warp_bytes;
  float4* const stage0 = (float4*)wbase;                                   // [NST][P1 P2 G1 G2][NB4]
  float4* const vec = (float4*)(wbase + NST * S::stage_bytes);            // [8][NB2][2]
  uint64_t* const bar = (uint64_t*)(wbase + NST * S::stage_bytes + S::vec_bytes);
  const long long nwarps = (long long)gridDim.x * S::warps;
  const long long gw = (long long)blockIdx.x * S::warps + wib;
  const long long per = (npair + nwarps - 1) / nwarps;
  const long long p0 = gw * per, p1 = p0 + per < npair ? p0 + per : npair;
  if (p0 >= p1) return;
  const long long n = p1 - p0;
  if (lane == 0) {
#pragma unroll
    for (int st = 0; st < NST; ++st) mbar_init(&bar[st], 1);
    fence_mbar_init();
  }
  __syncwarp();
  const uint64_t pol = policy_evict_first();
  auto issue = [&](long long i) {  // pair p0 + i into stage i % NST (lane 0)
    if (lane == 0) {
      const int st = (int)(i % NST);
      float4* dst = stage0 + (size_t)st * 4 * NB4;
      const size_t p = (size_t)(p0 + i);
      mbar_arrive_expect_tx(&bar[st], (uint32_t)S::stage_bytes);
      bulk_g2s(dst, P + p * 2 * NB4, (uint32_t)S::half_bytes, &bar[st], pol);
      bulk_g2s(dst + 2 * NB4, G + p * 2 * NB4, (uint32_t)S::half_bytes, &bar[st], pol);
    }
  };
#pragma unroll
  for (int i = 0; i < NST; ++i)
    if (i < n) issue(i);
  long long fail = -1;
  const int half = lane >> 4, b = lane & 15;
#pragma unroll 1
  for (long long i = 0; i < n; ++i) {
    const size_t p = (size_t)(p0 + i);
    const int2 kp2 = kk[p];
    const int k = kp2.x, kq = kp2.y;
    const bool rev = k < kq;
    // per-k vectors: v = 0..3 (Xbar, Ybar, rt, st) at k, 4..7 at k'; 32 float4 (x, S(x)) each
#pragma unroll
    for (int v = 0; v < 8; ++v)
      vec[v * 32 + lane] = dfv[2 * ((size_t)(v & 3) * nk2 + (size_t)(v < 4 ? k : kq) * NB2) + lane];
    const int st = (int)(i % NST);
    if (!__all_sync(FULL, mbar_wait_bounded(&bar[st], (uint32_t)((i / NST) & 1), errflag))) {
      fail = i;
      break;
    }
    __syncwarp();  // the vectors are visible to the warp
    const float4* P1 = stage0 + (size_t)st * 4 * NB4;
    const float4* P2 = P1 + NB4;
    const float4* G1 = P1 + 2 * NB4;
    const float4* G2 = P1 + 3 * NB4;
    auto V = [&](int v, int e) -> const float4* { return vec + v * 32 + 2 * e; };  // (x, S(x)) of element e
    // transposed contraction
    // half 0: conj(P1[a][b]) Xbar[k][a], conj(P2[b][a]) Ybar[k][a]; half 1: P2[a][b] Xbar[k'][a],
    // P1[b][a] Ybar[k'][a] -- one instruction stream, operands selected per half
    // (two partial sums per output -- the real-part and the imaginary-part products of p -- so that
    // four accumulation chains run side by side)
    D::acc s1, s2, t1, t2;
    D::zero(s1);
    D::zero(s2);
    D::zero(t1);
    D::zero(t2);
    {
      const float4* Pc = half ? P2 : P1;  // read by columns
      const float4* Pr = half ? P1 : P2;  // read by rows
      const int vx = half ? 4 : 0, vy = half ? 5 : 1;
      const float sg = half ? -1.f : 1.f;  // conj(p) x takes +Im p, p x takes -Im p (exact sign flips)
#pragma unroll 4
      for (int j = 0; j < NB2; ++j) {
        const int a = (j + b) & 15;
        const float4 x = Pc[a * NB2 + b], y = Pr[b * NB2 + a];
        const float4* X = V(vx, a);
        const float4* Y = V(vy, a);
        D::pmac(s1, X[0], df_bre(x));
        D::pmac(t1, X[1], make_float4(sg * x.y, sg * x.y, sg * x.w, sg * x.w));
        D::pmac(s2, Y[0], df_bre(y));
        D::pmac(t2, Y[1], make_float4(sg * y.y, sg * y.y, sg * y.w, sg * y.w));
      }
    }
    {  // s += t (double-float, per half)
      float4 u1 = make_float4(s1.h.x, s1.h.y, s1.l.x, s1.l.y), u2 = make_float4(s2.h.x, s2.h.y, s2.l.x, s2.l.y);
      D::red_add4(u1, make_float4(t1.h.x, t1.h.y, t1.l.x, t1.l.y));
      D::red_add4(u2, make_float4(t2.h.x, t2.h.y, t2.l.x, t2.l.y));
      s1 = D::acc{make_float2(u1.x, u1.y), make_float2(u1.z, u1.w)};
      s2 = D::acc{make_float2(u2.x, u2.y), make_float2(u2.z, u2.w)};
    }
    // gradient: element e = lane + 32 j of G1 and of G2, a = e / 16, c = e % 16 (the column)
    float4* g1o = G + p * 2 * NB4;
    float4* g2o = g1o + NB4;
#pragma unroll 2
    for (int j = 0; j < NB4 / 32; ++j) {
      const int e = lane + 32 * j, a = e >> 4, c = e & 15;
      // G1[a][c] += conj(Xbar[k][a]) rt[k'][c] (+ conj(st[k][a]) Ybar[k'][c])
      D::acc g = {make_float2(G1[e].x, G1[e].y), make_float2(G1[e].z, G1[e].w)};
      const float4 Xka = V(0, a)[0];
      const float4* rq = V(6, c);
      D::pmac(g, rq[0], df_bre(Xka));
      D::pmac(g, rq[1], df_bim(Xka));
      if (rev) {
        const float4 ska = V(3, a)[0];
        const float4* Yq = V(5, c);
        D::pmac(g, Yq[0], df_bre(ska));
        D::pmac(g, Yq[1], df_bim(ska));
      }
      D::renorm(g);
      g1o[e] = make_float4(g.h.x, g.h.y, g.l.x, g.l.y);
      // G2[a][c] += conj(Ybar[k][c]) st[k'][a] (+ conj(rt[k][c]) Xbar[k'][a])
      D::acc h2 = {make_float2(G2[e].x, G2[e].y), make_float2(G2[e].z, G2[e].w)};
      const float4 Ykc = V(1, c)[0];
      const float4* sq = V(7, a);
      D::pmac(h2, sq[0], df_bre(Ykc));
      D::pmac(h2, sq[1], df_bim(Ykc));
      if (rev) {
        const float4 rkc = V(2, c)[0];
        const float4* Xq = V(4, a);
        D::pmac(h2, Xq[0], df_bre(rkc));
        D::pmac(h2, Xq[1], df_bim(rkc));
      }
      D::renorm(h2);
      g2o[e] = make_float4(h2.h.x, h2.h.y, h2.l.x, h2.l.y);
    }
    // the stage and the vectors are free once every lane has read them: order those reads before the
    // next bulk copy into the stage (generic -> async proxy), then refill it
    fence_proxy_async();
    __syncwarp();
    if (i + NST < n) issue(i + NST);
    if (half == 0 || rev) {
      const int kt = half == 0 ? kq : k;
      double* ro = rtb + ((size_t)kt * NB2 + b) * 2;
      double* so = stb + ((size_t)kt * NB2 + b) * 2;
      atomicAdd(ro, D::re_d(s1));
      atomicAdd(ro + 1, D::im_d(s1));
      atomicAdd(so, D::re_d(s2));
      atomicAdd(so + 1, D::im_d(s2));
    }
  }
  if (fail >= 0) {  // drain the copies still in flight (bounded), then leave
    if (lane == 0) {
      const long long last = (fail + NST < n ? fail + NST : n) - 1;
      for (long long c = fail; c <= last; ++c) mbar_wait_bounded(&bar[c % NST], (uint32_t)((c / NST) & 1), nullptr, 1u << 16);
    }
    __syncwarp();
  }
}

// ubar (window) += D o rt_bar - D o st_bar; then ybar += ubar and, when kprev is set,
// kprev += c * ubar. One thread per state element.
template <int NB>
__global__ void k_adj_combine(int nk, int nbdm, int bs, int phase, double t, const double* __restrict__ ew,
                              const double2* __restrict__ ph, const double2* __restrict__ rtb,
                              const double2* __restrict__ stb, const double2* __restrict__ ubar,
                              double2* __restrict__ ybar, double2* __restrict__ kprev, double c) {
  constexpr int NB2 = NB * NB;
  const int nd2 = nbdm * nbdm;
  const long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (idx >= (long long)nk * nd2) return;
  const int k = (int)(idx / nd2), e = (int)(idx - (long long)k * nd2), ii = e / nbdm, jj = e - ii * nbdm;
  double2 u = ubar[idx];
  const int i = ii - bs, j = jj - bs;
  if (i >= 0 && i < NB && j >= 0 && j < NB) {
    const int w = i * NB + j;
    double2 D = mk2(1.0, 0.0);
    if (phase && i != j) D = ph ? ph[(size_t)k * NB2 + w] : ccis((ew[(size_t)k * NB + i] - ew[(size_t)k * NB + j]) * t);
    u = cadd(u, cmul(D, csub(rtb[(size_t)k * NB2 + w], stb[(size_t)k * NB2 + w])));
  }
  ybar[idx] = cadd(ybar[idx], u);
  if (kprev) kprev[idx] = cadd(kprev[idx], mk2(c * u.x, c * u.y));
}

// cotangent of an observable total (observable.h:356-366) with weight w:
// ybar[k][b][i] += w * prefac * conj(o_t(i, b)) for i in [bs, be)
__global__ void k_adj_obs(int nk, int nbdm, int bs, int be, const double2* __restrict__ obs,
                          const double* __restrict__ edm, double t, int picture, double w, double2* __restrict__ ybar) {
  const int nd2 = nbdm * nbdm;
  const long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (idx >= (long long)nk * nd2) return;
  const int k = (int)(idx / nd2), e = (int)(idx - (long long)k * nd2), b = e / nbdm, i = e - b * nbdm;
  if (i < bs || i >= be) return;
  const double2 oib = obs[(size_t)k * nd2 + i * nbdm + b];
  const double2 ot = (i == b || picture == 1) ? oib : cmul(oib, ccis((edm[(size_t)k * nbdm + i] - edm[(size_t)k * nbdm + b]) * t));
  ybar[idx] = cadd(ybar[idx], mk2(w * ot.x, -w * ot.y));
}

// out = y + c k; out = c x
__global__ void k_axpy(size_t n, double2* __restrict__ out, const double2* __restrict__ y, double c,
                       const double2* __restrict__ k) {
  const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i < n) out[i] = mk2(fma(c, k[i].x, y[i].x), fma(c, k[i].y, y[i].y));
}
__global__ void k_scale(size_t n, double2* __restrict__ out, double c, const double2* __restrict__ x) {
  const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i < n) out[i] = mk2(c * x[i].x, c * x[i].y);
}
// y_next = y + h/6 (k1 + 2 k2 + 2 k3 + k4)
__global__ void k_rk4_final(size_t n, double2* __restrict__ out, const double2* __restrict__ y,
                            const double2* __restrict__ K, size_t ks, double h) {
  const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double2 k1 = K[i], k2 = K[ks + i], k3 = K[2 * ks + i], k4 = K[3 * ks + i];
  const double sx = k1.x + 2.0 * k2.x + 2.0 * k3.x + k4.x, sy = k1.y + 2.0 * k2.y + 2.0 * k3.y + k4.y;
  out[i] = mk2(y[i].x + h / 6.0 * sx, y[i].y + h / 6.0 * sy);
}

}  // namespace dmd
