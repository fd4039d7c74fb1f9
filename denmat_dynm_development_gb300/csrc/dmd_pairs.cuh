// k-pair contraction kernels (the HBM-streaming part of the Lindblad RHS).
//
// For every stored pair p = (k, k') with P1, P2 in [a][b] = [(i1 i2)][(i3 i4)] order the four
// products of evolve_eph.cpp:99-106, phase-free (see dmd_kernels.cuh):
//   type 0  X_k [a] += sum_b P1[a][b]        rt_k'[b]
//   type 1  Y_k [b] += sum_a st_k'[a]        P2[a][b]
//   type 2  X_k'[a] += sum_b conj(P2[a][b])  rt_k[b]     (only when k < k')
//   type 3  Y_k'[b] += sum_a st_k[a]         conj(P1[a][b])   (only when k < k')
#pragma once
#include "dmd_common.cuh"

namespace dmd {

// Simple form: one thread per (pair, type, output element), FP64 FMAs, FP64 atomics into the
// per-k accumulators. Pair storage: [npair][2][NB4] complex128 (P1 block then P2 block).
template <int NB>
__global__ void k_pairs_f64_atomic(long long npair, const int2* __restrict__ kk, const double2* __restrict__ P,
                                   const double2* __restrict__ rs, double2* __restrict__ acc) {
  constexpr int NB2 = NB * NB, NB4 = NB2 * NB2, TPP = 4 * NB2;
  const long long gid = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  const long long p = gid / TPP;
  if (p >= npair) return;
  const int r = (int)(gid - p * TPP);
  const int type = r / NB2, a = r - type * NB2;
  const int2 pk = kk[p];
  const int k = pk.x, kp = pk.y;
  if (type >= 2 && !(k < kp)) return;
  const double2* P1 = P + (size_t)p * 2 * NB4;
  const double2* P2 = P1 + NB4;
  double2 s = mk2(0.0, 0.0);
  double2* dst;
  if (type == 0) {
    const double2* v = rs + (size_t)kp * 2 * NB2;
#pragma unroll
    for (int b = 0; b < NB2; ++b) s = cfma(__ldg(&P1[a * NB2 + b]), __ldg(&v[b]), s);
    dst = acc + (size_t)k * 2 * NB2 + a;
  } else if (type == 1) {
    const double2* v = rs + (size_t)kp * 2 * NB2 + NB2;
#pragma unroll
    for (int i = 0; i < NB2; ++i) s = cfma(__ldg(&v[i]), __ldg(&P2[i * NB2 + a]), s);
    dst = acc + (size_t)k * 2 * NB2 + NB2 + a;
  } else if (type == 2) {
    const double2* v = rs + (size_t)k * 2 * NB2;
#pragma unroll
    for (int b = 0; b < NB2; ++b) s = cfma_conja(__ldg(&P2[a * NB2 + b]), __ldg(&v[b]), s);
    dst = acc + (size_t)kp * 2 * NB2 + a;
  } else {
    const double2* v = rs + (size_t)k * 2 * NB2 + NB2;
#pragma unroll
    for (int i = 0; i < NB2; ++i) s = cfma_conja(__ldg(&P1[i * NB2 + a]), __ldg(&v[i]), s);
    dst = acc + (size_t)kp * 2 * NB2 + NB2 + a;
  }
  atomicAdd(&dst->x, s.x);
  atomicAdd(&dst->y, s.y);
}

}  // namespace dmd
