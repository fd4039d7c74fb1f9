// Sparse k-pair contraction (alg_sparseP / alg_Pin_is_sparse): only the stored elements of P1, P2.
//
// The reference keeps, per pair, the elements with |P| > thr_sparseP (default 1e-40) in COO form and
// multiplies them with sparse_zgemm (comm/sparse_matrix.cpp:6-40; sparse2D.h:9-200; the branch of
// evolve_eph.cpp:67-82, phases per element by compute_sPt, evolve_eph.cpp:194-203). Here the phases
// are factorised per k as in the dense forms (rt = conj(D) o rho, st = conj(D) o (1 - rho), the
// finish multiplies by D), and the products are regrouped by the k-point they update:
//
//   every pair (k, k') gives a forward contribution to target k from source k' with
//     X-matrix P1 (read by rows: X_k[a] += sum_b P1[a][b] rt_k'[b]) and
//     Y-matrix P2 (read by columns: Y_k[b] += sum_a st_k'[a] P2[a][b]);
//   a pair with k < k' also gives a reverse contribution to target k' from source k with
//     X-matrix conj(P2) (rows) and Y-matrix conj(P1) (columns)        (evolve_eph.cpp:101-106).
//
// Every output element (k, X or Y, a) is owned by one thread, which runs over its products of all
// the contributions to k: no atomics, and a fixed order of the sums. Each stored element is kept
// twice (once per direction, the reverse copy conjugated), which the forward/reverse symmetry of
// the dense kernels avoids; the sparse form pays where the fill is low enough (bench --sparse).
//
// Layout (ELL, lane-interleaved): the products of thread lane l of k-point k are a list of
// (element value, index into the coordinate array rs) -- the index names the source k-point, rt or
// st, and the element's other band-pair index. The lists of the 2 nb^2 threads of a k-point are
// padded with zeros to the longest one, L_k, and stored interleaved: product j of lane l at
// base_k + j (2 nb^2) + l. Consecutive threads then read consecutive values (coalesced), and the
// loads of a thread's products do not depend on each other.
#pragma once
#include "dmd_common.cuh"

namespace dmd {

template <int NB>
__global__ void __launch_bounds__(256) k_pairs_sparse(int nk, const long long* __restrict__ base,
                                                      const int* __restrict__ len, const double2* __restrict__ val,
                                                      const int* __restrict__ gidx, const double2* __restrict__ rs,
                                                      double2* __restrict__ acc) {
  constexpr int TPR = 2 * NB * NB;
  const long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  const long long k = g / TPR;
  if (k >= nk) return;
  const int l = (int)(g - k * TPR);
  const int L = len[k];
  const double2* vp = val + base[k] + l;
  const int* ip = gidx + base[k] + l;
  double2 s0 = mk2(0.0, 0.0), s1 = mk2(0.0, 0.0);
  int j = 0;
  for (; j + 4 <= L; j += 4) {
    const double2 v0 = __ldg(vp + (size_t)j * TPR), v1 = __ldg(vp + (size_t)(j + 1) * TPR);
    const double2 v2 = __ldg(vp + (size_t)(j + 2) * TPR), v3 = __ldg(vp + (size_t)(j + 3) * TPR);
    const int i0 = __ldg(ip + (size_t)j * TPR), i1 = __ldg(ip + (size_t)(j + 1) * TPR);
    const int i2 = __ldg(ip + (size_t)(j + 2) * TPR), i3 = __ldg(ip + (size_t)(j + 3) * TPR);
    s0 = cfma(v0, __ldg(rs + i0), s0);
    s1 = cfma(v1, __ldg(rs + i1), s1);
    s0 = cfma(v2, __ldg(rs + i2), s0);
    s1 = cfma(v3, __ldg(rs + i3), s1);
  }
  for (; j < L; ++j) s0 = cfma(__ldg(vp + (size_t)j * TPR), __ldg(rs + __ldg(ip + (size_t)j * TPR)), s0);
  acc[(size_t)k * TPR + l] = mk2(s0.x + s1.x, s0.y + s1.y);
}

}  // namespace dmd
