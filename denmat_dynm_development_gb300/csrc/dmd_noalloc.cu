// dmd_evolve_driver_noalloc: the scattering right-hand side on caller-owned device buffers, for
// callers that cannot allocate device memory -- code running while a CUDA graph is being captured,
// host frameworks whose memory pools own the whole device, or plug-ins that are handed device
// pointers but no allocator. It allocates nothing: its scratch (the phase-removed density matrices
// and the per-k sums, 4 * nk * nb^2 complex numbers) lives in the file-scope device array below,
// which every GPU that loads this library holds until the process exits.
//
// The array's host-side name is not a device address; the device address is obtained once per
// device with cudaGetSymbolAddress, on the first call made with that device current (so that first
// call should come before any stream capture). Every call shares the array and it keeps the last
// call's contents; the kernels clear what must start at zero. Calls whose work overlaps on the GPU
// (different streams, or another host thread) race on the array and must be serialised by the
// caller. The address is cached per device for the life of the process: resetting a device
// (cudaDeviceReset) after its first call is not supported, since the array then moves.
// This path is a plain FP64 reference-speed implementation (one thread per pair product with FP64
// atomics, one thread per k in the finish); the fast contraction is the handle-based one.
#include <cuda_runtime.h>

#include <mutex>

#include "dmd_common.cuh"
#include "dmd_gpu.h"

namespace {

constexpr size_t kScratchElems = (size_t)1 << 20;  // complex128 elements (16 MiB)
constexpr int kMaxDevices = 64;

__device__ __align__(256) double2 g_scratch[kScratchElems];

double2* g_scratch_addr[kMaxDevices] = {nullptr};
std::mutex g_scratch_mu;

int scratch_address(double2** out) {
  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess) return DMD_E_CUDA;
  if (dev < 0 || dev >= kMaxDevices) return DMD_E_ARG;
  std::lock_guard<std::mutex> lk(g_scratch_mu);
  if (!g_scratch_addr[dev]) {
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, g_scratch) != cudaSuccess || !p) return DMD_E_CUDA;
    g_scratch_addr[dev] = (double2*)p;
  }
  *out = g_scratch_addr[dev];
  return DMD_OK;
}

// rt_k = conj(D_k) o rho_k, st_k = conj(D_k) o (1 - rho_k) on the e-ph window, sums zeroed
template <int NB>
__global__ void k_na_prep(int nk, int nbdm, int bs, const double2* __restrict__ dm, const double* __restrict__ edm,
                          double t, int expt, double2* __restrict__ rs, double2* __restrict__ acc) {
  constexpr int NB2 = NB * NB;
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= nk * NB2) return;
  const int k = idx / NB2, ab = idx - k * NB2, i = ab / NB, j = ab - i * NB;
  const double2 r = dm[(size_t)k * nbdm * nbdm + (bs + i) * nbdm + bs + j];
  const double2 s = (i == j) ? mk2(1.0 - r.x, 0.0 - r.y) : mk2(-r.x, -r.y);
  double2 rt = r, st = s;
  if (expt) {
    const double2 d = ccis((edm[(size_t)k * nbdm + bs + i] - edm[(size_t)k * nbdm + bs + j]) * t);
    rt = cmul_rn(cconj(d), r);
    st = cmul_rn(cconj(d), s);
  }
  rs[(size_t)k * 2 * NB2 + ab] = rt;
  rs[(size_t)k * 2 * NB2 + NB2 + ab] = st;
  acc[(size_t)k * 2 * NB2 + ab] = mk2(0.0, 0.0);
  acc[(size_t)k * 2 * NB2 + NB2 + ab] = mk2(0.0, 0.0);
}

// one thread per (pair, product, output element) reading DMD's own P1 / P2 arrays and size_t pair
// indices; pairs with an index outside [0, nk) are skipped
template <int NB>
__global__ void k_na_pairs(long long npair, int nk, const unsigned long long* __restrict__ k1st,
                           const unsigned long long* __restrict__ k2nd, const double2* __restrict__ P1,
                           const double2* __restrict__ P2, const double2* __restrict__ rs, double2* __restrict__ acc) {
  constexpr int NB2 = NB * NB, NB4 = NB2 * NB2, TPP = 4 * NB2;
  const long long gid = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  const long long p = gid / TPP;
  if (p >= npair) return;
  const int r = (int)(gid - p * TPP);
  const int type = r / NB2, a = r - type * NB2;
  const unsigned long long k1 = k1st[p], k2 = k2nd[p];
  if (k1 >= (unsigned long long)nk || k2 >= (unsigned long long)nk) return;
  const int k = (int)k1, kp = (int)k2;
  if (type >= 2 && !(k < kp)) return;
  const double2* p1 = P1 + (size_t)p * NB4;
  const double2* p2 = P2 + (size_t)p * NB4;
  double2 s = mk2(0.0, 0.0);
  double2* dst;
  if (type == 0) {  // X_k[a] += P1[a][b] rt_k'[b]
    const double2* v = rs + (size_t)kp * 2 * NB2;
    for (int b = 0; b < NB2; ++b) s = cfma(p1[a * NB2 + b], v[b], s);
    dst = acc + (size_t)k * 2 * NB2 + a;
  } else if (type == 1) {  // Y_k[a] += st_k'[i] P2[i][a]
    const double2* v = rs + (size_t)kp * 2 * NB2 + NB2;
    for (int i = 0; i < NB2; ++i) s = cfma(v[i], p2[i * NB2 + a], s);
    dst = acc + (size_t)k * 2 * NB2 + NB2 + a;
  } else if (type == 2) {  // X_k'[a] += conj(P2[a][b]) rt_k[b]
    const double2* v = rs + (size_t)k * 2 * NB2;
    for (int b = 0; b < NB2; ++b) s = cfma_conja(p2[a * NB2 + b], v[b], s);
    dst = acc + (size_t)kp * 2 * NB2 + a;
  } else {  // Y_k'[a] += st_k[i] conj(P1[i][a])
    const double2* v = rs + (size_t)k * 2 * NB2 + NB2;
    for (int i = 0; i < NB2; ++i) s = cfma_conja(p1[i * NB2 + a], v[i], s);
    dst = acc + (size_t)kp * 2 * NB2 + NB2 + a;
  }
  atomicAdd(&dst->x, s.x);
  atomicAdd(&dst->y, s.y);
}

__device__ __forceinline__ double2 herm_up_na(const double2* A, int n, int i, int l) {
  if (i == l) return mk2(A[i * n + i].x, 0.0);
  return (i < l) ? A[i * n + l] : cconj(A[l * n + i]);
}

// per-k finish: c = (1 - rho) Pdm - dm1P rho (Hermitian operands from their upper triangles),
// ddmdt = prefac/2 (c + c^dagger) on the window, zero elsewhere (evolve_driver's set_mat)
template <int NB>
__global__ void k_na_finish(int nk, int nbdm, int bs, double prefac, int expt, double t,
                            const double2* __restrict__ dm, const double* __restrict__ edm,
                            const double2* __restrict__ acc, double2* __restrict__ out) {
  constexpr int NB2 = NB * NB;
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nk) return;
  const int nd = nbdm, nd2 = nd * nd;
  const double2* yk = dm + (size_t)k * nd2;
  const double2* X = acc + (size_t)k * 2 * NB2;
  const double2* Y = X + NB2;
  double2 rw[NB2], sw[NB2], Pdm[NB2], dmP[NB2], c[NB2];
  for (int i = 0; i < NB; ++i)
    for (int j = 0; j < NB; ++j) {
      const double2 r = yk[(bs + i) * nd + bs + j];
      rw[i * NB + j] = r;
      sw[i * NB + j] = (i == j) ? mk2(1.0 - r.x, 0.0 - r.y) : mk2(-r.x, -r.y);
      if (expt) {
        const double2 d = ccis((edm[(size_t)k * nd + bs + i] - edm[(size_t)k * nd + bs + j]) * t);
        Pdm[i * NB + j] = cmul_rn(d, X[i * NB + j]);
        dmP[i * NB + j] = cmul_rn(d, Y[i * NB + j]);
      } else {
        Pdm[i * NB + j] = X[i * NB + j];
        dmP[i * NB + j] = Y[i * NB + j];
      }
    }
  for (int i = 0; i < NB; ++i)
    for (int j = 0; j < NB; ++j) {
      double2 s = mk2(0.0, 0.0);
      for (int l = 0; l < NB; ++l) s = cadd_rn(s, cmul_rn(herm_up_na(sw, NB, i, l), Pdm[l * NB + j]));
      c[i * NB + j] = cmul_rn(mk2(1.0, 0.0), s);
    }
  for (int i = 0; i < NB; ++i)
    for (int j = 0; j < NB; ++j) {
      double2 s = mk2(0.0, 0.0);
      for (int l = 0; l < NB; ++l) s = cadd_rn(s, cmul_rn(dmP[i * NB + l], herm_up_na(rw, NB, l, j)));
      c[i * NB + j] = cadd_rn(cmul_rn(mk2(-1.0, 0.0), s), cmul_rn(mk2(1.0, 0.0), c[i * NB + j]));
    }
  double2* o = out + (size_t)k * nd2;
  for (int i = 0; i < nd2; ++i) o[i] = mk2(0.0, 0.0);
  const double pf = prefac * 0.5;
  for (int i = 0; i < NB; ++i)
    for (int j = 0; j < NB; ++j)
      o[(bs + i) * nd + bs + j] = cscale_rn(pf, cadd_rn(c[i * NB + j], cconj(c[j * NB + i])));
}

template <int NB>
int run_noalloc(int nk, int nbdm, int bs, long long npair, const unsigned long long* k1, const unsigned long long* k2,
                const double2* P1, const double2* P2, const double* edm, double prefac, int expt, double t,
                const double2* dm, double2* out, cudaStream_t st, double2* scratch) {
  constexpr int NB2 = NB * NB;
  double2* rs = scratch;
  double2* acc = scratch + (size_t)2 * nk * NB2;
  const int nprep = nk * NB2;
  // an error left pending by the caller's earlier work is theirs: report it without consuming it
  if (cudaPeekAtLastError() != cudaSuccess) return DMD_E_CUDA;
  k_na_prep<NB><<<(nprep + 255) / 256, 256, 0, st>>>(nk, nbdm, bs, dm, edm, t, expt, rs, acc);
  if (npair > 0) {
    const long long nthr = npair * 4LL * NB2;
    k_na_pairs<NB><<<(unsigned)((nthr + 255) / 256), 256, 0, st>>>(npair, nk, k1, k2, P1, P2, rs, acc);
  }
  k_na_finish<NB><<<(nk + 127) / 128, 128, 0, st>>>(nk, nbdm, bs, prefac, expt, t, dm, edm, acc, out);
  return cudaGetLastError() == cudaSuccess ? DMD_OK : DMD_E_CUDA;
}

}  // namespace

extern "C" int dmd_evolve_driver_noalloc(int32_t nk, int32_t nb_dm, int32_t bstart, int32_t bend, int64_t nkpair,
                                         const uint64_t* k1st, const uint64_t* k2nd, const double* P1,
                                         const double* P2, const double* e_dm, double prefac_eph, int32_t expt,
                                         double t, const double* dm, double* ddmdt_eph, void* stream) {
  const int nb = bend - bstart;
  if (nk <= 0 || nb_dm <= 0 || nb_dm > DMD_MAX_NBDM || bstart < 0 || bend > nb_dm || nb < 1 || nb > 4 ||
      nkpair < 0 || !e_dm || !dm || !ddmdt_eph)
    return DMD_E_ARG;
  if (nkpair > 0 && (!k1st || !k2nd || !P1 || !P2)) return DMD_E_ARG;
  if ((size_t)4 * nk * nb * nb > kScratchElems) return DMD_E_ARG;  // nk * nb^2 <= 262144
  if ((unsigned long long)nkpair * 16ULL * nb * nb > (1ULL << 62)) return DMD_E_ARG;
  double2* scratch = nullptr;
  int rc = scratch_address(&scratch);
  if (rc) return rc;
  cudaStream_t st = (cudaStream_t)stream;
  const unsigned long long* k1 = (const unsigned long long*)k1st;
  const unsigned long long* k2 = (const unsigned long long*)k2nd;
  const double2* p1 = (const double2*)P1;
  const double2* p2 = (const double2*)P2;
  const double2* y = (const double2*)dm;
  double2* o = (double2*)ddmdt_eph;
  switch (nb) {
    case 1: return run_noalloc<1>(nk, nb_dm, bstart, nkpair, k1, k2, p1, p2, e_dm, prefac_eph, expt, t, y, o, st, scratch);
    case 2: return run_noalloc<2>(nk, nb_dm, bstart, nkpair, k1, k2, p1, p2, e_dm, prefac_eph, expt, t, y, o, st, scratch);
    case 3: return run_noalloc<3>(nk, nb_dm, bstart, nkpair, k1, k2, p1, p2, e_dm, prefac_eph, expt, t, y, o, st, scratch);
    default: return run_noalloc<4>(nk, nb_dm, bstart, nkpair, k1, k2, p1, p2, e_dm, prefac_eph, expt, t, y, o, st, scratch);
  }
}
