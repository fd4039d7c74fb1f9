// C ABI of the GB300 Lindblad RHS (see include/dmd_gpu.h): handle, device layout, steppers.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <algorithm>
#include <atomic>
#include <string>
#include <thread>
#include <vector>

#include "dmd_adjoint.cuh"
#include "dmd_batched_tc.cuh"
#include "dmd_ee.cuh"
#include "dmd_gpu.h"
#include "dmd_kernels.cuh"
#include "dmd_layout.h"
#include "dmd_pairs.cuh"
#include "dmd_pairs_cb.cuh"
#include "dmd_sparse.cuh"

using namespace dmd;

namespace {
struct PairSource;
}

struct dmd_handle {
  int dev = 0;
  cudaStream_t st = nullptr;
  int nk = 0, nbdm = 0, bs = 0, be = 0, nb = 0, nb2 = 0, nb4 = 0;
  long long npair = 0;
  double prefac = 0;
  double add_scale = 0;        // scale of the additive operators (P += add_scale P_add)
  PairSource* src = nullptr;   // set while creating from files: where the raw operators come from
  int picture = 0, expt = 1, prec = 0;
  size_t nstate = 0;  // complex elements of the state (nrhs * nk * nbdm^2)
  size_t nstate1 = 0; // complex elements of one state (nk * nbdm^2)
  int nrhs = 1;       // batched form: states sharing P
  int brw = 4;        // batched form: states per warp in the contraction
  // device arrays
  double* d_ew = nullptr;      // [nk][nb]
  double* d_edm = nullptr;     // [nk][nbdm]
  int2* d_kk = nullptr;        // [npair] (per-thread form)
  double2* d_P = nullptr;      // [npair][2][nb4] (per-thread form) or the column-block element store
  // column-block layout (nb = 2)
  int use_cb = 0;
  int lin = 0;                 // linearized master equation (DMD_FLAG_LINEAR)
  int pcfg = 0;                // pair-kernel shape variant of the f64x form (DMD_PAIR_CFG)
  int pcfg64 = 1;              // pair-kernel shape variant of the f64 form (DMD_PAIR_CFG64)
  int* d_pos = nullptr;        // k -> energy rank
  int* d_inv = nullptr;        // energy rank -> k
  dmd::RowBlock* d_rb = nullptr;
  dmd::WorkItem* d_items = nullptr;
  int nitems = 0;
  long long nrb = 0;
  unsigned int* d_err = nullptr;  // device error flags (bounded waits)
  unsigned int* d_hflag = nullptr;  // set by the prep kernel when a state is not exactly Hermitian
  double2* d_acc0 = nullptr;   // deviation form: contraction of diag(f_ref), position order [nk][2][nb2]
  double* d_fref = nullptr;    // deviation form: window occupations [nk][nb]
  double2* d_ph = nullptr;     // phases D_k(i, j) of the current evaluation [nk][nb2]
  // batched form on the tensor cores (nb = 2, bf16 hi + lo): operator and coordinate blocks
  int use_tc = 0;
  uint16_t* d_tcB = nullptr;   // [blocks][256 x (hi 32 | lo 32)] bf16, per tile its column groups
  uint16_t* d_tcA = nullptr;   // [part][group][state block][128 x (hi 32 | lo 32)] bf16
  dmd::TcTile* d_tiles = nullptr;
  int ntiles = 0, ngroups = 0, nmb = 0;
  int tcst = 4;                // pipeline stages of the tensor-core contraction (autotuned: 4, 3, 2)
  int64_t pair_bytes = 0;      // stored operator bytes (dmd_pair_bytes)
  int adj = 0;                 // DMD_FLAG_ADJOINT: pair operators also in stored order (d_Praw, d_kkraw)
  double2* d_Praw = nullptr;   // [npair][2][nb4] folded P1, P2
  int2* d_kkraw = nullptr;
  float4* d_Padf = nullptr;    // adjoint of a double-float handle: the stored-order operators as double-floats
  int padf_ok = 0;             // d_Padf matches the current operators
  int eek = 0;                 // DMD_FLAG_EE: d_Praw, d_kkraw and d_dst kept for the e-e model
  // sparse form (DMD_FLAG_SPARSE): per k-point the products of its output threads, lane-interleaved
  int use_sp = 0;
  long long sp_nel = 0, sp_nslot = 0;  // stored elements (both directions), ELL slots with padding
  long long* d_sp_base = nullptr;    // [nk] first slot of each k-point
  int* d_sp_len = nullptr;           // [nk] products per thread (padded)
  double2* d_sp_val = nullptr;       // [nslot] element values
  int* d_sp_gidx = nullptr;          // [nslot] index into the coordinate array
  void* d_dst = nullptr;       // column-block destination of every stored pair (CbDst)
  // e-e model (dmd_ee_attach): P = P_base (d_Praw) + ee_scale P_ee, rebuilt from rho
  int ee_on = 0, ee_every = 0, ee_update = 0, ee_nv = 0;
  double ee_scale = 1, ee_nfree0 = 0, ee_nkfull = 1, ee_cell = 1, ee_eps = 1, ee_T = 1, ee_meff = 1;
  double ee_eppa = 0, ee_smear = 0;  // plasmon pole: energy and smearing in use
  int ee_gn = 1;
  dmd::EeArgs ee_args;
  double* d_ee_kvec = nullptr;
  int4* d_ee_kidx = nullptr;
  int* d_ee_kmap = nullptr;
  double2* d_ee_U = nullptr;
  float* d_ee_ewf = nullptr;
  double* d_ee_f = nullptr;
  double2* d_ee_dm = nullptr;
  double2* d_ee_dm1 = nullptr;
  float4* d_ee_dmf = nullptr;
  float4* d_ee_dm1f = nullptr;
  dmd::EeScreen* d_ee_scr = nullptr;
  double* d_ee_vqtab = nullptr;  // static RPA vq by q mesh index
  double2* d_ee_Aq = nullptr;     // plasmon-pole A(q), E^2(q) by q mesh index
  double2* d_ee_Eq2 = nullptr;
  double2* d_ee_Pee = nullptr;
  float2* d_x0y0 = nullptr;    // tensor-core form: contraction of diag(f_ref), back-transformed, by k
  float2* d_v0 = nullptr;      // tensor-core form: (prefac/2)(C0 + C0^dagger) by k
  double2* d_H = nullptr;      // [nk][nbdm^2]
  double2* d_eq = nullptr;     // [nk][nb2]
  double2* d_rs = nullptr;     // [nk][2][nb2] (per-thread form); Hermitian + anti-Hermitian coordinates (column-block form)
  double2* d_acc = nullptr;    // [nk][2][nb2]
  double2* d_y = nullptr;      // state
  double2* d_ytmp = nullptr;
  double2* d_y0 = nullptr;     // RKF45 retry copy
  double2* d_in = nullptr;     // host-call staging
  double2* d_in1 = nullptr;
  double2* d_out = nullptr;
  double2* d_K = nullptr;      // [6][nstate]
  double* d_tref = nullptr;    // [t0, h]
  long long* d_step = nullptr;
  double* d_red = nullptr;     // reduction partials
  int* d_coef_i = nullptr;     // RKF45 coefficient tables
  double* d_coef = nullptr;
  int* d_flag = nullptr;
  double2* d_obs[8] = {nullptr};
  double* d_f[8] = {nullptr};
  double obs_prefac[8] = {0};
  double t = 0;                // time of the device state
  long long launches = 0;
  cudaGraphExec_t g_rk4 = nullptr;
  cudaGraphExec_t g_rk4_rec = nullptr;  // the RK4 step that also copies its stage inputs and sums to d_rec
  double2* d_rec = nullptr;             // [4][nstate] stage inputs, then [4][nk 2 nb^2] forward sums
  std::string err;
  // timing / profiling
  cudaEvent_t tev[2] = {nullptr, nullptr};
  int prof_on = 0;
  struct Rec {
    int cls;
    cudaEvent_t a, b;
  };
  std::vector<Rec> prof_pending;
  std::vector<cudaEvent_t> ev_pool;
  double prof_ms[5] = {0, 0, 0, 0, 0};  // prep, contraction, finish, step counter, e-e rebuild
  long long prof_n[5] = {0, 0, 0, 0, 0};
};

namespace {

const char* kStatus[] = {"ok", "invalid argument", "out of memory", "file error", "CUDA error", "device wait timed out",
                         "non-finite state", "wrong call order", "no CUDA device", "ODE step failure"};

int fail(dmd_handle* h, int code, const std::string& msg) {
  if (h) h->err = msg;
  return code;
}

#define CK(call)                                                                                   \
  do {                                                                                             \
    cudaError_t e_ = (call);                                                                       \
    if (e_ != cudaSuccess)                                                                         \
      return fail(h, e_ == cudaErrorMemoryAllocation ? DMD_E_NOMEM : DMD_E_CUDA,                   \
                  std::string(#call) + ": " + cudaGetErrorString(e_));                             \
  } while (0)

#define CKL()                                                                                      \
  do {                                                                                             \
    cudaError_t e_ = cudaGetLastError();                                                           \
    if (e_ != cudaSuccess) return fail(h, DMD_E_CUDA, std::string("launch: ") + cudaGetErrorString(e_)); \
  } while (0)

template <typename T>
int dalloc(dmd_handle* h, T** p, size_t n) {
  CK(cudaMalloc((void**)p, (n ? n : 1) * sizeof(T)));
  return DMD_OK;
}

inline unsigned blocks_for(long long n, int tpb) { return (unsigned)((n + tpb - 1) / tpb); }

// doubles of the reduction scratch: RKF45 error blocks of the whole state, observable partials
size_t red_elems(const dmd_handle* h) {
  const size_t a = 4096, b = (2 * h->nstate + 255) / 256 + 64, c = 2 * ((size_t)h->nk / 256 + 1) * h->nrhs;
  return a > b ? (a > c ? a : c) : (b > c ? b : c);
}

// bytes of one stored Q element per arithmetic
int elem_bytes(int prec) { return (prec == DMD_PREC_F32 || prec == DMD_PREC_BF16X2) ? 8 : 16; }
// the reduced-precision forms contract rho - diag(f_ref) only
bool deviation_form(int prec) { return prec == DMD_PREC_F32 || prec == DMD_PREC_BF16X2; }

cudaEvent_t pool_event(dmd_handle* h) {
  if (!h->ev_pool.empty()) {
    cudaEvent_t e = h->ev_pool.back();
    h->ev_pool.pop_back();
    return e;
  }
  cudaEvent_t e = nullptr;
  cudaEventCreate(&e);
  return e;
}

// brackets one kernel launch with events when profiling is on
struct ProfScope {
  dmd_handle* h;
  int cls;
  cudaEvent_t a = nullptr;
  ProfScope(dmd_handle* h_, int c) : h(h_), cls(c) {
    if (h->prof_on) {
      a = pool_event(h);
      cudaEventRecord(a, h->st);
    }
  }
  ~ProfScope() {
    if (h->prof_on && a) {
      cudaEvent_t b = pool_event(h);
      cudaEventRecord(b, h->st);
      h->prof_pending.push_back({cls, a, b});
    }
  }
};

// accumulate finished profiling records (call after the stream is synchronised)
void prof_harvest(dmd_handle* h) {
  for (auto& r : h->prof_pending) {
    float ms = 0;
    if (cudaEventElapsedTime(&ms, r.a, r.b) == cudaSuccess) {
      h->prof_ms[r.cls] += ms;
      h->prof_n[r.cls] += 1;
    }
    h->ev_pool.push_back(r.a);
    h->ev_pool.push_back(r.b);
  }
  h->prof_pending.clear();
}

// ---------------------------------------------------------------------------------------------
// one RHS evaluation on device buffers: prep -> pairs -> finish
// ---------------------------------------------------------------------------------------------
template <int NB>
int launch_prep(dmd_handle* h, const double2* y, const TimeArg& ta) {
  const int n = h->nk * NB * NB;
  ProfScope ps(h, 0);
  if (!h->use_cb) {
    k_prep<NB><<<blocks_for(n, 256), 256, 0, h->st>>>(h->nk, h->nbdm, h->bs, y, h->d_ew, ta, h->expt, h->d_rs, h->d_acc,
                                                       h->d_ph);
  } else {
    // deviation coordinates for the reduced-precision and the linearized forms
    const double* fref = (deviation_form(h->prec) || h->lin) ? h->d_fref : nullptr;
    // batched form: a thread serves up to 8 states of its (k, element), so the phase is computed once
    const int qc = h->nrhs < 8 ? h->nrhs : 8;
    const dim3 g(blocks_for(n, 256), (h->nrhs + qc - 1) / qc);
    if (h->prec == DMD_PREC_F64X)
      k_prep_herm<ArithDF, NB><<<g, 256, 0, h->st>>>(h->nk, h->nbdm, h->bs, y, h->d_ew, h->d_inv, ta, h->expt,
                                                      (float2*)h->d_rs, h->d_acc, h->d_hflag, fref, h->d_acc0, h->lin,
                                                      h->nrhs, qc, h->d_ph, 1);
    else if (h->use_tc)  // one thread per (rank, state chunk) for the tensor-core form
      k_prep_tc<NB><<<dim3(blocks_for(h->nk, 128), (h->nrhs + qc - 1) / qc), 128, 0, h->st>>>(
          h->nk, h->nbdm, h->bs, y, h->d_ew, h->d_inv, ta, h->expt, (float*)h->d_rs, h->d_hflag, fref, h->nrhs, qc,
          (float2*)h->d_ph);
    else if (deviation_form(h->prec))
      k_prep_herm<ArithF32, NB><<<g, 256, 0, h->st>>>(h->nk, h->nbdm, h->bs, y, h->d_ew, h->d_inv, ta, h->expt,
                                                       (float*)h->d_rs, h->use_tc ? nullptr : h->d_acc, h->d_hflag,
                                                       fref, h->d_acc0, h->lin, h->nrhs, qc, h->d_ph, h->use_tc ? 0 : 1);
    else
      k_prep_herm<ArithF64, NB><<<g, 256, 0, h->st>>>(h->nk, h->nbdm, h->bs, y, h->d_ew, h->d_inv, ta, h->expt,
                                                       (double*)h->d_rs, h->d_acc, h->d_hflag, fref, h->d_acc0, h->lin,
                                                       h->nrhs, qc, h->d_ph, 1);
  }
  h->launches++;
  CKL();
  return DMD_OK;
}

// the Hermitian pass and the gated anti-Hermitian pass of the nb = 2 contraction
template <typename A, int NB, int L, int NST, int MB, int RW = 1, bool FA = false>
void herm_pair_launches(dmd_handle* h, const typename A::relem* rs, size_t half) {
  typedef CbTmaSmem<A, NB, L, NST, RW, FA> S;
  const size_t cstride = (size_t)h->nk * 2 * h->nb2;  // coordinates and sums per state
  const long long warps = (long long)h->nitems * ((h->nrhs + RW - 1) / RW);
  const unsigned g = blocks_for(warps, 4);
  k_pairs_herm<A, NB, L, NST, MB, false, RW, FA><<<g, 128, S::cta_bytes, h->st>>>(
      h->d_items, h->nitems, h->d_rb, (const typename A::elem*)h->d_P, rs, (double*)h->d_acc, h->nk, nullptr, h->d_err,
      h->nrhs, cstride, 2 * cstride);
  k_pairs_herm<A, NB, L, NST, MB, true, RW, FA><<<g, 128, S::cta_bytes, h->st>>>(
      h->d_items, h->nitems, h->d_rb, (const typename A::elem*)h->d_P, rs + half, (double*)h->d_acc, h->nk,
      h->d_hflag, h->d_err, h->nrhs, cstride, 2 * cstride);
}

template <typename A, int NB, int L, int NST, int MB, int RW = 1, bool FA = false>
cudaError_t herm_pair_attrs() {
  const int bytes = (int)CbTmaSmem<A, NB, L, NST, RW, FA>::cta_bytes;
  cudaError_t e = cudaFuncSetAttribute(k_pairs_herm<A, NB, L, NST, MB, false, RW, FA>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(k_pairs_herm<A, NB, L, NST, MB, true, RW, FA>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
  return e;
}

// tensor-core batched form: pack the coordinates, then the Hermitian pass and the gated
// anti-Hermitian pass (dmd_batched_tc.cuh)
template <int NB>
void tc_launches(dmd_handle* h, size_t half) {
  const size_t per = (size_t)h->nrhs * h->nk * NB * NB;
  k_pack_tc<NB><<<dim3(blocks_for((long long)per, 256), 2), 256, 0, h->st>>>(h->nk, h->nrhs, h->ngroups, h->nmb,
                                                                         (const float*)h->d_rs, h->d_tcA, h->d_hflag);
  const size_t apart = (size_t)h->ngroups * h->nmb * TC_ABLOCK;
  const size_t astride = (size_t)h->nk * 2 * h->nb2;
  const unsigned g = (unsigned)((size_t)h->ntiles * h->nmb);
  const float ysign = h->lin ? 0.f : -1.f;  // s = -r (deviation form) or 0 (linearized form)
  float2* accf = (float2*)h->d_acc;          // FP32 sums in the tensor-core form
  auto pass = [&](auto kfwd, auto kimag, size_t smem) {
    kfwd<<<g, 128, smem, h->st>>>(h->d_tiles, h->ntiles, h->d_tcB, h->d_tcA, h->nmb, h->nrhs, h->nk, accf, astride,
                                  ysign, nullptr, h->d_err);
    kimag<<<g, 128, smem, h->st>>>(h->d_tiles, h->ntiles, h->d_tcB, h->d_tcA + apart, h->nmb, h->nrhs, h->nk, accf,
                                   astride, ysign, h->d_hflag, h->d_err);
  };
  // pipeline depth (the shape the autotuner chooses): 4, 3 or 2 stages of 48 KB
  if (h->tcst == 3) pass(k_pairs_tc<false, 3, NB>, k_pairs_tc<true, 3, NB>, tc_smem_bytes(3));
  else if (h->tcst == 2) pass(k_pairs_tc<false, 2, NB>, k_pairs_tc<true, 2, NB>, tc_smem_bytes(2));
  else pass(k_pairs_tc<false, 4, NB>, k_pairs_tc<true, 4, NB>, tc_smem_bytes(4));
  (void)half;
  h->launches += 1;  // the packing launch; the two passes are counted with the other forms
}

template <int NB>
int launch_pairs(dmd_handle* h) {
  if (h->npair == 0) return DMD_OK;
  ProfScope ps(h, 1);
  if (h->use_sp) {  // stored elements only, one thread per output element of every k-point
    k_pairs_sparse<NB><<<blocks_for((long long)h->nk * 2 * NB * NB, 256), 256, 0, h->st>>>(
        h->nk, h->d_sp_base, h->d_sp_len, h->d_sp_val, h->d_sp_gidx, h->d_rs, h->d_acc);
  } else if (!h->use_cb) {
    const long long nthr = h->npair * 4LL * NB * NB;
    k_pairs_f64_atomic<NB><<<blocks_for(nthr, 256), 256, 0, h->st>>>(h->npair, h->d_kk, h->d_P, h->d_rs, h->d_acc);
  } else {
    if constexpr (NB == 2 || NB == 4) {
      // Hermitian coordinates; the second launch carries the anti-Hermitian part of a state that is
      // not exactly Hermitian and returns at once unless the prep kernel raised d_hflag
      const size_t half = (size_t)h->nk * 2 * h->nb2 * h->nrhs;  // coordinates per part
      if (h->use_tc) {
        tc_launches<NB>(h, half);
      } else if (h->nrhs > 1) {  // batched form: reduced-precision arithmetics only (dmd_create)
        const float* rs = (const float*)h->d_rs;
        if (h->prec == DMD_PREC_BF16X2) herm_pair_launches<ArithBF2, NB, 4, 2, 2, 4>(h, rs, half);
        else if (h->brw == 8) herm_pair_launches<ArithF32, NB, 4, 2, 2, 8>(h, rs, half);
        else herm_pair_launches<ArithF32, NB, 4, 2, 2, 4>(h, rs, half);
      } else if (h->prec == DMD_PREC_F64X) {
        const float2* rs = (const float2*)h->d_rs;
        if constexpr (NB == 4) {
          herm_pair_launches<ArithDF, NB, 2, 2, 4>(h, rs, half);
        } else {
          switch (h->pcfg) {
            case 1: herm_pair_launches<ArithDF, NB, 2, 3, 3>(h, rs, half); break;
            case 2: herm_pair_launches<ArithDF, NB, 1, 4, 4>(h, rs, half); break;
            case 3: herm_pair_launches<ArithDF, NB, 1, 3, 4>(h, rs, half); break;
            case 4: herm_pair_launches<ArithDF, NB, 1, 6, 3>(h, rs, half); break;
            default: herm_pair_launches<ArithDF, NB, 2, 2, 4>(h, rs, half); break;
          }
        }
      } else if (h->prec == DMD_PREC_F32) {
        herm_pair_launches<ArithF32, NB, 4, 2, 5>(h, (const float*)h->d_rs, half);
      } else if (h->prec == DMD_PREC_BF16X2) {
        herm_pair_launches<ArithBF2, NB, 4, 2, 5>(h, (const float*)h->d_rs, half);
      } else {
        const double* rs = (const double*)h->d_rs;
        if constexpr (NB == 2) {
          // shapes of the FP64 contraction (autotuned; 1 by default): 0 reduces the forward partials
          // over the warp; 1-3 add them with FP64 reductions in L2 (off the FP64 pipe: 2.65 -> 2.47 ms
          // per launch on the 9.7M-pair workload), with 4 or 5 CTAs per SM
          switch (h->pcfg64) {
            case 1: herm_pair_launches<ArithF64, NB, 2, 2, 4, 1, true>(h, rs, half); break;
            case 2: herm_pair_launches<ArithF64, NB, 2, 2, 5, 1, true>(h, rs, half); break;
            case 3: herm_pair_launches<ArithF64, NB, 1, 4, 5, 1, true>(h, rs, half); break;
            default: herm_pair_launches<ArithF64, NB, 2, 2, 4>(h, rs, half); break;
          }
        } else {
          herm_pair_launches<ArithF64, NB, 2, 2, 4>(h, rs, half);
        }
      }
      h->launches++;
    }
  }
  h->launches++;
  CKL();
  return DMD_OK;
}

template <int NB>
int launch_finish(dmd_handle* h, FinishArgs a) {
  ProfScope ps(h, 2);
  const dim3 g(blocks_for(h->nk, 128), h->nrhs);
  if constexpr (NB == 2 || NB == 4) {
    if (h->use_tc) {  // split FP64 / FP32 finish of the tensor-core form
      if (NB == 4 && h->nbdm == NB)  // one thread per row: a quarter of the registers
        k_finish_rows<NB><<<dim3(blocks_for(h->nk, 128 / NB), h->nrhs), 128, 0, h->st>>>(a);
      else if (h->nbdm == NB) k_finish<NB, NB, true><<<g, 128, 0, h->st>>>(a);
      else k_finish<NB, 0, true><<<g, 128, 0, h->st>>>(a);
      h->launches++;
      CKL();
      return DMD_OK;
    }
  }
  if (h->nbdm == NB) k_finish<NB, NB><<<g, 128, 0, h->st>>>(a);
  else k_finish<NB><<<g, 128, 0, h->st>>>(a);
  h->launches++;
  CKL();
  return DMD_OK;
}

FinishArgs base_finish(dmd_handle* h, const double2* y) {
  FinishArgs a;
  memset(&a, 0, sizeof(a));
  a.nk = h->nk;
  a.nbdm = h->nbdm;
  a.bs = h->bs;
  a.prefac = h->prefac;
  a.picture = h->picture;
  a.phase = h->expt;
  a.ew = h->d_ew;
  a.edm = h->d_edm;
  a.H = h->d_H;
  a.eq = h->d_eq;
  a.y = y;
  a.acc = h->d_acc;
  a.ph = h->expt ? h->d_ph : nullptr;  // written by the prep kernels when the phase is on
  a.fref = h->d_fref;
  a.x0y0 = h->d_x0y0;
  a.v0 = h->d_v0;
  a.ph32 = h->use_tc ? (const float2*)h->d_ph : nullptr;  // the tensor-core prep stores FP32 phases
  a.pos = h->use_cb ? h->d_pos : nullptr;
  a.herm = h->use_cb;
  a.lin = h->lin;
  a.hflag = h->use_cb ? h->d_hflag : nullptr;
  a.nrhs = h->nrhs;
  a.sstride = h->nstate1;
  a.astride = (size_t)h->nk * 2 * h->nb2;
  a.want_eph = 1;
  a.want_coh = (h->picture == DMD_PICTURE_SCHRODINGER || h->d_H) ? 1 : 0;
  return a;
}

template <int NB>
int ee_rebuild(dmd_handle* h, const double2* y, const TimeArg& ta, bool eq);

template <int NB>
int rhs_impl(dmd_handle* h, const double2* y, const TimeArg& ta, FinishArgs fa) {
  int s;
  if constexpr (NB == 2 || NB == 4) {
    // e-e operators rebuilt from this state first (update_scatt_inside, DensityMatrix_Dynamics.h:263)
    if (h->ee_on && h->ee_every && fa.want_eph && (s = ee_rebuild<NB>(h, y, ta, false))) return s;
  }
  if (fa.want_eph) {
    if ((s = launch_prep<NB>(h, y, ta))) return s;
    if ((s = launch_pairs<NB>(h))) return s;
  }
  fa.ta = ta;
  return launch_finish<NB>(h, fa);
}

int rhs(dmd_handle* h, const double2* y, const TimeArg& ta, FinishArgs fa) {
  switch (h->nb) {
    case 1: return rhs_impl<1>(h, y, ta, fa);
    case 2: return rhs_impl<2>(h, y, ta, fa);
    case 3: return rhs_impl<3>(h, y, ta, fa);
    case 4: return rhs_impl<4>(h, y, ta, fa);
  }
  return fail(h, DMD_E_ARG, "nb out of range");
}

TimeArg time_value(double t) {
  TimeArg ta;
  ta.t = t;
  ta.tref = nullptr;
  ta.step = nullptr;
  ta.stage = 0;
  return ta;
}

// plain RHS f(t, in) -> out on device buffers
int rhs_plain(dmd_handle* h, double t, const double2* in, double2* out) {
  FinishArgs fa = base_finish(h, in);
  fa.mode = 0;
  fa.out = out;
  return rhs(h, in, time_value(t), fa);
}

// pair operators in stored order, folded with the additive operators: dP [npair][2][nb4], dkk [npair]
int upload_raw(dmd_handle* h, const dmd_desc* d, double2* dP, int2* dkk);

int upload_pairs(dmd_handle* h, const dmd_desc* d) { return upload_raw(h, d, h->d_P, h->d_kk); }

int upload_raw(dmd_handle* h, const dmd_desc* d, double2* dP, int2* dkk) {
  const size_t nb4 = (size_t)h->nb4;
  const size_t chunk = (size_t)1 << 16;  // pairs per staging chunk
  double2* stage = nullptr;
  CK(cudaMallocHost((void**)&stage, chunk * 2 * nb4 * sizeof(double2)));
  int2* kst = nullptr;
  cudaError_t e = cudaMallocHost((void**)&kst, chunk * sizeof(int2));
  if (e != cudaSuccess) { cudaFreeHost(stage); return fail(h, DMD_E_NOMEM, "pinned staging"); }
  int rc = DMD_OK;
  for (long long p0 = 0; p0 < h->npair && rc == DMD_OK; p0 += (long long)chunk) {
    const size_t n = (size_t)std::min<long long>((long long)chunk, h->npair - p0);
    for (size_t q = 0; q < n; ++q) {
      const uint64_t k1 = d->k1st[p0 + q], k2 = d->k2nd[p0 + q];
      if (k1 >= (uint64_t)h->nk || k2 >= (uint64_t)h->nk) { rc = fail(h, DMD_E_ARG, "k-pair index out of range"); break; }
      kst[q] = make_int2((int)k1, (int)k2);
      const double* s1 = d->P1 + 2 * (p0 + q) * nb4;
      const double* s2 = d->P2 + 2 * (p0 + q) * nb4;
      double2* o = stage + q * 2 * nb4;
      for (size_t j = 0; j < nb4; ++j) {
        double2 v1 = make_double2(s1[2 * j], s1[2 * j + 1]);
        double2 v2 = make_double2(s2[2 * j], s2[2 * j + 1]);
        if (d->P1_add) {  // P += P_add * scale (ElectronImpurity.cpp:38-39, ElectronPhonon.cpp:96-97)
          const double* a1 = d->P1_add + 2 * (p0 + q) * nb4;
          const double* a2 = d->P2_add + 2 * (p0 + q) * nb4;
          v1.x = v1.x + a1[2 * j] * d->add_scale;
          v1.y = v1.y + a1[2 * j + 1] * d->add_scale;
          v2.x = v2.x + a2[2 * j] * d->add_scale;
          v2.y = v2.y + a2[2 * j + 1] * d->add_scale;
        }
        o[j] = v1;
        o[nb4 + j] = v2;
      }
    }
    if (rc) break;
    e = cudaMemcpy(dP + (size_t)p0 * 2 * nb4, stage, n * 2 * nb4 * sizeof(double2), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(dkk + p0, kst, n * sizeof(int2), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) rc = fail(h, DMD_E_CUDA, std::string("P upload: ") + cudaGetErrorString(e));
  }
  cudaFreeHost(stage);
  cudaFreeHost(kst);
  return rc;
}

struct cd {
  double re, im;
};

// Hermitian coordinates v = M q of an nb x nb Hermitian matrix, column j = (p1, p2) of M:
// p1 == p2: v_(p1p1) = q_j;  p1 < p2: v_(p1p2) += q_j, v_(p2p1) += q_j;  p1 > p2: v_(p2p1) += i q_j,
// v_(p1p2) += -i q_j. Returns the entries (index into v, coefficient as (re, im) in {0, +-1}).
__host__ __device__ int herm_col(int nb, int j, int* idx, int* cre, int* cim) {
  const int p1 = j / nb, p2 = j % nb;
  if (p1 == p2) {
    idx[0] = j; cre[0] = 1; cim[0] = 0;
    return 1;
  }
  if (p1 < p2) {
    idx[0] = j; cre[0] = 1; cim[0] = 0;
    idx[1] = p2 * nb + p1; cre[1] = 1; cim[1] = 0;
    return 2;
  }
  idx[0] = p2 * nb + p1; cre[0] = 0; cim[0] = 1;
  idx[1] = j; cre[1] = 0; cim[1] = -1;
  return 2;
}

// z * (cr + i ci) for cr, ci in {0, +-1}: exact
__host__ __device__ inline cd cmul_unit(cd z, int cr, int ci) {
  if (ci == 0) return cr > 0 ? z : cd{-z.re, -z.im};
  return ci > 0 ? cd{-z.im, z.re} : cd{z.im, -z.re};
}

// Q1 = M^H P1 M and Q2 = M^T P2 conj(M) (both nb^2 x nb^2 row-major), the operators of the
// Hermitian-coordinate contraction (dmd_pairs_cb.cuh)
__host__ __device__ void herm_transform(int nb, const cd* P1, const cd* P2, cd* Q1, cd* Q2) {
  const int n2 = nb * nb;
  int ia[2], ra[2], ja[2], ib[2], rb[2], jb[2];
  for (int a = 0; a < n2; ++a) {
    const int na = herm_col(nb, a, ia, ra, ja);
    for (int b = 0; b < n2; ++b) {
      const int nbb = herm_col(nb, b, ib, rb, jb);
      cd q1 = {0, 0}, q2 = {0, 0};
      for (int u = 0; u < na; ++u)
        for (int v = 0; v < nbb; ++v) {
          const cd p1 = P1[ia[u] * n2 + ib[v]], p2 = P2[ia[u] * n2 + ib[v]];
          const cd t1 = cmul_unit(cmul_unit(p1, ra[u], -ja[u]), rb[v], jb[v]);  // conj(ca) P1 cb
          const cd t2 = cmul_unit(cmul_unit(p2, ra[u], ja[u]), rb[v], -jb[v]);  // ca P2 conj(cb)
          q1.re += t1.re;
          q1.im += t1.im;
          q2.re += t2.re;
          q2.im += t2.im;
        }
      Q1[a * n2 + b] = q1;
      Q2[a * n2 + b] = q2;
    }
  }
}

__host__ __device__ uint32_t bf16_bits(float x) {  // round to nearest even (finite values)
  uint32_t u;
  memcpy(&u, &x, 4);
  u += 0x7fffu + ((u >> 16) & 1u);
  return u >> 16;
}
__host__ __device__ float bf16_value(uint32_t b) {
  const uint32_t u = b << 16;
  float x;
  memcpy(&x, &u, 4);
  return x;
}
// one 32-bit word: bf16(x) in the upper half, bf16(x - that) in the lower half
__host__ __device__ uint32_t pack_bf2(double x) {
  const float xf = (float)x;
  const uint32_t hi = bf16_bits(xf);
  const uint32_t lo = bf16_bits((float)(x - (double)bf16_value(hi)));
  return (hi << 16) | lo;
}

__host__ __device__ void pack_elem(int prec, cd v, unsigned char* out) {
  if (prec == DMD_PREC_F64X) {
    const float xh = (float)v.re, yh = (float)v.im;
    const float f[4] = {xh, yh, (float)(v.re - (double)xh), (float)(v.im - (double)yh)};  // high parts, low parts
    memcpy(out, f, 16);
  } else if (prec == DMD_PREC_F32) {
    const float f[2] = {(float)v.re, (float)v.im};
    memcpy(out, f, 8);
  } else if (prec == DMD_PREC_BF16X2) {
    const uint32_t w[2] = {pack_bf2(v.re), pack_bf2(v.im)};
    memcpy(out, w, 8);
  } else {
    const double f[2] = {v.re, v.im};
    memcpy(out, f, 16);
  }
}


// Raw pair operators in stored order, read in chunks: P1 [cnt][nb4], P2 [cnt][nb4] and, when
// present, P1_add, P2_add after them (complex128), into one host buffer.
struct PairSource {
  virtual ~PairSource() {}
  virtual bool has_add() const = 0;
  virtual int read(long long p0, long long cnt, double2* dst) = 0;  // DMD_OK or an error code
  std::string err;
};

struct ArraySource : PairSource {
  const dmd_desc* d;
  size_t nb4;
  ArraySource(const dmd_desc* d_, int nb4_) : d(d_), nb4((size_t)nb4_) {}
  bool has_add() const override { return d->P1_add != nullptr; }
  int read(long long p0, long long cnt, double2* dst) override {
    const size_t n = (size_t)cnt * nb4;
    const double* src[4] = {d->P1, d->P2, d->P1_add, d->P2_add};
    for (int m = 0; m < (has_add() ? 4 : 2); ++m) memcpy(dst + m * n, src[m] + 2 * (size_t)p0 * nb4, n * 16);
    return DMD_OK;
  }
};

// where stored pair src goes in the column-block element store, and what the deviation fold needs
struct CbDst {
  int32_t b0;           // first slot of its row block
  int16_t n, i;         // pairs in the row block, slot
  int32_t pr, pc;       // energy ranks of its row and column k-points (stored orientation)
  int32_t kr, kc;       // the k-points themselves
  int32_t flags;        // bit 0: stored transposed, bit 1: reverse term (k1 < k2)
  int32_t pad;
};

// One thread per pair of a chunk: fold the additive operators, orient, transform to Hermitian
// coordinates (Q1 = M^H P1 M, Q2 = M^T P2 conj(M)), pack in the arithmetic's format and store at
// the pair's slot (element-major inside its row block: Q1 row-major, then Q2 column-major). In the
// deviation form the contraction of diag(f_ref) through the pair is added to acc0 (FP64 atomics).
// Operators of the chunk's pair j, operator m (P1, P2): element e at raw[m sseg + j spair + e], the
// additive ones (or null) at add[m aseg + j apair + e].
struct FillSrc {
  const double2* raw;
  size_t sseg, spair;
  const double2* add;
  size_t aseg, apair;
};

template <int NB>
__global__ void k_cb_fill(long long p0, long long cnt, FillSrc src, double add_scale, const CbDst* __restrict__ dst,
                          int lin, int prec, int esz, unsigned char* __restrict__ store, const double* __restrict__ fw,
                          double* __restrict__ acc0) {
  constexpr int NB2 = NB * NB, NB4 = NB2 * NB2, NE = 2 * NB4;
  const long long j = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (j >= cnt) return;
  const CbDst dd = dst[p0 + j];
  const bool tr = dd.flags & 1, rev = (dd.flags >> 1) & 1;
  cd Pe[2][NB4];
  for (int m = 0; m < 2; ++m) {
    const int sm = tr ? 1 - m : m;  // the transposed pair carries (conj P2, conj P1)
    const double2* sp = src.raw + sm * src.sseg + (size_t)j * src.spair;
    const double2* ap = src.add ? src.add + sm * src.aseg + (size_t)j * src.apair : nullptr;
    for (int e = 0; e < NB4; ++e) {
      double x = sp[e].x, yv = sp[e].y;
      if (ap) {  // P += P_add * scale (ElectronImpurity.cpp:38-39, ElectronPhonon.cpp:87-100)
        x = __dadd_rn(x, __dmul_rn(ap[e].x, add_scale));
        yv = __dadd_rn(yv, __dmul_rn(ap[e].y, add_scale));
      }
      if (lin ? (m == 1) : tr) yv = -yv;
      Pe[m][e] = cd{x, yv};
    }
  }
  cd Q[2][NB4];
  herm_transform(NB, Pe[0], Pe[1], Q[0], Q[1]);
  if (acc0) {  // what the contraction adds for diag(f_ref), in FP64 (see k_prep_herm)
    const double* fr = fw + (size_t)dd.kr * NB;
    const double* fc = fw + (size_t)dd.kc * NB;
    double* ar = acc0 + (size_t)dd.pr * 2 * NB2 * 2;
    double* ac = acc0 + (size_t)dd.pc * 2 * NB2 * 2;
    for (int a = 0; a < NB2; ++a) {
      double x0 = 0, x1 = 0, y0 = 0, y1 = 0, u0 = 0, u1 = 0, v0 = 0, v1 = 0;
      for (int i = 0; i < NB; ++i) {
        const int ii = i * NB + i;
        const cd q1 = Q[0][a * NB2 + ii], q2 = Q[1][ii * NB2 + a];
        x0 = __dadd_rn(x0, __dmul_rn(q1.re, fc[i]));
        x1 = __dadd_rn(x1, __dmul_rn(q1.im, fc[i]));
        y0 = __dadd_rn(y0, __dmul_rn(q2.re, __dsub_rn(1.0, fc[i])));
        y1 = __dadd_rn(y1, __dmul_rn(q2.im, __dsub_rn(1.0, fc[i])));
        if (rev) {
          const cd q1c = Q[0][ii * NB2 + a], q2c = Q[1][a * NB2 + ii];
          u0 = __dadd_rn(u0, __dmul_rn(q1c.re, __dsub_rn(1.0, fr[i])));
          u1 = __dsub_rn(u1, __dmul_rn(q1c.im, __dsub_rn(1.0, fr[i])));
          v0 = __dadd_rn(v0, __dmul_rn(q2c.re, fr[i]));
          v1 = __dsub_rn(v1, __dmul_rn(q2c.im, fr[i]));
        }
      }
      atomicAdd(&ar[2 * a], x0);
      atomicAdd(&ar[2 * a + 1], x1);
      atomicAdd(&ar[2 * (NB2 + a)], y0);
      atomicAdd(&ar[2 * (NB2 + a) + 1], y1);
      if (rev) {
        atomicAdd(&ac[2 * (NB2 + a)], u0);
        atomicAdd(&ac[2 * (NB2 + a) + 1], u1);
        atomicAdd(&ac[2 * a], v0);
        atomicAdd(&ac[2 * a + 1], v1);
      }
    }
  }
  for (int e = 0; e < NE; ++e) {
    // stored element e: Q1 row-major for e < nb^4; Q2 column-major after it (e = nb^4 + cc nb^2 + a
    // holds Q2[a][cc])
    cd qv;
    if (e < NB4) {
      qv = Q[0][e];
    } else {
      const int q = e - NB4, cc = q / NB2, a = q % NB2;
      qv = Q[1][a * NB2 + cc];
    }
    pack_elem(prec, qv, store + ((size_t)dd.b0 * NE + (size_t)e * dd.n + dd.i) * esz);
  }
}

struct CbDst;
int fill_pairs_cb(dmd_handle* h, PairSource& src, const std::vector<CbDst>& dst, bool dev);

// column-block layout upload: pairs permuted into row blocks, element-major inside each block,
// folded with the optional additive operators and converted to the arithmetic's element format
int upload_pairs_cb(dmd_handle* h, const dmd_desc* d) {
  const int nb = h->nb, nb4 = h->nb4;
  std::vector<double> ew((size_t)h->nk * nb);
  for (int k = 0; k < h->nk; ++k)
    for (int b = 0; b < nb; ++b) ew[(size_t)k * nb + b] = d->e_dm[(size_t)k * h->nbdm + h->bs + b];
  dmd::PairLayout L;
  const int G = h->nb2 / 4, W = 32 / G;  // lanes per pair, columns per column block
  // pairs per work item: 512 (a warp's share on large workloads), fewer when the workload would
  // not give every SM its 16 resident warps
  int ppi = 512 / G;
  {
    int nsm = 0;
    if (cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, h->dev) != cudaSuccess || nsm <= 0) nsm = 1;
    const long long want = (long long)nsm * 16;
    if (h->npair / ppi < want) ppi = (int)std::max<long long>(1, h->npair / want);
  }
  if (!dmd::build_pair_layout(h->nk, nb, ew.data(), h->npair, d->k1st, d->k2nd, ppi, W, L))
    return fail(h, DMD_E_ARG, "k-pair index out of range");
  h->nitems = (int)L.items.size();
  h->nrb = (long long)L.rb.size();
  // pair-kernel shape (stage lines, resident CTAs per SM); 0 is the default, the others serve tuning
  if (const char* v = getenv("DMD_PAIR_CFG")) h->pcfg = atoi(v);
  if (const char* v = getenv("DMD_PAIR_CFG64")) h->pcfg64 = atoi(v);
  if (nb == 2) {
    cudaError_t (*const attrs[])() = {
        herm_pair_attrs<ArithDF, 2, 2, 2, 4>, herm_pair_attrs<ArithDF, 2, 2, 3, 3>, herm_pair_attrs<ArithDF, 2, 1, 4, 4>,
        herm_pair_attrs<ArithDF, 2, 1, 3, 4>, herm_pair_attrs<ArithDF, 2, 1, 6, 3>, herm_pair_attrs<ArithF64, 2, 2, 2, 4>,
        herm_pair_attrs<ArithF64, 2, 2, 2, 4, 1, true>, herm_pair_attrs<ArithF64, 2, 2, 2, 5, 1, true>,
        herm_pair_attrs<ArithF64, 2, 1, 4, 5, 1, true>,
        herm_pair_attrs<ArithF32, 2, 4, 2, 5>, herm_pair_attrs<ArithBF2, 2, 4, 2, 5>,
        herm_pair_attrs<ArithF32, 2, 4, 2, 2, 4>, herm_pair_attrs<ArithF32, 2, 4, 2, 2, 8>,
        herm_pair_attrs<ArithBF2, 2, 4, 2, 2, 4>};
    for (auto fn : attrs) CK(fn());
  } else {
    cudaError_t (*const attrs[])() = {herm_pair_attrs<ArithDF, 4, 2, 2, 4>, herm_pair_attrs<ArithF64, 4, 2, 2, 4>,
                                      herm_pair_attrs<ArithF32, 4, 4, 2, 5>, herm_pair_attrs<ArithBF2, 4, 4, 2, 5>,
                                      herm_pair_attrs<ArithF32, 4, 4, 2, 2, 4>, herm_pair_attrs<ArithF32, 4, 4, 2, 2, 8>,
                                      herm_pair_attrs<ArithBF2, 4, 4, 2, 2, 4>};
    for (auto fn : attrs) CK(fn());
  }
  int rc;
  if ((rc = dalloc(h, &h->d_pos, (size_t)h->nk)) || (rc = dalloc(h, &h->d_rb, L.rb.size())) ||
      (rc = dalloc(h, &h->d_items, L.items.size())))
    return rc;
  CK(cudaMemcpy(h->d_pos, L.pos.data(), L.pos.size() * 4, cudaMemcpyHostToDevice));
  if ((rc = dalloc(h, &h->d_inv, (size_t)h->nk))) return rc;
  CK(cudaMemcpy(h->d_inv, L.inv.data(), L.inv.size() * 4, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(h->d_rb, L.rb.data(), L.rb.size() * sizeof(dmd::RowBlock), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(h->d_items, L.items.data(), L.items.size() * sizeof(dmd::WorkItem), cudaMemcpyHostToDevice));
  const int esz = elem_bytes(h->prec);
  // deviation form: the constant contraction of diag(f_ref), position order [nk][2][nb2]
  const bool dev = deviation_form(h->prec) && !h->lin;
  std::vector<double> fw;
  if (dev || h->lin) {
    fw.assign((size_t)h->nk * nb, 0.0);
    if (d->f_ref)
      for (int k = 0; k < h->nk; ++k)
        for (int b = 0; b < nb; ++b) fw[(size_t)k * nb + b] = d->f_ref[(size_t)k * h->nbdm + h->bs + b];
    if ((rc = dalloc(h, &h->d_fref, fw.size()))) return rc;
    CK(cudaMemcpy(h->d_fref, fw.data(), fw.size() * 8, cudaMemcpyHostToDevice));
  }
  if (dev) {
    if ((rc = dalloc(h, &h->d_acc0, (size_t)h->nk * 2 * h->nb2))) return rc;
    CK(cudaMemset(h->d_acc0, 0, (size_t)h->nk * 2 * h->nb2 * 16));
  }
  // destination of every stored pair
  std::vector<CbDst> dst((size_t)h->npair);
  for (size_t r = 0; r < L.rb.size(); ++r) {
    const size_t b0 = L.rb[r].pair0;
    const int n = __builtin_popcount(L.rb[r].mask);
    for (int i = 0; i < n; ++i) {
      const size_t src = L.src[b0 + i];
      const bool tr = L.transposed[b0 + i] != 0;
      const uint64_t kr = tr ? d->k2nd[src] : d->k1st[src], kc = tr ? d->k1st[src] : d->k2nd[src];
      CbDst& o = dst[src];
      o.b0 = (int32_t)b0;
      o.n = (int16_t)n;
      o.i = (int16_t)i;
      o.kr = (int32_t)kr;
      o.kc = (int32_t)kc;
      o.pr = L.pos[kr];
      o.pc = L.pos[kc];
      o.flags = (tr ? 1 : 0) | (d->k1st[src] < d->k2nd[src] ? 2 : 0);
      o.pad = 0;
    }
  }
  PairSource* srcp = h->src ? h->src : nullptr;
  ArraySource arrays(d, nb4);
  if (!srcp) srcp = &arrays;
  return fill_pairs_cb(h, *srcp, dst, dev);
}

// Streams the raw operators through two pinned chunks and the fill kernel: the host reads chunk
// c + 1 while the device converts chunk c.
int fill_pairs_cb(dmd_handle* h, PairSource& src, const std::vector<CbDst>& dst, bool dev) {
  const int nb4 = h->nb4, esz = elem_bytes(h->prec);
  const int nseg = src.has_add() ? 4 : 2;
  const size_t per_pair = (size_t)nseg * nb4 * 16;
  long long chunk = std::max<long long>(1, std::min<long long>(h->npair, (256LL << 20) / (long long)per_pair));
  if (const char* v = getenv("DMD_FILL_CHUNK")) chunk = std::max(1LL, std::min<long long>(chunk, atoll(v)));  // tests
  CbDst* d_dst = nullptr;
  int rc;
  if ((rc = dalloc(h, &d_dst, dst.size()))) return rc;
  double2* pin[2] = {nullptr, nullptr};
  double2* dev_raw[2] = {nullptr, nullptr};
  cudaEvent_t done[2] = {nullptr, nullptr};
  auto cleanup = [&]() {
    cudaStreamSynchronize(h->st);
    for (int b = 0; b < 2; ++b) {
      if (pin[b]) cudaFreeHost(pin[b]);
      if (dev_raw[b]) cudaFree(dev_raw[b]);
      if (done[b]) cudaEventDestroy(done[b]);
    }
    cudaFree(d_dst);
  };
  cudaError_t e = cudaMemcpy(d_dst, dst.data(), dst.size() * sizeof(CbDst), cudaMemcpyHostToDevice);
  for (int b = 0; b < 2 && e == cudaSuccess; ++b) {
    e = cudaMallocHost((void**)&pin[b], (size_t)chunk * per_pair);
    if (e == cudaSuccess) e = cudaMalloc((void**)&dev_raw[b], (size_t)chunk * per_pair);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&done[b], cudaEventDisableTiming);
  }
  if (e != cudaSuccess) {
    cleanup();
    return fail(h, e == cudaErrorMemoryAllocation ? DMD_E_NOMEM : DMD_E_CUDA,
                std::string("pair staging: ") + cudaGetErrorString(e));
  }
  int b = 0;
  for (long long p0 = 0; p0 < h->npair; p0 += chunk, b ^= 1) {
    const long long cnt = std::min<long long>(chunk, h->npair - p0);
    if (cudaEventSynchronize(done[b]) != cudaSuccess) break;  // the copy out of this buffer has finished
    if ((rc = src.read(p0, cnt, pin[b]))) {
      cleanup();
      return fail(h, rc, src.err.empty() ? "reading the pair operators" : src.err);
    }
    // the chunk is contiguous in pin[b] with segment stride cnt * nb4
    e = cudaMemcpyAsync(dev_raw[b], pin[b], (size_t)cnt * per_pair, cudaMemcpyHostToDevice, h->st);
    if (e != cudaSuccess) break;
    cudaEventRecord(done[b], h->st);
    const unsigned g = blocks_for(cnt, 128);
    double* a0 = dev ? (double*)h->d_acc0 : nullptr;
    const size_t nn = (size_t)cnt * nb4;
    const FillSrc fs = {dev_raw[b], nn, (size_t)nb4, src.has_add() ? dev_raw[b] + 2 * nn : nullptr, nn, (size_t)nb4};
    if (h->nb == 2)
      k_cb_fill<2><<<g, 128, 0, h->st>>>(p0, cnt, fs, h->add_scale, d_dst, h->lin, h->prec, esz,
                                         (unsigned char*)h->d_P, h->d_fref, a0);
    else
      k_cb_fill<4><<<g, 128, 0, h->st>>>(p0, cnt, fs, h->add_scale, d_dst, h->lin, h->prec, esz,
                                         (unsigned char*)h->d_P, h->d_fref, a0);
    e = cudaGetLastError();
    if (e != cudaSuccess) break;
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(h->st);
  if (e == cudaSuccess && (h->eek || h->adj)) {  // kept for the e-e model's refills, dmd_add_operators
    h->d_dst = d_dst;
    d_dst = nullptr;
  }
  cleanup();
  if (e != cudaSuccess) return fail(h, DMD_E_CUDA, std::string("pair fill: ") + cudaGetErrorString(e));
  return DMD_OK;
}

// Effective P1, P2 of stored pair src in its given orientation (k1 <- k2): folded with the additive
// operators (ElectronImpurity.cpp:38-39, ElectronPhonon.cpp:96-97); the linearized form carries
// conj(Lji) in the P2 slot (the reverse operator, see dmd_pairs_cb.cuh)
void pair_operators(const dmd_handle* h, const dmd_desc* d, size_t src, cd* P1, cd* P2) {
  const int nb4 = h->nb4;
  for (int m = 0; m < 2; ++m) {
    const double* sp = (m == 0 ? d->P1 : d->P2) + 2 * src * nb4;
    const double* ap = (m == 0 ? d->P1_add : d->P2_add);
    cd* out = m == 0 ? P1 : P2;
    for (int e = 0; e < nb4; ++e) {
      double x = sp[2 * e], yv = sp[2 * e + 1];
      if (ap) {
        x = x + ap[2 * src * nb4 + 2 * e] * d->add_scale;
        yv = yv + ap[2 * src * nb4 + 2 * e + 1] * d->add_scale;
      }
      if (h->lin && m == 1) yv = -yv;
      out[e] = {x, yv};
    }
  }
}

// Tensor-core batched form (nb = 2, dmd_batched_tc.cuh): every stored pair becomes the directed
// operators (k1 <- k2): A = Q1, B = Q2 and, with the reverse term (k1 < k2, evolve_eph.cpp:101),
// (k2 <- k1): A = conj(Q2), B = conj(Q1). They are bucketed by the row tile of their target
// (16 energy ranks); a tile's column groups (8 ranks) between the first and the last it touches form
// dense blocks laid out as the MMA reads them, split into bf16 hi + lo. Tiles are built on host threads.
template <int NB>
cudaError_t tc_attrs() {
  cudaError_t e = cudaSuccess;
  auto set = [&](auto k, int nst) {
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tc_smem_bytes(nst));
  };
  set(k_pairs_tc<false, 4, NB>, 4);
  set(k_pairs_tc<true, 4, NB>, 4);
  set(k_pairs_tc<false, 3, NB>, 3);
  set(k_pairs_tc<true, 3, NB>, 3);
  set(k_pairs_tc<false, 2, NB>, 2);
  set(k_pairs_tc<true, 2, NB>, 2);
  return e;
}

// Sparse form: the stored elements (|P| > kSparseThr) regrouped by the k-point and output element
// they update (dmd_sparse.cuh). The operators are read in chunks from the handle's source (arrays or
// files) and folded with the additive operators in FP64 as the dense forms fold them; every pair
// (k1, k2) gives its forward products to k1 (P1 rows, P2 columns, sources in k2's coordinates) and,
// for k1 < k2, the reverse ones to k2 (conj(P2) rows, conj(P1) columns, sources in k1's).
constexpr double kSparseThr = 1e-40;  // the reference's default alg_thr_sparseP (parameters.cpp:120)

int upload_pairs_sparse(dmd_handle* h, const dmd_desc* d) {
  const int nb2 = h->nb2, TPR = 2 * nb2;
  const size_t nb4 = (size_t)h->nb4;
  const long long np = h->npair;
  const int nk = h->nk;
  // pass 1 over the pair list: the pairs that feed each k-point (forward and reverse), as
  // (pair, direction) in pair order
  std::vector<long long> rowptr((size_t)nk + 1, 0);
  for (long long p = 0; p < np; ++p) {
    const uint64_t k1 = d->k1st[p], k2 = d->k2nd[p];
    if (k1 >= (uint64_t)nk || k2 >= (uint64_t)nk) return fail(h, DMD_E_ARG, "k-pair index out of range");
    rowptr[k1 + 1]++;
    if (k1 < k2) rowptr[k2 + 1]++;
  }
  for (int k = 0; k < nk; ++k) rowptr[k + 1] += rowptr[k];
  // pass 2 over the operators: per pair, the count of stored elements in every row and column of
  // P1 and P2, and the elements themselves (compact, in pair order)
  std::vector<uint8_t> cnt((size_t)np * 4 * nb2);  // [pair][P1 rows | P1 cols | P2 rows | P2 cols]
  std::vector<long long> pe((size_t)np + 1, 0);    // first stored element of each pair
  std::vector<double2> ev;                         // P1's stored elements (row-major), then P2's
  std::vector<uint8_t> ei;                         // their (row, column) as row * nb^2 + column
  ArraySource asrc(d, h->nb4);
  PairSource* src = h->src ? h->src : &asrc;
  const bool add = src->has_add();
  const long long chunk = std::max<long long>(1, (256LL << 20) / (long long)(4 * nb4 * 16));
  std::vector<double2> buf((size_t)std::min(chunk, std::max<long long>(np, 1)) * 4 * nb4);
  for (long long p0 = 0; p0 < np; p0 += chunk) {
    const long long nc = std::min(chunk, np - p0);
    int rc = src->read(p0, nc, buf.data());
    if (rc) return fail(h, rc, src->err.empty() ? std::string("reading the pair operators") : src->err);
    const size_t n = (size_t)nc * nb4;
    double2* P1 = buf.data();
    double2* P2 = P1 + n;
    if (add) {  // P += add_scale P_add (ElectronImpurity.cpp:38-39)
      const double2* A1 = P2 + n;
      const double2* A2 = A1 + n;
      for (size_t i = 0; i < n; ++i) {
        P1[i] = mk2(P1[i].x + h->add_scale * A1[i].x, P1[i].y + h->add_scale * A1[i].y);
        P2[i] = mk2(P2[i].x + h->add_scale * A2[i].x, P2[i].y + h->add_scale * A2[i].y);
      }
    }
    for (long long q = 0; q < nc; ++q) {
      const long long p = p0 + q;
      uint8_t* c = &cnt[(size_t)p * 4 * nb2];
      for (int m = 0; m < 2; ++m) {
        const double2* M = (m ? P2 : P1) + (size_t)q * nb4;
        for (int a = 0; a < nb2; ++a)
          for (int b = 0; b < nb2; ++b) {
            const double2 v = M[(size_t)a * nb2 + b];
            if (std::sqrt(v.x * v.x + v.y * v.y) > kSparseThr) {
              ev.push_back(v);
              ei.push_back((uint8_t)(a * nb2 + b));
              c[2 * m * nb2 + a]++;
              c[(2 * m + 1) * nb2 + b]++;
            }
          }
      }
      pe[(size_t)p + 1] = (long long)ev.size();
    }
  }
  // the products per output thread of every k-point: L_k = the longest list among its threads
  std::vector<int> len((size_t)nk, 0);
  std::vector<long long> base((size_t)nk + 1, 0);
  {
    std::vector<int> cl((size_t)nk * TPR, 0);
    for (long long p = 0; p < np; ++p) {
      const int k1 = (int)d->k1st[p], k2 = (int)d->k2nd[p];
      const uint8_t* c = &cnt[(size_t)p * 4 * nb2];
      for (int a = 0; a < nb2; ++a) {
        cl[(size_t)k1 * TPR + a] += c[a];                    // X_k1[a]: row a of P1
        cl[(size_t)k1 * TPR + nb2 + a] += c[3 * nb2 + a];    // Y_k1[a]: column a of P2
        if (k1 < k2) {
          cl[(size_t)k2 * TPR + a] += c[2 * nb2 + a];        // X_k2[a]: row a of conj(P2)
          cl[(size_t)k2 * TPR + nb2 + a] += c[nb2 + a];      // Y_k2[a]: column a of conj(P1)
        }
      }
    }
    for (int k = 0; k < nk; ++k) {
      int m = 0;
      for (int l = 0; l < TPR; ++l) m = std::max(m, cl[(size_t)k * TPR + l]);
      len[k] = m;
      base[(size_t)k + 1] = base[k] + (long long)m * TPR;
    }
  }
  const long long nslot = base[nk];
  std::vector<double2> val((size_t)std::max<long long>(1, nslot), mk2(0.0, 0.0));
  std::vector<int> gidx((size_t)std::max<long long>(1, nslot), 0);
  std::vector<int> fillc((size_t)nk * TPR, 0);
  auto put = [&](int k, int l, double2 v, int gi) {
    const long long s = base[k] + (long long)fillc[(size_t)k * TPR + l]++ * TPR + l;
    val[(size_t)s] = v;
    gidx[(size_t)s] = gi;
  };
  for (long long p = 0; p < np; ++p) {
    const int k1 = (int)d->k1st[p], k2 = (int)d->k2nd[p];
    const bool rev = k1 < k2;
    long long e = pe[(size_t)p];
    for (int m = 0; m < 2; ++m) {
      const uint8_t* c = &cnt[(size_t)p * 4 * nb2 + 2 * m * nb2];
      long long ne = 0;
      for (int a = 0; a < nb2; ++a) ne += c[a];
      for (long long q = 0; q < ne; ++q, ++e) {
        const int a = ei[(size_t)e] / nb2, b = ei[(size_t)e] % nb2;
        const double2 v = ev[(size_t)e], vc = mk2(v.x, -v.y);
        if (m == 0) {  // P1[a][b]: X_k1[a] += P1 rt_k2[b]; reverse Y_k2[b] += st_k1[a] conj(P1)
          put(k1, a, v, k2 * TPR + b);
          if (rev) put(k2, nb2 + b, vc, k1 * TPR + nb2 + a);
        } else {       // P2[a][b]: Y_k1[b] += st_k2[a] P2; reverse X_k2[a] += conj(P2) rt_k1[b]
          put(k1, nb2 + b, v, k2 * TPR + nb2 + a);
          if (rev) put(k2, a, vc, k1 * TPR + b);
        }
      }
    }
  }
  h->sp_nel = 0;
  for (long long p = 0; p < np; ++p) {
    const long long ne = pe[(size_t)p + 1] - pe[(size_t)p];
    h->sp_nel += ne * (d->k1st[p] < d->k2nd[p] ? 2 : 1);
  }
  h->sp_nslot = nslot;
  int rc;
  if ((rc = dalloc(h, &h->d_sp_base, (size_t)nk)) || (rc = dalloc(h, &h->d_sp_len, (size_t)nk)) ||
      (rc = dalloc(h, &h->d_sp_val, val.size())) || (rc = dalloc(h, &h->d_sp_gidx, gidx.size())))
    return rc;
  CK(cudaMemcpy(h->d_sp_base, base.data(), (size_t)nk * sizeof(long long), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(h->d_sp_len, len.data(), (size_t)nk * sizeof(int), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(h->d_sp_val, val.data(), val.size() * 16, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(h->d_sp_gidx, gidx.data(), gidx.size() * 4, cudaMemcpyHostToDevice));
  h->pair_bytes = (int64_t)(nslot * 20 + (long long)nk * 12);
  return DMD_OK;
}

int upload_pairs_tc(dmd_handle* h, const dmd_desc* d) {
  const int nb = h->nb, nk = h->nk;
  std::vector<double> ew((size_t)nk * nb);
  for (int k = 0; k < nk; ++k)
    for (int b = 0; b < nb; ++b) ew[(size_t)k * nb + b] = d->e_dm[(size_t)k * h->nbdm + h->bs + b];
  dmd::PairLayout L;  // only the energy ranks are used
  if (!dmd::build_pair_layout(nk, nb, ew.data(), h->npair, d->k1st, d->k2nd, 512, 32, L))
    return fail(h, DMD_E_ARG, "k-pair index out of range");
  L.rb.clear();
  L.items.clear();
  L.src.clear();
  if (nb == 4) CK(tc_attrs<4>());
  else CK(tc_attrs<2>());
  // rows per tile and columns per group: a block is 128 X rows (TR rows x nb^2 x re|im) by K = 32
  // (CG columns x nb^2)
  const int TR = tc_tr(h->nb2), CG = tc_cg(h->nb2);
  h->ntiles = (nk + TR - 1) / TR;
  h->ngroups = (nk + CG - 1) / CG;
  h->nmb = (h->nrhs + TC_M - 1) / TC_M;
  int rc;
  if ((rc = dalloc(h, &h->d_pos, (size_t)nk)) || (rc = dalloc(h, &h->d_inv, (size_t)nk))) return rc;
  CK(cudaMemcpy(h->d_pos, L.pos.data(), (size_t)nk * 4, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(h->d_inv, L.inv.data(), (size_t)nk * 4, cudaMemcpyHostToDevice));
  // directed entries (src << 1 | reverse) bucketed by row tile
  const size_t np = (size_t)h->npair;
  std::vector<size_t> start((size_t)h->ntiles + 1, 0);
  auto row_of = [&](size_t src, int dir) { return L.pos[dir ? d->k2nd[src] : d->k1st[src]]; };
  auto col_of = [&](size_t src, int dir) { return L.pos[dir ? d->k1st[src] : d->k2nd[src]]; };
  for (size_t p = 0; p < np; ++p) {
    start[row_of(p, 0) / TR + 1]++;
    if (d->k1st[p] < d->k2nd[p]) start[row_of(p, 1) / TR + 1]++;
  }
  for (int t = 0; t < h->ntiles; ++t) start[t + 1] += start[t];
  std::vector<uint64_t> ent(start[h->ntiles]);
  {
    std::vector<size_t> fill(start.begin(), start.end() - 1);
    for (size_t p = 0; p < np; ++p) {
      ent[fill[row_of(p, 0) / TR]++] = (uint64_t)p << 1;
      if (d->k1st[p] < d->k2nd[p]) ent[fill[row_of(p, 1) / TR]++] = ((uint64_t)p << 1) | 1u;
    }
  }
  std::vector<TcTile> tiles(h->ntiles);
  int64_t nblocks = 0;
  for (int t = 0; t < h->ntiles; ++t) {
    int gmin = INT32_MAX, gmax = -1;
    for (size_t e = start[t]; e < start[t + 1]; ++e) {
      const int g = col_of(ent[e] >> 1, (int)(ent[e] & 1)) / CG;
      gmin = std::min(gmin, g);
      gmax = std::max(gmax, g);
    }
    tiles[t].boff = nblocks;
    if (gmax < 0) {
      tiles[t].g0 = tiles[t].g1 = 0;
    } else {
      tiles[t].g0 = gmin;
      tiles[t].g1 = gmax + 1;
      nblocks += gmax + 1 - gmin;
    }
  }
  if ((rc = dalloc(h, &h->d_tiles, tiles.size())) || (rc = dalloc(h, &h->d_tcB, (size_t)nblocks * TC_BLOCK)) ||
      (rc = dalloc(h, &h->d_tcA, (size_t)2 * h->ngroups * h->nmb * TC_ABLOCK)))
    return rc;
  CK(cudaMemcpy(h->d_tiles, tiles.data(), tiles.size() * sizeof(TcTile), cudaMemcpyHostToDevice));
  h->pair_bytes = nblocks * (int64_t)TC_BLOCK_BYTES;
  CK(cudaMemset(h->d_tcA, 0, (size_t)2 * h->ngroups * h->nmb * TC_ABLOCK * 2));
  // deviation form: acc0 = contraction of diag(f_ref) in FP64, position order [nk][2][nb2]
  const bool dev = deviation_form(h->prec) && !h->lin;
  std::vector<double> fw;
  std::vector<cd> acc0;
  if (dev || h->lin) {
    fw.assign((size_t)nk * nb, 0.0);
    if (d->f_ref)
      for (int k = 0; k < nk; ++k)
        for (int b = 0; b < nb; ++b) fw[(size_t)k * nb + b] = d->f_ref[(size_t)k * h->nbdm + h->bs + b];
    if (dev) acc0.assign((size_t)nk * 2 * h->nb2, cd{0, 0});
  }
  // tiles in chunks of at most kChunk blocks (one tile at least), one pinned staging buffer
  const int64_t kChunk = 1024;
  int64_t maxb = kChunk;
  for (const TcTile& tl : tiles) maxb = std::max<int64_t>(maxb, tl.g1 - tl.g0);
  uint16_t* stage = nullptr;
  CK(cudaMallocHost((void**)&stage, (size_t)maxb * TC_BLOCK * 2));
  unsigned nthr = std::thread::hardware_concurrency();
  nthr = nthr < 1 ? 1 : (nthr > 32 ? 32 : nthr);
  int out = DMD_OK;
  const int n2 = h->nb2;
  for (int t0 = 0; t0 < h->ntiles && out == DMD_OK;) {
    int t1 = t0;
    int64_t nb_chunk = 0;
    while (t1 < h->ntiles && (t1 == t0 || nb_chunk + (tiles[t1].g1 - tiles[t1].g0) <= maxb)) {
      nb_chunk += tiles[t1].g1 - tiles[t1].g0;
      ++t1;
    }
    const int64_t b0 = tiles[t0].boff;
    std::atomic<int> next(t0);
    auto work = [&]() {
      std::vector<double> f64;
      cd P1[256], P2[256], Q1[256], Q2[256], A[256], Bm[256];
      for (int t; (t = next.fetch_add(1)) < t1;) {
        const TcTile& tl = tiles[t];
        const int nblk = tl.g1 - tl.g0;
        if (nblk == 0) continue;
        f64.assign((size_t)nblk * 2 * TC_N * TC_K, 0.0);  // [block][X|Y][n][kk]
        for (size_t e = start[t]; e < start[t + 1]; ++e) {
          const size_t src = ent[e] >> 1;
          const int dir = (int)(ent[e] & 1);
          pair_operators(h, d, src, P1, P2);
          herm_transform(nb, P1, P2, Q1, Q2);
          for (int i = 0; i < n2 * n2; ++i) {
            A[i] = dir ? cd{Q2[i].re, -Q2[i].im} : Q1[i];
            Bm[i] = dir ? cd{Q1[i].re, -Q1[i].im} : Q2[i];
          }
          const int rp = row_of(src, dir), cp = col_of(src, dir);
          const int r = rp - t * TR, blk = cp / CG - tl.g0, c = cp % CG;
          double* fx = &f64[(size_t)blk * 2 * TC_N * TC_K];
          double* fy = fx + TC_N * TC_K;
          for (int a = 0; a < n2; ++a)
            for (int j = 0; j < n2; ++j) {
              // X'_row[a] += A[a][j] r_col[j]: n = (r, a, re|im), kk = (c, j)
              const cd x = A[a * n2 + j];
              fx[((r * n2 + a) * 2) * TC_K + c * n2 + j] += x.re;
              fx[((r * n2 + a) * 2 + 1) * TC_K + c * n2 + j] += x.im;
              // Y'_row[j] += B[a][j] s_col[a]: n = (r, j, re|im), kk = (c, a)
              const cd y = Bm[a * n2 + j];
              fy[((r * n2 + j) * 2) * TC_K + c * n2 + a] += y.re;
              fy[((r * n2 + j) * 2 + 1) * TC_K + c * n2 + a] += y.im;
            }
          if (dev) {  // what the contraction adds for diag(f_ref) of the column (see k_prep_herm)
            const uint64_t kc = dir ? d->k1st[src] : d->k2nd[src];
            cd* ar = &acc0[(size_t)rp * 2 * n2];
            for (int a = 0; a < n2; ++a)
              for (int i = 0; i < nb; ++i) {
                const int ii = i * nb + i;
                const double fc = fw[kc * nb + i];
                ar[a].re += A[a * n2 + ii].re * fc;
                ar[a].im += A[a * n2 + ii].im * fc;
                ar[n2 + a].re += Bm[ii * n2 + a].re * (1 - fc);
                ar[n2 + a].im += Bm[ii * n2 + a].im * (1 - fc);
              }
          }
        }
        uint16_t* dst0 = stage + (size_t)(tl.boff - b0) * TC_BLOCK;
        for (int blk = 0; blk < nblk; ++blk)
          for (int m = 0; m < 2; ++m)
            for (int n = 0; n < TC_N; ++n)
              for (int kk = 0; kk < TC_K; ++kk) {
                const uint32_t w = pack_bf2(f64[(((size_t)blk * 2 + m) * TC_N + n) * TC_K + kk]);
                uint16_t* pl = dst0 + (size_t)blk * TC_BLOCK + (size_t)m * TC_PLANE;
                pl[tc_ci(n, kk)] = (uint16_t)(w >> 16);
                pl[tc_ci(n, kk + 32)] = (uint16_t)(w & 0xffffu);
              }
      }
    };
    std::vector<std::thread> pool;
    for (unsigned i = 1; i < nthr; ++i) pool.emplace_back(work);
    work();
    for (auto& th : pool) th.join();
    cudaError_t e = cudaMemcpy(h->d_tcB + (size_t)b0 * TC_BLOCK, stage, (size_t)nb_chunk * TC_BLOCK * 2,
                               cudaMemcpyHostToDevice);
    if (e != cudaSuccess) out = fail(h, DMD_E_CUDA, std::string("operator upload: ") + cudaGetErrorString(e));
    t0 = t1;
  }
  cudaFreeHost(stage);
  if (out == DMD_OK && (dev || h->lin)) {
    if ((out = dalloc(h, &h->d_fref, fw.size()))) return out;
    CK(cudaMemcpy(h->d_fref, fw.data(), fw.size() * 8, cudaMemcpyHostToDevice));
  }
  if (out == DMD_OK && dev) {
    // the split finish (k_finish<nb, ., true>): X0, Y0 back-transformed by k and the constant
    // V0 = (prefac/2)(C0 + C0^dagger), C0 = (1 - F) X0 - Y0 F (Hermitian reads of diagonal F)
    const int n2 = h->nb2;
    std::vector<float2> x0y0((size_t)nk * 2 * n2);
    std::vector<float2> v0((size_t)nk * n2);
    const double pf = 0.5 * h->prefac;
    for (int k = 0; k < nk; ++k) {
      const cd* a = &acc0[(size_t)L.pos[k] * 2 * n2];
      cd X[16], Y[16];  // nb^2 <= 16
      for (int e = 0; e < n2; ++e) {
        X[e] = a[e];
        Y[e] = a[n2 + e];
      }
      for (int i = 0; i < nb; ++i)
        for (int j = i + 1; j < nb; ++j) {  // X = (M^H)^-1 X' (dmd_kernels.cuh, k_finish)
          const cd xu = X[i * nb + j], xl = X[j * nb + i], yu = Y[i * nb + j], yl = Y[j * nb + i];
          X[i * nb + j] = {0.5 * (xu.re - xl.im), 0.5 * (xu.im + xl.re)};
          X[j * nb + i] = {0.5 * (xu.re + xl.im), 0.5 * (xu.im - xl.re)};
          Y[i * nb + j] = {0.5 * (yu.re - yl.im), 0.5 * (yu.im + yl.re)};
          Y[j * nb + i] = {0.5 * (yu.re + yl.im), 0.5 * (yu.im - yl.re)};
        }
      const double* f = &fw[(size_t)k * nb];
      cd C[16];
      for (int i = 0; i < nb; ++i)
        for (int j = 0; j < nb; ++j)
          C[i * nb + j] = {(1 - f[i]) * X[i * nb + j].re - Y[i * nb + j].re * f[j],
                           (1 - f[i]) * X[i * nb + j].im - Y[i * nb + j].im * f[j]};
      for (int i = 0; i < nb; ++i)
        for (int j = 0; j < nb; ++j) {
          const cd c1 = C[i * nb + j], c2 = C[j * nb + i];
          v0[(size_t)k * n2 + i * nb + j] = make_float2((float)(pf * (c1.re + c2.re)), (float)(pf * (c1.im - c2.im)));
          x0y0[(size_t)k * 2 * n2 + i * nb + j] = make_float2((float)X[i * nb + j].re, (float)X[i * nb + j].im);
          x0y0[(size_t)k * 2 * n2 + n2 + i * nb + j] = make_float2((float)Y[i * nb + j].re, (float)Y[i * nb + j].im);
        }
    }
    if ((out = dalloc(h, &h->d_x0y0, x0y0.size())) || (out = dalloc(h, &h->d_v0, v0.size()))) return out;
    CK(cudaMemcpy(h->d_x0y0, x0y0.data(), x0y0.size() * 8, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(h->d_v0, v0.data(), v0.size() * 8, cudaMemcpyHostToDevice));
  }
  return out;
}

// the captured RK4 steps hold kernel arguments: capture again at the next use
void drop_graphs(dmd_handle* h) {
  if (h->g_rk4) cudaGraphExecDestroy(h->g_rk4);
  if (h->g_rk4_rec) cudaGraphExecDestroy(h->g_rk4_rec);
  h->g_rk4 = h->g_rk4_rec = nullptr;
}

void release(dmd_handle* h) {
  if (!h) return;
  cudaSetDevice(h->dev);
  if (h->g_rk4) cudaGraphExecDestroy(h->g_rk4);
  if (h->g_rk4_rec) cudaGraphExecDestroy(h->g_rk4_rec);
  void* ptrs[] = {h->d_err, h->d_pos, h->d_rb, h->d_items, h->d_ew, h->d_edm, h->d_kk, h->d_P, h->d_H, h->d_eq, h->d_rs, h->d_acc, h->d_y, h->d_ytmp,
                  h->d_y0, h->d_in, h->d_in1, h->d_out, h->d_K, h->d_tref, h->d_step, h->d_red, h->d_coef_i,
                  h->d_coef, h->d_flag, h->d_hflag, h->d_acc0, h->d_fref, h->d_tcB, h->d_tcA, h->d_tiles, h->d_ph, h->d_inv, h->d_x0y0, h->d_v0, h->d_Praw, h->d_kkraw,
                  h->d_dst, h->d_ee_kvec, h->d_ee_kidx, h->d_ee_kmap, h->d_ee_U, h->d_ee_ewf, h->d_ee_f,
                  h->d_ee_dm, h->d_ee_dm1, h->d_ee_dmf, h->d_ee_dm1f, h->d_ee_scr, h->d_ee_Pee, h->d_ee_vqtab,
                  h->d_sp_base, h->d_sp_len, h->d_sp_val, h->d_sp_gidx, h->d_Padf, h->d_ee_Aq, h->d_ee_Eq2, h->d_rec};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  for (int i = 0; i < 8; ++i) {
    if (h->d_obs[i]) cudaFree(h->d_obs[i]);
    if (h->d_f[i]) cudaFree(h->d_f[i]);
  }
  for (auto& r : h->prof_pending) {
    cudaEventDestroy(r.a);
    cudaEventDestroy(r.b);
  }
  for (auto e : h->ev_pool) cudaEventDestroy(e);
  for (auto e : h->tev)
    if (e) cudaEventDestroy(e);
  if (h->st) cudaStreamDestroy(h->st);
}

// ---------------------------------------------------------------------------------------------
// e-e model: P = P_base + scale P_ee(rho) (dmd_ee.cuh), refilled into the column-block store
// ---------------------------------------------------------------------------------------------
template <int NB>
int ee_rebuild(dmd_handle* h, const double2* y, const TimeArg& ta, bool eq) {
  constexpr int NB2 = NB * NB, NB4 = NB2 * NB2;
  ProfScope ps(h, 4);
  EeArgs a = h->ee_args;
  if (!eq) {  // the window density matrix of y in the Schrodinger picture
    k_ee_dm<NB><<<blocks_for((long long)h->nk * NB2, 256), 256, 0, h->st>>>(
        h->nk, h->nbdm, h->bs, y, h->d_ew, ta, h->picture == DMD_PICTURE_INTERACTION ? 1 : 0, h->d_ee_dm, h->d_ee_dm1,
        h->d_ee_dmf, h->d_ee_dm1f);
    a.dm = h->d_ee_dm;
    a.dm1 = h->d_ee_dm1;
    a.dmf = h->d_ee_dmf;
    a.dm1f = h->d_ee_dm1f;
    a.f = nullptr;
  } else {  // the set-up: occupations instead of rho (calc_A1f, calc_A1fbar)
    a.dm = a.dm1 = nullptr;
    a.dmf = a.dm1f = nullptr;
    a.f = h->d_ee_f;
  }
  k_ee_screen<<<1, 256, 0, h->st>>>(h->nk, NB, h->ee_nv, h->d_ee_dm, (!eq && h->ee_update) ? 1 : 0, h->ee_nfree0,
                                    h->ee_nkfull, h->ee_cell, h->ee_eps, h->ee_T, h->ee_meff, h->d_ee_scr);
  // FP64 handles contract in FP64, the others in double-float on the FP32 pipes
  constexpr int WPC = ee_warps_per_cta(NB);
  const unsigned grid = (unsigned)((h->npair + WPC - 1) / WPC);
  if (h->prec == DMD_PREC_F64) {
    if (a.dynamic) k_ee_pairs<NB, EeF64, true><<<grid, 32 * WPC, 0, h->st>>>(a);
    else k_ee_pairs<NB, EeF64><<<grid, 32 * WPC, 0, h->st>>>(a);
  } else {
    if (a.dynamic) k_ee_pairs<NB, EeDF, true><<<grid, 32 * WPC, 0, h->st>>>(a);
    else k_ee_pairs<NB, EeDF><<<grid, 32 * WPC, 0, h->st>>>(a);
  }
  const bool dev = deviation_form(h->prec) && !h->lin;
  if (dev && cudaMemsetAsync(h->d_acc0, 0, (size_t)h->nk * 2 * NB2 * sizeof(double2), h->st) != cudaSuccess)
    return fail(h, DMD_E_CUDA, "e-e refill");
  const FillSrc fs = {h->d_Praw, (size_t)NB4, (size_t)2 * NB4, h->d_ee_Pee, (size_t)NB4, (size_t)2 * NB4};
  k_cb_fill<NB><<<blocks_for(h->npair, 128), 128, 0, h->st>>>(0, h->npair, fs, h->ee_scale, (const CbDst*)h->d_dst,
                                                              h->lin, h->prec, elem_bytes(h->prec),
                                                              (unsigned char*)h->d_P, h->d_fref,
                                                              dev ? (double*)h->d_acc0 : nullptr);
  h->launches += eq ? 3 : 4;
  CKL();
  return DMD_OK;
}

int ee_rebuild_nb(dmd_handle* h, const double2* y, const TimeArg& ta, bool eq) {
  return h->nb == 2 ? ee_rebuild<2>(h, y, ta, eq) : ee_rebuild<4>(h, y, ta, eq);
}

// ---------------------------------------------------------------------------------------------
// adjoint (dmd_adjoint_rk4): work buffers, forward RK4 with stored stage inputs, one VJP
// ---------------------------------------------------------------------------------------------
// page-locked host buffer (freed on scope exit)
struct PinnedStage {
  void* p = nullptr;
  bool alloc(size_t bytes) { return cudaHostAlloc(&p, bytes, cudaHostAllocDefault) == cudaSuccess; }
  ~PinnedStage() {
    if (p) cudaFreeHost(p);
  }
};

// memcpy split over host threads (first-touch page faults of a fresh destination run in parallel)
void parallel_copy(void* dst, const void* src, size_t bytes) {
  const unsigned nt = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
  if (bytes < (8u << 20) || nt == 1) {
    memcpy(dst, src, bytes);
    return;
  }
  std::vector<std::thread> th;
  const size_t part = (bytes / nt + 4095) / 4096 * 4096;
  for (unsigned i = 0; i < nt; ++i) {
    const size_t b0 = (size_t)i * part;
    if (b0 >= bytes) break;
    const size_t nb = std::min(part, bytes - b0);
    th.emplace_back([=] { memcpy((char*)dst + b0, (const char*)src + b0, nb); });
  }
  for (auto& t : th) t.join();
}

struct AdjWork {
  dmd_handle* h = nullptr;
  std::vector<void*> owned;
  double2 *ck = nullptr, *U = nullptr, *yb = nullptr, *ub = nullptr, *kb = nullptr, *tmp = nullptr;
  double2 *Xb = nullptr, *Yb = nullptr, *rt = nullptr, *st = nullptr, *rtb = nullptr, *stb = nullptr, *G = nullptr;
  float4* dfv = nullptr;  // double-float form: (x, S(x)) of Xbar, Ybar, rt, st
  double2* A = nullptr;    // forward sums (d_acc) at every stage input of the stretch being reversed
  ~AdjWork() {
    for (void* p : owned) cudaFree(p);
  }
  template <typename T>
  int get(T** p, size_t n) {
    int rc = dalloc(h, p, n);
    if (rc == DMD_OK) owned.push_back((void*)*p);
    return rc;
  }
};

// y_out = one RK4 step of y; the stage inputs u1..u4 go to U[0..3] (stride n) when U is set, and the
// forward sums of the four evaluations (d_acc) to A[0..3] (stride nk 2 nb^2) when A is set
int adj_rk4_step(dmd_handle* h, const double2* y, double t, double dt, double2* U, double2* y_out, double2* tmp,
                 double2* A = nullptr) {
  const size_t n = h->nstate, na = (size_t)h->nk * 2 * h->nb2;
  const unsigned g = blocks_for((long long)n, 256);
  double2* K = h->d_K;
  int rc;
  auto keep = [&](int q) -> int {
    if (A) CK(cudaMemcpyAsync(A + (size_t)q * na, h->d_acc, na * 16, cudaMemcpyDeviceToDevice, h->st));
    return DMD_OK;
  };
  if (U) CK(cudaMemcpyAsync(U, y, n * 16, cudaMemcpyDeviceToDevice, h->st));
  if ((rc = rhs_plain(h, t, y, K)) || (rc = keep(0))) return rc;
  double2* u = U ? U + n : tmp;
  k_axpy<<<g, 256, 0, h->st>>>(n, u, y, 0.5 * dt, K);
  if ((rc = rhs_plain(h, t + 0.5 * dt, u, K + n)) || (rc = keep(1))) return rc;
  u = U ? U + 2 * n : tmp;
  k_axpy<<<g, 256, 0, h->st>>>(n, u, y, 0.5 * dt, K + n);
  if ((rc = rhs_plain(h, t + 0.5 * dt, u, K + 2 * n)) || (rc = keep(2))) return rc;
  u = U ? U + 3 * n : tmp;
  k_axpy<<<g, 256, 0, h->st>>>(n, u, y, dt, K + 2 * n);
  if ((rc = rhs_plain(h, t + dt, u, K + 3 * n)) || (rc = keep(3))) return rc;
  k_rk4_final<<<g, 256, 0, h->st>>>(n, y_out, y, K, n, dt);
  h->launches += 5;
  CKL();
  return DMD_OK;
}

// the nb = 4 double-float adjoint pair pass (k_adj_pairs_bulk4): a persistent grid of two CTAs per
// SM; shape from DMD_ADJ_BULK_SHAPE (0: 1 stage x 5 warps, the default; 1: 1 stage x 4 warps;
// 2: 2 stages x 2 warps)
template <int NST, int W>
int adj_bulk4_launch_shape(dmd_handle* h, const int2* kk, const float4* dfv, size_t nk2, double* rtb, double* stb,
                           float4* G) {
  typedef AdjBulkSmem<NST, W> S;
  // set on every launch: the attribute belongs to the current device's context, and handles may
  // live on different devices
  CK(cudaFuncSetAttribute(k_adj_pairs_bulk4<NST, W>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)S::cta_bytes));
  int nsm = 0;
  if (cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, h->dev) != cudaSuccess || nsm <= 0) nsm = 1;
  const long long ctas = std::min<long long>((long long)nsm * 2, (h->npair + S::warps - 1) / S::warps);
  k_adj_pairs_bulk4<NST, W><<<(unsigned)ctas, 32 * S::warps, S::cta_bytes, h->st>>>(h->npair, kk, h->d_Padf, dfv,
                                                                                     nk2, rtb, stb, G, h->d_err);
  return DMD_OK;
}

int adj_bulk4_launch(dmd_handle* h, const int2* kk, const float4* dfv, size_t nk2, double* rtb, double* stb, float4* G) {
  static int shape = -1;
  if (shape < 0) {
    const char* e = getenv("DMD_ADJ_BULK_SHAPE");
    shape = e ? atoi(e) : 0;
  }
  if (shape == 1) return adj_bulk4_launch_shape<1, 4>(h, kk, dfv, nk2, rtb, stb, G);
  if (shape == 2) return adj_bulk4_launch_shape<2, 2>(h, kk, dfv, nk2, rtb, stb, G);
  return adj_bulk4_launch_shape<1, 5>(h, kk, dfv, nk2, rtb, stb, G);
}

// ybar += VJP_f(u, t)(vbar); kprev += c * VJP_f(u, t)(vbar) when kprev is set. accs: the forward sums
// at u kept when u was evaluated (the phases are then recomputed from t), or null to evaluate them
template <int NB>
int adj_vjp_nb(dmd_handle* h, AdjWork& w, const double2* u, double t, const double2* vbar, double2* kprev, double c,
               const double2* accs) {
  int rc;
  if (!accs) {
    const TimeArg ta = time_value(t);
    if ((rc = launch_prep<NB>(h, u, ta)) || (rc = launch_pairs<NB>(h))) return rc;  // forward sums at u
    CK(cudaMemsetAsync(h->d_hflag, 0, sizeof(unsigned int), h->st));
  }
  const size_t nk2 = (size_t)h->nk * NB * NB;
  const double2* ph = (h->expt && !accs) ? h->d_ph : nullptr;
  AdjLocalArgs a;
  a.nk = h->nk;
  a.nbdm = h->nbdm;
  a.bs = h->bs;
  a.picture = h->picture;
  a.phase = h->expt;
  a.herm = h->use_cb;
  a.lin = h->lin;
  a.want_coh = (h->picture == DMD_PICTURE_SCHRODINGER || h->d_H) ? 1 : 0;
  a.prefac = h->prefac;
  a.t = t;
  a.u = u;
  a.vbar = vbar;
  a.acc = accs ? accs : h->d_acc;
  a.pos = h->use_cb ? h->d_pos : nullptr;
  a.ph = ph;
  a.ew = h->d_ew;
  a.edm = h->d_edm;
  a.H = h->d_H;
  a.Xb = w.Xb;
  a.Yb = w.Yb;
  a.rt = w.rt;
  a.st = w.st;
  a.ubar = w.ub;
  a.rtb = w.rtb;  // zeroed by k_adj_local before the pair pass adds into them
  a.stb = w.stb;
  a.dfv = w.dfv;
  a.nk2 = nk2;
  k_adj_local<NB><<<blocks_for(h->nk, 128), 128, 0, h->st>>>(a);
  if (h->npair > 0) {
    const int2* kk = h->use_cb ? h->d_kkraw : h->d_kk;
    if (w.dfv && NB == 4) {  // double-float, one warp per pair, operators and gradient staged by bulk copies
      if ((rc = adj_bulk4_launch(h, kk, w.dfv, nk2, (double*)w.rtb, (double*)w.stb, (float4*)w.G))) return rc;
    } else if (w.dfv) {  // double-float products on the FP32 pipes
      k_adj_pairs_df<NB><<<blocks_for(h->npair * NB * NB, 128), 128, 0, h->st>>>(
          h->npair, kk, h->d_Padf, w.dfv, nk2, (double*)w.rtb, (double*)w.stb, (float4*)w.G);
    } else {
      const double2* P = h->use_cb ? h->d_Praw : h->d_P;
      k_adj_pairs<NB><<<blocks_for(h->npair * NB * NB, 128), 128, 0, h->st>>>(h->npair, kk, P, w.Xb, w.Yb, w.rt, w.st,
                                                                             (double*)w.rtb, (double*)w.stb, w.G);
    }
  }
  k_adj_combine<NB><<<blocks_for((long long)h->nstate, 256), 256, 0, h->st>>>(
      h->nk, h->nbdm, h->bs, h->expt, t, h->d_ew, ph, w.rtb, w.stb, w.ub, w.yb, kprev, c);
  h->launches += 3;
  CKL();
  return DMD_OK;
}

int adj_vjp(dmd_handle* h, AdjWork& w, const double2* u, double t, const double2* vbar, double2* kprev, double c,
            const double2* accs) {
  switch (h->nb) {
    case 1: return adj_vjp_nb<1>(h, w, u, t, vbar, kprev, c, accs);
    case 2: return adj_vjp_nb<2>(h, w, u, t, vbar, kprev, c, accs);
    case 3: return adj_vjp_nb<3>(h, w, u, t, vbar, kprev, c, accs);
    case 4: return adj_vjp_nb<4>(h, w, u, t, vbar, kprev, c, accs);
  }
  return fail(h, DMD_E_ARG, "nb out of range");
}

// total of observable `slot` on the device state y at time t (dmd_measure's reduction)
int measure_on(dmd_handle* h, int slot, int bstart, int bend, const double2* y, double t, double* tot) {
  const unsigned nbk = blocks_for(h->nk, 256);
  if (2 * nbk > red_elems(h)) return fail(h, DMD_E_ARG, "nk too large for the observable reduction");
  k_measure<<<nbk, 256, 0, h->st>>>(h->nk, h->nbdm, bstart, bend, h->d_obs[slot], h->d_f[slot], h->d_edm, t,
                                    h->picture, y, h->d_red);
  h->launches++;
  CKL();
  std::vector<double> part(2 * nbk);
  CK(cudaMemcpyAsync(part.data(), h->d_red, 2 * nbk * 8, cudaMemcpyDeviceToHost, h->st));
  CK(cudaStreamSynchronize(h->st));
  double s1 = 0;
  for (unsigned b = 0; b < nbk; ++b) s1 += part[2 * b];
  *tot = s1 * h->obs_prefac[slot];
  return DMD_OK;
}

int check_state(dmd_handle* h) {
  unsigned int derr = 0;
  CK(cudaMemcpyAsync(&derr, h->d_err, sizeof(derr), cudaMemcpyDeviceToHost, h->st));
  CK(cudaStreamSynchronize(h->st));
  if (derr) {
    cudaMemsetAsync(h->d_err, 0, sizeof(derr), h->st);
    return fail(h, DMD_E_TIMEOUT, "a bounded device wait gave up (bulk copy did not complete)");
  }
  const size_t n = 2 * h->nstate;
  CK(cudaMemsetAsync(h->d_flag, 0, sizeof(int), h->st));
  k_nan_scan<<<blocks_for((long long)n, 256), 256, 0, h->st>>>(n, (const double*)h->d_y, h->d_flag);
  h->launches++;
  CKL();
  int flag = 0;
  CK(cudaMemcpyAsync(&flag, h->d_flag, sizeof(int), cudaMemcpyDeviceToHost, h->st));
  CK(cudaStreamSynchronize(h->st));
  if (flag) return fail(h, DMD_E_NAN, "non-finite value in the density matrix");
  return DMD_OK;
}

}  // namespace

extern "C" {

const char* dmd_strerror(int s) {
  if (s < 0 || s > 9) return "unknown status";
  return kStatus[s];
}

const char* dmd_last_error(const dmd_handle* h) { return h ? h->err.c_str() : "null handle"; }

static int create_impl(const dmd_desc* d, dmd_handle** out, PairSource* src) {
  if (!out) return DMD_E_ARG;
  *out = nullptr;
  if (!d) return DMD_E_ARG;
  if (d->nk <= 0 || d->nb_dm <= 0 || d->nb_dm > DMD_MAX_NBDM || d->bstart < 0 || d->bend > d->nb_dm ||
      d->bend - d->bstart < 1 || d->bend - d->bstart > 4 || d->nkpair < 0 || !d->e_dm)
    return DMD_E_ARG;
  if (d->nkpair > 0 && (!d->k1st || !d->k2nd || (!src && (!d->P1 || !d->P2)))) return DMD_E_ARG;
  if (!src && (d->P1_add == nullptr) != (d->P2_add == nullptr)) return DMD_E_ARG;
  if (d->flags & ~(DMD_FLAG_LINEAR | DMD_FLAG_ADJOINT | DMD_FLAG_EE | DMD_FLAG_SPARSE)) return DMD_E_ARG;
  if ((d->flags & DMD_FLAG_SPARSE) && (d->precision != DMD_PREC_F64 || d->nrhs > 1 ||
                                       (d->flags & (DMD_FLAG_LINEAR | DMD_FLAG_ADJOINT | DMD_FLAG_EE))))
    return DMD_E_ARG;
  if ((d->flags & DMD_FLAG_ADJOINT) && d->nrhs > 1) return DMD_E_ARG;
  const int nrhs = d->nrhs > 1 ? d->nrhs : 1;
  // batched form: FP32 or bf16 hi+lo storage on the column-block contraction
  if (nrhs > 1 && (d->precision != DMD_PREC_F32 && d->precision != DMD_PREC_BF16X2)) return DMD_E_ARG;
  if ((d->flags & DMD_FLAG_LINEAR) &&
      (!d->f_ref || d->P1_add || (d->bend - d->bstart != 2 && d->bend - d->bstart != 4) || d->nkpair == 0))
    return DMD_E_ARG;
  if (d->precision < DMD_PREC_F64 || d->precision > DMD_PREC_BF16X2) return DMD_E_ARG;
  // the FP32-pair and reduced-precision forms exist for the column-block contraction (nb = 2, 4)
  const int nbw = d->bend - d->bstart;
  if (d->precision != DMD_PREC_F64 && ((nbw != 2 && nbw != 4) || d->nkpair == 0)) return DMD_E_ARG;
  if (d->picture != DMD_PICTURE_INTERACTION && d->picture != DMD_PICTURE_SCHRODINGER) return DMD_E_ARG;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return DMD_E_NODEV;
  if (d->device < 0 || d->device >= ndev) return DMD_E_ARG;
  dmd_handle* h = new dmd_handle();
  h->dev = d->device;
  h->nk = d->nk;
  h->nbdm = d->nb_dm;
  h->bs = d->bstart;
  h->be = d->bend;
  h->nb = d->bend - d->bstart;
  h->nb2 = h->nb * h->nb;
  h->nb4 = h->nb2 * h->nb2;
  h->npair = d->nkpair;
  h->prefac = d->prefac_eph;
  h->add_scale = d->add_scale;
  h->picture = d->picture;
  h->expt = d->expt ? 1 : 0;
  h->prec = d->precision;
  h->lin = (d->flags & DMD_FLAG_LINEAR) ? 1 : 0;
  h->adj = (d->flags & DMD_FLAG_ADJOINT) ? 1 : 0;
  h->eek = (d->flags & DMD_FLAG_EE) ? 1 : 0;
  h->use_sp = (d->flags & DMD_FLAG_SPARSE) ? 1 : 0;
  h->nrhs = nrhs;
  h->nstate1 = (size_t)h->nk * h->nbdm * h->nbdm;
  h->nstate = h->nstate1 * nrhs;
  if (const char* v = getenv("DMD_BATCH_RW")) h->brw = atoi(v) == 8 ? 8 : 4;
  // batched bf16 hi + lo form with nb = 2: the tensor-core contraction (DMD_BATCH_TC=0 keeps the
  // CUDA-core column-block form)
  {
    const char* v = getenv("DMD_BATCH_TC");
    h->use_tc = (nrhs > 1 && (h->nb == 2 || h->nb == 4) && h->npair > 0 && h->prec == DMD_PREC_BF16X2 && !(v && atoi(v) == 0)) ? 1 : 0;
  }
  int rc = DMD_OK;
  auto bail = [&](int code) {
    std::string m = h->err;
    release(h);
    delete h;
    fprintf(stderr, "dmd_create: %s\n", m.c_str());
    return code;
  };
  if (cudaSetDevice(h->dev) != cudaSuccess) return bail(DMD_E_CUDA);
  if (cudaStreamCreateWithFlags(&h->st, cudaStreamNonBlocking) != cudaSuccess) return bail(DMD_E_CUDA);
  const size_t nk = h->nk, nbdm = h->nbdm;
  if ((rc = dalloc(h, &h->d_ew, nk * h->nb)) || (rc = dalloc(h, &h->d_edm, nk * nbdm)) ||
      (rc = dalloc(h, &h->d_kk, (h->nb == 2 || h->nb == 4 || h->use_sp) ? 1 : (size_t)h->npair)) ||
      (rc = dalloc(h, &h->d_P, (h->use_tc || h->use_sp) ? 1 : ((size_t)h->npair * 2 * h->nb4 * elem_bytes(h->prec) + 15) / 16)) ||
      (rc = dalloc(h, &h->d_rs, nk * 2 * h->nb2 * nrhs)) || (rc = dalloc(h, &h->d_acc, nk * 2 * h->nb2 * nrhs)) ||
      (rc = dalloc(h, &h->d_y, h->nstate)) || (rc = dalloc(h, &h->d_ytmp, h->nstate)) ||
      (rc = dalloc(h, &h->d_y0, h->nstate)) || (rc = dalloc(h, &h->d_in, h->nstate)) ||
      (rc = dalloc(h, &h->d_in1, h->nstate)) || (rc = dalloc(h, &h->d_out, h->nstate)) ||
      (rc = dalloc(h, &h->d_K, 6 * h->nstate)) || (rc = dalloc(h, &h->d_tref, 2)) ||
      (rc = dalloc(h, &h->d_step, 1)) || (rc = dalloc(h, &h->d_red, red_elems(h))) || (rc = dalloc(h, &h->d_coef_i, 64)) ||
      (rc = dalloc(h, &h->d_coef, 64)) || (rc = dalloc(h, &h->d_flag, 1)) || (rc = dalloc(h, &h->d_err, 1)) ||
      (rc = dalloc(h, &h->d_hflag, 1)) || (rc = dalloc(h, &h->d_ph, nk * h->nb2)))
    return bail(rc);
  std::vector<double> ew(nk * h->nb);
  for (size_t k = 0; k < nk; ++k)
    for (int b = 0; b < h->nb; ++b) ew[k * h->nb + b] = d->e_dm[k * nbdm + h->bs + b];
  if (cudaMemcpy(h->d_ew, ew.data(), ew.size() * 8, cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(h->d_edm, d->e_dm, nk * nbdm * 8, cudaMemcpyHostToDevice) != cudaSuccess)
    return bail(fail(h, DMD_E_CUDA, "upload energies"));
  if (d->Hcoh) {
    if ((rc = dalloc(h, &h->d_H, h->nstate1))) return bail(rc);
    if (cudaMemcpy(h->d_H, d->Hcoh, h->nstate1 * 16, cudaMemcpyHostToDevice) != cudaSuccess)
      return bail(fail(h, DMD_E_CUDA, "upload H"));
  }
  h->use_cb = ((h->nb == 2 || h->nb == 4) && h->npair > 0 && !h->use_sp) ? 1 : 0;
  if (!h->use_tc)
    h->pair_bytes = h->use_cb ? (int64_t)h->npair * 2 * h->nb4 * elem_bytes(h->prec) : (int64_t)h->npair * 2 * h->nb4 * 16;
  if (src && !h->use_sp && (!h->use_cb || h->use_tc || h->adj))
    return bail(fail(h, DMD_E_ARG, "streamed operators need the column-block or the sparse form"));
  if (h->eek && (!h->use_cb || h->use_tc || h->nrhs != 1 || h->lin || src || h->adj))
    return bail(fail(h, DMD_E_ARG, "DMD_FLAG_EE needs nb = 2 or 4, a single state, no linearization, no adjoint "
                                   "(P_ee depends on rho) and the operators as arrays"));
  h->src = src;
  rc = h->use_tc ? upload_pairs_tc(h, d) : h->use_sp ? upload_pairs_sparse(h, d) : h->use_cb ? upload_pairs_cb(h, d)
                                                                                  : upload_pairs(h, d);
  h->src = nullptr;
  if (rc) return bail(rc);
  if ((h->adj || h->eek) && h->use_cb && h->npair > 0) {  // stored-order P: the adjoint, the e-e refill
    if ((rc = dalloc(h, &h->d_Praw, (size_t)h->npair * 2 * h->nb4)) || (rc = dalloc(h, &h->d_kkraw, (size_t)h->npair)) ||
        (rc = upload_raw(h, d, h->d_Praw, h->d_kkraw)))
      return bail(rc);
  }
  if (cudaMemset(h->d_y, 0, h->nstate * 16) != cudaSuccess || cudaMemset(h->d_step, 0, 8) != cudaSuccess ||
      cudaMemset(h->d_err, 0, sizeof(unsigned int)) != cudaSuccess ||
      cudaMemset(h->d_hflag, 0, sizeof(unsigned int)) != cudaSuccess)
    return bail(fail(h, DMD_E_CUDA, "init"));
  *out = h;
  return DMD_OK;
}

int dmd_create(const dmd_desc* d, dmd_handle** out) { return create_impl(d, out, nullptr); }

}  // extern "C"

namespace {
// DMD's operator files (complex128 [nkpair][nb^4], ldbd_P1_lindblad.bin etc.), read chunk by chunk
struct FileSource : PairSource {
  FILE* f[4] = {nullptr, nullptr, nullptr, nullptr};
  size_t nb4 = 0;
  bool add = false;
  ~FileSource() override {
    for (FILE* x : f)
      if (x) fclose(x);
  }
  bool has_add() const override { return add; }
  int open(int m, const char* path, long long npair) {
    f[m] = fopen(path, "rb");
    if (!f[m]) {
      err = std::string("cannot open ") + path;
      return DMD_E_FILE;
    }
    if (fseeko(f[m], 0, SEEK_END) != 0 || ftello(f[m]) != (off_t)(npair * (long long)nb4 * 16)) {
      err = std::string("size of ") + path + " does not match nkpair * nb^4 complex128";
      return DMD_E_FILE;
    }
    fseeko(f[m], 0, SEEK_SET);
    return DMD_OK;
  }
  int read(long long p0, long long cnt, double2* dst) override {
    const size_t n = (size_t)cnt * nb4;
    for (int m = 0; m < (add ? 4 : 2); ++m) {
      if (fseeko(f[m], (off_t)(p0 * (long long)nb4 * 16), SEEK_SET) != 0 || fread(dst + m * n, 16, n, f[m]) != n) {
        err = "short read of a pair-operator file";
        return DMD_E_FILE;
      }
    }
    return DMD_OK;
  }
};
// DMD's sparse operator files (alg.Pin_is_sparse: sparse2D / sparse_mat, comm/sparse2D.h:115-128,
// comm/sparse_matrix.h:30-36): per pair a count ns (int32, <prefix>_ns.bin), then ns values
// (complex128, _s.bin) with their row and column indices (int32, _i.bin, _j.bin), read in pair order
// and written densely into the chunk (optional dense additive files as in FileSource)
struct SparseFileSource : PairSource {
  FILE* f[2][4] = {{nullptr, nullptr, nullptr, nullptr}, {nullptr, nullptr, nullptr, nullptr}};
  FileSource add;  // the dense additive operators in its slots 0 and 1
  size_t nb4 = 0, nb2 = 0;
  long long next = 0;  // the next pair the streams are positioned at
  std::vector<double2> sv;
  std::vector<int32_t> si, sj;
  ~SparseFileSource() override {
    for (auto& g : f)
      for (FILE* x : g)
        if (x) fclose(x);
  }
  bool has_add() const override { return add.add; }
  int open(int m, const std::string& prefix, long long npair) {
    const char* sfx[4] = {"_ns.bin", "_s.bin", "_i.bin", "_j.bin"};
    for (int q = 0; q < 4; ++q) {
      const std::string path = prefix + sfx[q];
      f[m][q] = fopen(path.c_str(), "rb");
      if (!f[m][q]) {
        err = "cannot open " + path;
        return DMD_E_FILE;
      }
    }
    if (fseeko(f[m][0], 0, SEEK_END) != 0 || ftello(f[m][0]) != (off_t)(npair * 4)) {
      err = prefix + "_ns.bin does not hold one int32 count per k-pair";
      return DMD_E_FILE;
    }
    fseeko(f[m][0], 0, SEEK_SET);
    return DMD_OK;
  }
  int read(long long p0, long long cnt, double2* dst) override {
    if (p0 != next) {
      err = "sparse operator files are read in pair order";
      return DMD_E_FILE;
    }
    const size_t n = (size_t)cnt * nb4;
    std::vector<int32_t> ns((size_t)cnt);
    for (int m = 0; m < 2; ++m) {
      double2* out = dst + m * n;
      memset(out, 0, n * 16);
      if (fread(ns.data(), 4, (size_t)cnt, f[m][0]) != (size_t)cnt) {
        err = "short read of an _ns.bin file";
        return DMD_E_FILE;
      }
      long long tot = 0;
      for (int32_t c : ns) {
        if (c < 0 || (size_t)c > nb4) {
          err = "invalid element count in an _ns.bin file";
          return DMD_E_FILE;
        }
        tot += c;
      }
      sv.resize((size_t)tot);
      si.resize((size_t)tot);
      sj.resize((size_t)tot);
      if (fread(sv.data(), 16, (size_t)tot, f[m][1]) != (size_t)tot || fread(si.data(), 4, (size_t)tot, f[m][2]) != (size_t)tot ||
          fread(sj.data(), 4, (size_t)tot, f[m][3]) != (size_t)tot) {
        err = "short read of a sparse operator file";
        return DMD_E_FILE;
      }
      size_t q = 0;
      for (long long p = 0; p < cnt; ++p)
        for (int32_t c = 0; c < ns[(size_t)p]; ++c, ++q) {
          const int32_t a = si[q], b = sj[q];
          if (a < 0 || b < 0 || (size_t)a >= nb2 || (size_t)b >= nb2) {
            err = "element index out of range in a sparse operator file";
            return DMD_E_FILE;
          }
          double2& o = out[(size_t)p * nb4 + (size_t)a * nb2 + b];  // repeated (i, j) add up
          o.x += sv[q].x;
          o.y += sv[q].y;
        }
    }
    if (add.add) {  // dense additive operators: segments 2 and 3
      add.add = false;  // FileSource reads its two slots
      const int rc = add.read(p0, cnt, dst + 2 * n);
      add.add = true;
      if (rc != DMD_OK) {
        err = add.err;
        return DMD_E_FILE;
      }
    }
    next = p0 + cnt;
    return DMD_OK;
  }
};
}  // namespace

extern "C" {

int dmd_create_from_sparse_files(const dmd_desc* d, const char* sp1_prefix, const char* sp2_prefix,
                                 const char* p1_add_path, const char* p2_add_path, dmd_handle** out) {
  if (!d || !out || !sp1_prefix || !sp2_prefix || (p1_add_path == nullptr) != (p2_add_path == nullptr))
    return DMD_E_ARG;
  if (d->bend - d->bstart < 1 || d->bend - d->bstart > 4 || d->nkpair < 0) return DMD_E_ARG;
  const int nb = d->bend - d->bstart;
  SparseFileSource ss;
  ss.nb2 = (size_t)nb * nb;
  ss.nb4 = ss.nb2 * ss.nb2;
  if (ss.open(0, sp1_prefix, d->nkpair) != DMD_OK || ss.open(1, sp2_prefix, d->nkpair) != DMD_OK) {
    fprintf(stderr, "dmd_create_from_sparse_files: %s\n", ss.err.c_str());
    return DMD_E_FILE;
  }
  if (p1_add_path) {
    ss.add.nb4 = ss.nb4;
    ss.add.add = true;
    if (ss.add.open(0, p1_add_path, d->nkpair) != DMD_OK || ss.add.open(1, p2_add_path, d->nkpair) != DMD_OK) {
      fprintf(stderr, "dmd_create_from_sparse_files: %s\n", ss.add.err.c_str());
      return DMD_E_FILE;
    }
  }
  dmd_desc dc = *d;
  dc.P1 = dc.P2 = dc.P1_add = dc.P2_add = nullptr;
  const char* tc = getenv("DMD_BATCH_TC");
  const bool tc_form = d->nrhs > 1 && nb == 2 && d->precision == DMD_PREC_BF16X2 && !(tc && atoi(tc) == 0);
  if (!(d->flags & DMD_FLAG_SPARSE) &&
      !((nb == 2 || nb == 4) && d->nkpair > 0 && !tc_form && !(d->flags & DMD_FLAG_ADJOINT)))
    return DMD_E_ARG;  // the other forms take dense operators (dmd_create, dmd_create_from_files)
  return create_impl(&dc, out, &ss);
}

int dmd_create_from_files(const dmd_desc* d, const char* p1_path, const char* p2_path, const char* p1_add_path,
                          const char* p2_add_path, dmd_handle** out) {
  if (!d || !out || !p1_path || !p2_path || (p1_add_path == nullptr) != (p2_add_path == nullptr)) return DMD_E_ARG;
  if (d->bend - d->bstart < 1 || d->bend - d->bstart > 4 || d->nkpair < 0) return DMD_E_ARG;
  const int nb = d->bend - d->bstart;
  FileSource fs;
  fs.nb4 = (size_t)nb * nb * nb * nb;
  fs.add = p1_add_path != nullptr;
  const char* paths[4] = {p1_path, p2_path, p1_add_path, p2_add_path};
  for (int m = 0; m < (fs.add ? 4 : 2); ++m)
    if (fs.open(m, paths[m], d->nkpair) != DMD_OK) {
      fprintf(stderr, "dmd_create_from_files: %s\n", fs.err.c_str());
      return DMD_E_FILE;
    }
  dmd_desc dc = *d;
  dc.P1 = dc.P2 = dc.P1_add = dc.P2_add = nullptr;
  const char* tc = getenv("DMD_BATCH_TC");
  const bool tc_form = d->nrhs > 1 && nb == 2 && d->precision == DMD_PREC_BF16X2 && !(tc && atoi(tc) == 0);
  if (((nb == 2 || nb == 4) && d->nkpair > 0 && !tc_form && !(d->flags & DMD_FLAG_ADJOINT)) ||
      (d->flags & DMD_FLAG_SPARSE))
    return create_impl(&dc, out, &fs);  // streamed: two chunks of the files in host memory at a time
  // the other forms take the operators from host memory
  std::vector<double> buf[4];
  const size_t n = (size_t)d->nkpair * fs.nb4;
  for (int m = 0; m < (fs.add ? 4 : 2); ++m) buf[m].resize(2 * (n ? n : 1));
  if (n) {
    for (int m = 0; m < (fs.add ? 4 : 2); ++m) {
      if (fseeko(fs.f[m], 0, SEEK_SET) != 0 || fread(buf[m].data(), 16, n, fs.f[m]) != n) return DMD_E_FILE;
    }
  }
  dc.P1 = buf[0].data();
  dc.P2 = buf[1].data();
  if (fs.add) {
    dc.P1_add = buf[2].data();
    dc.P2_add = buf[3].data();
  }
  return create_impl(&dc, out, nullptr);
}

int dmd_destroy(dmd_handle* h) {
  if (!h) return DMD_E_ARG;
  release(h);
  delete h;
  return DMD_OK;
}

int dmd_set_ddmdt_eq(dmd_handle* h, const double* eq) {
  if (!h) return DMD_E_ARG;
  CK(cudaSetDevice(h->dev));
  CK(cudaStreamSynchronize(h->st));
  drop_graphs(h);  // the captured step holds the drift pointer: capture again at the next dmd_rk4
  if (!eq) {
    if (h->d_eq) cudaFree(h->d_eq);
    h->d_eq = nullptr;
    return DMD_OK;
  }
  if (!h->d_eq) {
    int rc = dalloc(h, &h->d_eq, (size_t)h->nk * h->nb2);
    if (rc) return rc;
  }
  CK(cudaMemcpy(h->d_eq, eq, (size_t)h->nk * h->nb2 * 16, cudaMemcpyHostToDevice));
  return DMD_OK;
}

int dmd_func(dmd_handle* h, double t, const double* y, double* dydt) {
  if (!h || !y || !dydt) return DMD_E_ARG;
  CK(cudaSetDevice(h->dev));
  CK(cudaMemcpyAsync(h->d_in, y, h->nstate * 16, cudaMemcpyHostToDevice, h->st));
  int rc = rhs_plain(h, t, h->d_in, h->d_out);
  if (rc) return rc;
  CK(cudaMemcpyAsync(dydt, h->d_out, h->nstate * 16, cudaMemcpyDeviceToHost, h->st));
  CK(cudaStreamSynchronize(h->st));
  return DMD_OK;
}

int dmd_evolve_driver(dmd_handle* h, double t, const double* dm, const double* dm1, double* ddmdt) {
  if (!h || !dm || !ddmdt) return DMD_E_ARG;
  (void)dm1;  // the kernels form 1 - dm themselves (set_oneminusdm, DenMat.cpp:249-261)
  CK(cudaSetDevice(h->dev));
  CK(cudaMemcpyAsync(h->d_in, dm, h->nstate * 16, cudaMemcpyHostToDevice, h->st));
  FinishArgs fa = base_finish(h, h->d_in);
  fa.want_coh = 0;
  fa.mode = 0;
  fa.out = h->d_out;
  int rc = rhs(h, h->d_in, time_value(t), fa);
  if (rc) return rc;
  CK(cudaMemcpyAsync(ddmdt, h->d_out, h->nstate * 16, cudaMemcpyDeviceToHost, h->st));
  CK(cudaStreamSynchronize(h->st));
  return DMD_OK;
}

int dmd_evolve_coh(dmd_handle* h, double t, const double* dm, double* out) {
  if (!h || !dm || !out) return DMD_E_ARG;
  CK(cudaSetDevice(h->dev));
  CK(cudaMemcpyAsync(h->d_in, dm, h->nstate * 16, cudaMemcpyHostToDevice, h->st));
  FinishArgs fa = base_finish(h, h->d_in);
  fa.want_eph = 0;
  fa.want_coh = 1;
  fa.mode = 0;
  fa.out = h->d_out;
  int rc = rhs(h, h->d_in, time_value(t), fa);
  if (rc) return rc;
  CK(cudaMemcpyAsync(out, h->d_out, h->nstate * 16, cudaMemcpyDeviceToHost, h->st));
  CK(cudaStreamSynchronize(h->st));
  return DMD_OK;
}

int dmd_set_state(dmd_handle* h, double t, const double* y) {
  if (!h || !y) return DMD_E_ARG;
  CK(cudaSetDevice(h->dev));
  CK(cudaMemcpyAsync(h->d_y, y, h->nstate * 16, cudaMemcpyHostToDevice, h->st));
  CK(cudaStreamSynchronize(h->st));
  h->t = t;
  return DMD_OK;
}

int dmd_get_state(dmd_handle* h, double* t, double* y) {
  if (!h) return DMD_E_ARG;
  CK(cudaSetDevice(h->dev));
  if (y) CK(cudaMemcpyAsync(y, h->d_y, h->nstate * 16, cudaMemcpyDeviceToHost, h->st));
  CK(cudaStreamSynchronize(h->st));
  if (t) *t = h->t;
  return DMD_OK;
}

// RK4 step launches (captured into a graph by dmd_rk4). With recU / recA, the step also copies each
// stage's input (before its evaluation, which may overwrite it with the next stage's) to recU[s] and
// its forward sums (after the contraction) to recA[s].
static int rk4_step_launches(dmd_handle* h, double2* recU = nullptr, double2* recA = nullptr) {
  const size_t na = (size_t)h->nk * 2 * h->nb2;
  for (int s = 0; s < 4; ++s) {
    TimeArg ta;
    ta.t = 0;
    ta.tref = h->d_tref;
    ta.step = h->d_step;
    ta.stage = s;
    const double2* in = (s == 0) ? h->d_y : h->d_ytmp;
    FinishArgs fa = base_finish(h, in);
    fa.mode = 1;
    fa.stage = s;
    fa.tref = h->d_tref;
    fa.step = h->d_step;
    fa.K = h->d_K;
    fa.ybase = h->d_y;
    fa.ytmp = h->d_ytmp;
    if (recU) CK(cudaMemcpyAsync(recU + (size_t)s * h->nstate, in, h->nstate * 16, cudaMemcpyDeviceToDevice, h->st));
    int rc = rhs(h, in, ta, fa);
    if (rc) return rc;
    if (recA) CK(cudaMemcpyAsync(recA + (size_t)s * na, h->d_acc, na * 16, cudaMemcpyDeviceToDevice, h->st));
  }
  {
    ProfScope ps(h, 3);
    k_step_inc<<<1, 32, 0, h->st>>>(h->d_step);
  }
  h->launches++;
  CKL();
  return DMD_OK;
}

int dmd_rk4(dmd_handle* h, double dt, int64_t nsteps) {
  if (!h || nsteps < 0 || !(dt == dt)) return DMD_E_ARG;
  if (nsteps == 0) return DMD_OK;
  CK(cudaSetDevice(h->dev));
  const double tref[2] = {h->t, dt};
  const long long zero = 0;
  CK(cudaMemcpyAsync(h->d_tref, tref, 16, cudaMemcpyHostToDevice, h->st));
  CK(cudaMemcpyAsync(h->d_step, &zero, 8, cudaMemcpyHostToDevice, h->st));
  // pageable sources: wait so the host values stay valid
  CK(cudaStreamSynchronize(h->st));
  if (h->prof_on) {  // one step at a time, events around every kernel
    for (int64_t s = 0; s < nsteps; ++s) {
      int rc = rk4_step_launches(h);
      if (rc) return rc;
      CK(cudaStreamSynchronize(h->st));
      prof_harvest(h);
    }
    h->t = h->t + (double)nsteps * dt;
    return check_state(h);
  }
  if (!h->g_rk4) {
    cudaGraph_t g;
    const long long l0 = h->launches;
    CK(cudaStreamBeginCapture(h->st, cudaStreamCaptureModeThreadLocal));
    int rc = rk4_step_launches(h);
    cudaError_t e = cudaStreamEndCapture(h->st, &g);
    if (rc) return rc;
    if (e != cudaSuccess) return fail(h, DMD_E_CUDA, std::string("graph capture: ") + cudaGetErrorString(e));
    e = cudaGraphInstantiate(&h->g_rk4, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return fail(h, DMD_E_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(e));
    h->launches = l0;  // captured launches are counted when the graph runs
  }
  const long long per_step = h->npair ? (h->use_tc ? 21 : h->use_cb ? 17 : 13) : 9;
  for (int64_t s = 0; s < nsteps; ++s) {
    CK(cudaGraphLaunch(h->g_rk4, h->st));
    h->launches += per_step;
  }
  h->t = h->t + (double)nsteps * dt;  // = t0 + n*h as the stage times see it
  CK(cudaStreamSynchronize(h->st));
  return check_state(h);
}

int dmd_euler(dmd_handle* h, double dt, int64_t nsteps) {
  if (!h || nsteps < 0) return DMD_E_ARG;
  CK(cudaSetDevice(h->dev));
  for (int64_t s = 0; s < nsteps; ++s) {
    const double tref[2] = {h->t, dt};
    CK(cudaMemcpyAsync(h->d_tref, tref, 16, cudaMemcpyHostToDevice, h->st));
    FinishArgs fa = base_finish(h, h->d_y);
    fa.mode = 2;
    fa.tref = h->d_tref;
    fa.ybase = h->d_y;
    int rc = rhs(h, h->d_y, time_value(h->t), fa);
    if (rc) return rc;
    CK(cudaStreamSynchronize(h->st));
    h->t += dt;  // sdmk->t += dt_current() (DensityMatrix_Dynamics.h:232)
  }
  return check_state(h);
}

// ---------------------------------------------------------------------------------------------
// RKF45: gsl_odeiv2_driver_apply restated over device-resident state (see oracle/gsl_rkf45.c for
// the CPU statement of the same algorithm)
// ---------------------------------------------------------------------------------------------
namespace {
const double kAh[] = {1.0 / 4.0, 3.0 / 8.0, 12.0 / 13.0, 1.0, 1.0 / 2.0};
const double kB3[] = {3.0 / 32.0, 9.0 / 32.0};
const double kB4[] = {1932.0 / 2197.0, -7200.0 / 2197.0, 7296.0 / 2197.0};
const double kB5[] = {8341.0 / 4104.0, -32832.0 / 4104.0, 29440.0 / 4104.0, -845.0 / 4104.0};
const double kB6[] = {-6080.0 / 20520.0, 41040.0 / 20520.0, -28352.0 / 20520.0, 9295.0 / 20520.0, -5643.0 / 20520.0};
const double kC[] = {902880.0 / 7618050.0, 3953664.0 / 7618050.0, 3855735.0 / 7618050.0, -1371249.0 / 7618050.0,
                     277020.0 / 7618050.0};
const double kE[] = {1.0 / 360.0, -128.0 / 4275.0, -2197.0 / 75240.0, 1.0 / 50.0, 2.0 / 55.0};

struct Rkf {
  dmd_handle* h;
  int64_t nfev = 0;
  double* K(int j) { return (double*)(h->d_K + (size_t)j * h->nstate); }
};

int comb(dmd_handle* h, const double* base, int nterms, const int* kidx, const double* coef, double hs, int premul,
         double* out) {
  // coefficients by value through a small device table (copied from pageable host memory)
  int ibuf[8];
  double cbuf[8];
  for (int i = 0; i < nterms; ++i) {
    ibuf[i] = kidx[i];
    cbuf[i] = coef[i];
  }
  CK(cudaMemcpyAsync(h->d_coef_i, ibuf, sizeof(int) * nterms, cudaMemcpyHostToDevice, h->st));
  CK(cudaMemcpyAsync(h->d_coef, cbuf, sizeof(double) * nterms, cudaMemcpyHostToDevice, h->st));
  const size_t n = 2 * h->nstate;
  k_rk_comb<<<blocks_for((long long)n, 256), 256, 0, h->st>>>(n, base, (const double*)h->d_K, 2 * h->nstate, nterms,
                                                              h->d_coef_i, h->d_coef, hs, premul, out);
  h->launches++;
  CKL();
  CK(cudaStreamSynchronize(h->st));  // the small tables are reused by the next call
  return DMD_OK;
}

int feval(Rkf& r, double t, const double* y, double* out) {
  r.nfev++;
  return rhs_plain(r.h, t, (const double2*)y, (double2*)out);
}

int rkf45_step(Rkf& r, double t, double hs, double* y, double* rmax, double eps_abs, double eps_rel) {
  dmd_handle* h = r.h;
  double* yt = (double*)h->d_ytmp;
  int rc;
  const int i1[] = {0};
  if ((rc = comb(h, y, 1, i1, &kAh[0], hs, 1, yt))) return rc;
  if ((rc = feval(r, t + kAh[0] * hs, yt, r.K(1)))) return rc;
  const int i2[] = {0, 1};
  if ((rc = comb(h, y, 2, i2, kB3, hs, 0, yt))) return rc;
  if ((rc = feval(r, t + kAh[1] * hs, yt, r.K(2)))) return rc;
  const int i3[] = {0, 1, 2};
  if ((rc = comb(h, y, 3, i3, kB4, hs, 0, yt))) return rc;
  if ((rc = feval(r, t + kAh[2] * hs, yt, r.K(3)))) return rc;
  const int i4[] = {0, 1, 2, 3};
  if ((rc = comb(h, y, 4, i4, kB5, hs, 0, yt))) return rc;
  if ((rc = feval(r, t + kAh[3] * hs, yt, r.K(4)))) return rc;
  const int i5[] = {0, 1, 2, 3, 4};
  if ((rc = comb(h, y, 5, i5, kB6, hs, 0, yt))) return rc;
  if ((rc = feval(r, t + kAh[4] * hs, yt, r.K(5)))) return rc;
  const int i6[] = {0, 2, 3, 4, 5};
  if ((rc = comb(h, y, 5, i6, kC, hs, 0, y))) return rc;
  // error estimate and control ratio on the updated y
  int ebuf[5] = {0, 2, 3, 4, 5};
  CK(cudaMemcpyAsync(h->d_coef_i, ebuf, sizeof(ebuf), cudaMemcpyHostToDevice, h->st));
  CK(cudaMemcpyAsync(h->d_coef, kE, sizeof(kE), cudaMemcpyHostToDevice, h->st));
  const size_t n = 2 * h->nstate;
  const unsigned nbk = blocks_for((long long)n, 256);
  if (nbk > red_elems(h)) return fail(h, DMD_E_ARG, "state too large for the error reduction");
  k_rk_err<<<nbk, 256, 0, h->st>>>(n, y, (const double*)h->d_K, 2 * h->nstate, 5, h->d_coef_i, h->d_coef, hs, eps_abs,
                                   eps_rel, h->d_red);
  h->launches++;
  CKL();
  std::vector<double> bm(nbk);
  CK(cudaMemcpyAsync(bm.data(), h->d_red, nbk * 8, cudaMemcpyDeviceToHost, h->st));
  CK(cudaStreamSynchronize(h->st));
  double m = 2.2250738585072014e-308;
  for (double v : bm) m = v > m ? v : m;
  *rmax = m;
  return DMD_OK;
}

}  // namespace

int dmd_rkf45_apply(dmd_handle* h, double t1, double* hstep, double hmin, double hmax, double epsabs, double epsrel,
                    int64_t* nfev) {
  if (!h || !hstep) return DMD_E_ARG;
  CK(cudaSetDevice(h->dev));
  Rkf r;
  r.h = h;
  double* y = (double*)h->d_y;
  double* y0 = (double*)h->d_y0;
  const size_t bytes = h->nstate * 16;
  const int sign = (*hstep > 0.0) ? 1 : -1;
  if (sign * (t1 - h->t) < 0.0) return fail(h, DMD_E_ODE, "integration limits and step direction disagree");
  int rc;
  while (sign * (t1 - h->t) > 0.0) {
    // gsl_odeiv2_evolve_apply
    const double t0 = h->t;
    double h0 = *hstep;
    const double dt = t1 - t0;
    if ((dt < 0.0 && h0 > 0.0) || (dt > 0.0 && h0 < 0.0)) return fail(h, DMD_E_ODE, "step direction");
    CK(cudaMemcpyAsync(y0, y, bytes, cudaMemcpyDeviceToDevice, h->st));
    if ((rc = feval(r, t0, y, r.K(0)))) return rc;  // dydt_in
    for (;;) {
      int final_step = 0;
      if ((dt >= 0.0 && h0 > dt) || (dt < 0.0 && h0 < dt)) {
        h0 = dt;
        final_step = 1;
      }
      double rmax;
      if ((rc = rkf45_step(r, t0, h0, y, &rmax, epsabs, epsrel))) return rc;
      h->t = final_step ? t1 : t0 + h0;
      const double h_old = h0;
      // standard control, order 5
      int dec = 0;
      if (rmax > 1.1) {
        double q = 0.9 / pow(rmax, 1.0 / 5.0);
        if (q < 0.2) q = 0.2;
        h0 = q * h_old;
        dec = 1;
      } else if (rmax < 0.5) {
        double q = 0.9 / pow(rmax, 1.0 / 6.0);
        if (q > 5.0) q = 5.0;
        if (q < 1.0) q = 1.0;
        h0 = q * h_old;
      }
      if (dec) {
        volatile double t_curr = h->t, t_next = h->t + h0;
        if (fabs(h0) < fabs(h_old) && t_next != t_curr) {
          CK(cudaMemcpyAsync(y, y0, bytes, cudaMemcpyDeviceToDevice, h->st));
          h->t = t0;
          continue;  // retry with the smaller step (dydt_in reused)
        }
        h0 = h_old;
      }
      break;
    }
    *hstep = h0;
    if (fabs(*hstep) > hmax) *hstep = sign * hmax;
    if (fabs(*hstep) < hmin) {
      if (nfev) *nfev = r.nfev;
      return fail(h, DMD_E_ODE, "step size below hmin (GSL_ENOPROG)");
    }
  }
  if (nfev) *nfev = r.nfev;
  return check_state(h);
}

int dmd_set_observable(dmd_handle* h, int slot, const double* obs, const double* f, double prefac) {
  if (!h || slot < 0 || slot >= 8 || !obs || !f) return DMD_E_ARG;
  CK(cudaSetDevice(h->dev));
  int rc;
  if (!h->d_obs[slot] && (rc = dalloc(h, &h->d_obs[slot], h->nstate1))) return rc;
  if (!h->d_f[slot] && (rc = dalloc(h, &h->d_f[slot], (size_t)h->nk * h->nbdm))) return rc;
  CK(cudaMemcpy(h->d_obs[slot], obs, h->nstate1 * 16, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(h->d_f[slot], f, (size_t)h->nk * h->nbdm * 8, cudaMemcpyHostToDevice));
  h->obs_prefac[slot] = prefac;
  return DMD_OK;
}

int dmd_measure(dmd_handle* h, int slot, int bstart, int bend, double* tot, double* tot_amp) {
  if (!h || slot < 0 || slot >= 8 || !h->d_obs[slot] || bstart < 0 || bend > h->nbdm || bstart > bend) return DMD_E_ARG;
  CK(cudaSetDevice(h->dev));
  const unsigned nbk = blocks_for(h->nk, 256);
  if (2 * nbk > 4096) return fail(h, DMD_E_ARG, "nk too large for the observable reduction");
  k_measure<<<nbk, 256, 0, h->st>>>(h->nk, h->nbdm, bstart, bend, h->d_obs[slot], h->d_f[slot], h->d_edm, h->t,
                                    h->picture, h->d_y, h->d_red);
  h->launches++;
  CKL();
  std::vector<double> part(2 * nbk);
  CK(cudaMemcpyAsync(part.data(), h->d_red, 2 * nbk * 8, cudaMemcpyDeviceToHost, h->st));
  CK(cudaStreamSynchronize(h->st));
  double s1 = 0, s2 = 0;
  for (unsigned b = 0; b < nbk; ++b) {
    s1 += part[2 * b];
    s2 += part[2 * b + 1];
  }
  if (tot) *tot = s1 * h->obs_prefac[slot];
  if (tot_amp) *tot_amp = s2 * h->obs_prefac[slot];
  return DMD_OK;
}

int dmd_measure_batch(dmd_handle* h, int slot, int bstart, int bend, double* tot, double* tot_amp) {
  if (!h || slot < 0 || slot >= 8 || !h->d_obs[slot] || bstart < 0 || bend > h->nbdm || bstart > bend) return DMD_E_ARG;
  CK(cudaSetDevice(h->dev));
  const unsigned nbk = blocks_for(h->nk, 256);
  k_measure<<<dim3(nbk, h->nrhs), 256, 0, h->st>>>(h->nk, h->nbdm, bstart, bend, h->d_obs[slot], h->d_f[slot],
                                                   h->d_edm, h->t, h->picture, h->d_y, h->d_red, h->nstate1);
  h->launches++;
  CKL();
  std::vector<double> part(2 * (size_t)nbk * h->nrhs);
  CK(cudaMemcpyAsync(part.data(), h->d_red, part.size() * 8, cudaMemcpyDeviceToHost, h->st));
  CK(cudaStreamSynchronize(h->st));
  for (int q = 0; q < h->nrhs; ++q) {
    double s1 = 0, s2 = 0;
    for (unsigned b = 0; b < nbk; ++b) {
      s1 += part[2 * ((size_t)q * nbk + b)];
      s2 += part[2 * ((size_t)q * nbk + b) + 1];
    }
    if (tot) tot[q] = s1 * h->obs_prefac[slot];
    if (tot_amp) tot_amp[q] = s2 * h->obs_prefac[slot];
  }
  return DMD_OK;
}

int dmd_adjoint_rk4(dmd_handle* h, double t0, const double* y0, double dt, int64_t nsteps, int64_t checkpoint,
                    int slot, int bstart, int bend, int64_t nobs, const int64_t* obs_step,
                    const double* obs_weight, double* s_obs, double* dJdP, double* dJdy0) {
  if (!h || !y0 || nsteps < 1 || checkpoint < 1 || nobs < 0 || (nobs > 0 && (!obs_step || !obs_weight)))
    return DMD_E_ARG;
  if (slot < 0 || slot >= 8 || !h->d_obs[slot] || bstart < 0 || bend > h->nbdm || bstart > bend) return DMD_E_ARG;
  if (!h->adj) return fail(h, DMD_E_ARG, "dmd_adjoint_rk4 needs a handle created with DMD_FLAG_ADJOINT");
  if (h->lin || h->d_eq || h->nrhs != 1 || h->ee_on)
    return fail(h, DMD_E_ARG, "dmd_adjoint_rk4: linearized form, equilibrium drift, batches and an attached e-e "
                              "model are not supported");
  for (int64_t i = 0; i < nobs; ++i)
    if (obs_step[i] < 0 || obs_step[i] > nsteps || (i > 0 && obs_step[i] < obs_step[i - 1]))
      return fail(h, DMD_E_ARG, "obs_step must be ascending in [0, nsteps]");
  CK(cudaSetDevice(h->dev));
  const size_t n = h->nstate;
  const size_t nk2 = (size_t)h->nk * h->nb2;
  const size_t np = (size_t)h->npair * 2 * h->nb4;
  // When the stage inputs and forward sums of every step fit in 40 % of the free device memory, the
  // forward pass keeps them and the backward pass recomputes nothing (one stretch); otherwise the
  // trajectory is reversed stretch by stretch from checkpoints every `checkpoint` steps.
  size_t free_b = 0, total_b = 0;
  if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) free_b = 0;
  const double all_bytes = (double)nsteps * 4.0 * (double)(n + (size_t)h->nk * 2 * h->nb2) * 16.0;
  const char* kv = getenv("DMD_ADJ_KEEP_ALL");  // 0: always reverse by stretches (tests of that path)
  const bool keep_all = !(kv && atoi(kv) == 0) && all_bytes <= 0.4 * (double)free_b;
  if (keep_all) checkpoint = nsteps;
  const int64_t nseg = (nsteps + checkpoint - 1) / checkpoint, seglen = checkpoint < nsteps ? checkpoint : nsteps;
  AdjWork w;
  w.h = h;
  int rc;
  if ((rc = w.get(&w.ck, (size_t)nseg * n)) || (rc = w.get(&w.U, (size_t)seglen * 4 * n)) || (rc = w.get(&w.yb, n)) ||
      (rc = w.get(&w.ub, n)) || (rc = w.get(&w.kb, 4 * n)) || (rc = w.get(&w.tmp, 3 * n)) || (rc = w.get(&w.Xb, nk2)) ||
      (rc = w.get(&w.Yb, nk2)) || (rc = w.get(&w.rt, nk2)) || (rc = w.get(&w.st, nk2)) || (rc = w.get(&w.rtb, nk2)) ||
      (rc = w.get(&w.stb, nk2)) || (rc = w.get(&w.G, np)) ||
      (rc = w.get(&w.A, (size_t)seglen * 4 * (size_t)h->nk * 2 * h->nb2)))
    return rc;
  const size_t na = (size_t)h->nk * 2 * h->nb2;
  // double-float handles run the backward pair pass in double-float arithmetic (k_adj_pairs_df)
  const bool dfb = h->prec == DMD_PREC_F64X;
  if (dfb) {
    if ((rc = w.get(&w.dfv, 8 * nk2))) return rc;
    if (!h->d_Padf && (rc = dalloc(h, &h->d_Padf, np))) return rc;
    if (!h->padf_ok && np) {
      k_p_to_df<<<blocks_for((long long)np, 256), 256, 0, h->st>>>(np, h->use_cb ? h->d_Praw : h->d_P, h->d_Padf);
      h->launches++;
      CKL();
      h->padf_ok = 1;
    }
  }
  CK(cudaMemsetAsync(w.G, 0, (np ? np : 1) * 16, h->st));
  CK(cudaMemsetAsync(w.yb, 0, n * 16, h->st));
  CK(cudaMemcpyAsync(w.ck, y0, n * 16, cudaMemcpyHostToDevice, h->st));
  // forward: checkpoints at multiples of `checkpoint`, observed totals
  int64_t j = 0;
  double2* cur = w.ck;
  double2* spare[2] = {w.tmp + n, w.tmp + 2 * n};
  int sp = 0;
  for (; j < nobs && obs_step[j] == 0; ++j) {
    double v;
    if ((rc = measure_on(h, slot, bstart, bend, cur, t0, &v))) return rc;
    if (s_obs) s_obs[j] = v;
  }
  if (keep_all && !h->prof_on) {
    // the forward pass as captured RK4 steps (the handle's graph of dmd_rk4 plus copies of every
    // stage input and forward sums into d_rec), each step's stage data then moved to its slot; the
    // handle's own state and time are restored afterwards
    double2* ysave = nullptr;
    if ((rc = w.get(&ysave, n))) return rc;
    if (!h->d_rec && (rc = dalloc(h, &h->d_rec, 4 * (n + na)))) return rc;
    const double tsave = h->t;
    const double tref[2] = {t0, dt};
    const long long zero = 0;
    CK(cudaMemcpyAsync(ysave, h->d_y, n * 16, cudaMemcpyDeviceToDevice, h->st));
    CK(cudaMemcpyAsync(h->d_y, w.ck, n * 16, cudaMemcpyDeviceToDevice, h->st));
    CK(cudaMemcpyAsync(h->d_tref, tref, 16, cudaMemcpyHostToDevice, h->st));
    CK(cudaMemcpyAsync(h->d_step, &zero, 8, cudaMemcpyHostToDevice, h->st));
    CK(cudaStreamSynchronize(h->st));  // pageable sources
    if (!h->g_rk4_rec) {
      cudaGraph_t g;
      const long long l0 = h->launches;
      CK(cudaStreamBeginCapture(h->st, cudaStreamCaptureModeThreadLocal));
      rc = rk4_step_launches(h, h->d_rec, h->d_rec + 4 * n);
      cudaError_t e = cudaStreamEndCapture(h->st, &g);
      if (rc) return rc;
      if (e != cudaSuccess) return fail(h, DMD_E_CUDA, std::string("graph capture: ") + cudaGetErrorString(e));
      e = cudaGraphInstantiate(&h->g_rk4_rec, g, 0);
      cudaGraphDestroy(g);
      if (e != cudaSuccess) return fail(h, DMD_E_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(e));
      h->launches = l0;
    }
    const long long per_step = h->npair ? (h->use_tc ? 21 : h->use_cb ? 17 : 13) : 9;
    for (int64_t s = 0; s < nsteps; ++s) {
      CK(cudaGraphLaunch(h->g_rk4_rec, h->st));
      h->launches += per_step;
      CK(cudaMemcpyAsync(w.U + (size_t)s * 4 * n, h->d_rec, 4 * n * 16, cudaMemcpyDeviceToDevice, h->st));
      CK(cudaMemcpyAsync(w.A + (size_t)s * 4 * na, h->d_rec + 4 * n, 4 * na * 16, cudaMemcpyDeviceToDevice, h->st));
      for (; j < nobs && obs_step[j] == s + 1; ++j) {
        double v;
        if ((rc = measure_on(h, slot, bstart, bend, h->d_y, t0 + (double)(s + 1) * dt, &v))) return rc;
        if (s_obs) s_obs[j] = v;
      }
    }
    CK(cudaMemcpyAsync(h->d_y, ysave, n * 16, cudaMemcpyDeviceToDevice, h->st));
    h->t = tsave;
  }
  for (int64_t s = 0; s < nsteps && !(keep_all && !h->prof_on); ++s) {
    double2* next = ((s + 1) % checkpoint == 0 && (s + 1) < nsteps) ? w.ck + (size_t)((s + 1) / checkpoint) * n
                                                                      : spare[sp];
    if ((rc = adj_rk4_step(h, cur, t0 + (double)s * dt, dt, keep_all ? w.U + (size_t)s * 4 * n : nullptr, next,
                           w.tmp, keep_all ? w.A + (size_t)s * 4 * na : nullptr)))
      return rc;
    for (; j < nobs && obs_step[j] == s + 1; ++j) {
      double v;
      if ((rc = measure_on(h, slot, bstart, bend, next, t0 + (double)(s + 1) * dt, &v))) return rc;
      if (s_obs) s_obs[j] = v;
    }
    if (next == spare[sp]) sp ^= 1;
    cur = next;
  }
  // backward
  const unsigned gn = blocks_for((long long)n, 256);
  j = nobs - 1;
  for (int64_t sg = nseg - 1; sg >= 0; --sg) {
    const int64_t n0 = sg * checkpoint, n1 = std::min<int64_t>(n0 + checkpoint, nsteps);
    const double2* y = w.ck + (size_t)sg * n;
    for (int64_t s = n0; s < n1 && !keep_all; ++s) {  // stage inputs of the stretch
      double2* out = spare[sp];
      if ((rc = adj_rk4_step(h, y, t0 + (double)s * dt, dt, w.U + (size_t)(s - n0) * 4 * n, out, w.tmp,
                             w.A + (size_t)(s - n0) * 4 * na)))
        return rc;
      y = out;
      sp ^= 1;
    }
    for (int64_t s = n1 - 1; s >= n0; --s) {
      const double t = t0 + (double)s * dt;
      for (; j >= 0 && obs_step[j] == s + 1; --j) {
        k_adj_obs<<<gn, 256, 0, h->st>>>(h->nk, h->nbdm, bstart, bend, h->d_obs[slot], h->d_edm, t + dt, h->picture,
                                         obs_weight[j] * h->obs_prefac[slot], w.yb);
        h->launches++;
      }
      const double cst[4] = {dt / 6.0, dt / 3.0, dt / 3.0, dt / 6.0};
      for (int q = 0; q < 4; ++q) k_scale<<<gn, 256, 0, h->st>>>(n, w.kb + q * n, cst[q], w.yb);
      h->launches += 4;
      CKL();
      const double2* U = w.U + (size_t)(s - n0) * 4 * n;
      const double2* As = w.A + (size_t)(s - n0) * 4 * na;  // forward sums of the four stages
      if ((rc = adj_vjp(h, w, U + 3 * n, t + dt, w.kb + 3 * n, w.kb + 2 * n, dt, As + 3 * na)) ||
          (rc = adj_vjp(h, w, U + 2 * n, t + 0.5 * dt, w.kb + 2 * n, w.kb + n, 0.5 * dt, As + 2 * na)) ||
          (rc = adj_vjp(h, w, U + n, t + 0.5 * dt, w.kb + n, w.kb, 0.5 * dt, As + na)) ||
          (rc = adj_vjp(h, w, U, t, w.kb, nullptr, 0.0, As)))
        return rc;
    }
  }
  for (; j >= 0 && obs_step[j] == 0; --j) {
    k_adj_obs<<<gn, 256, 0, h->st>>>(h->nk, h->nbdm, bstart, bend, h->d_obs[slot], h->d_edm, t0, h->picture,
                                     obs_weight[j] * h->obs_prefac[slot], w.yb);
    h->launches++;
  }
  if (dJdP && np) {  // device G is [pair][P1 | P2][nb4] with dJ = Re sum(dP o G): conj(G) in FP64 in place
    if (dfb) k_df_to_f64<<<blocks_for((long long)np, 256), 256, 0, h->st>>>(np, (float4*)w.G, 1);
    else k_conj<<<blocks_for((long long)np, 256), 256, 0, h->st>>>(np, w.G);
    h->launches++;
  }
  CKL();
  if (dJdy0) CK(cudaMemcpyAsync(dJdy0, w.yb, n * 16, cudaMemcpyDeviceToHost, h->st));
  if (dJdP && np) {  // out: [P1 | P2][pair][nb4], dJ/dRe P = Re G, dJ/dIm P = -Im G: each half gathered on
                     // the device in chunks and copied contiguously
    const size_t nb4 = (size_t)h->nb4, npair = (size_t)h->npair;
    const size_t chunk = std::max<size_t>(1, std::min<size_t>(npair, (256u << 20) / (nb4 * 16)));
    double2* tmp = nullptr;
    if ((rc = w.get(&tmp, chunk * nb4))) return rc;
    PinnedStage stage;  // page-locked staging, then a threaded copy into the caller's (pageable) array
    if (!stage.alloc(chunk * nb4 * 16)) return fail(h, DMD_E_NOMEM, "dmd_adjoint_rk4: page-locked staging buffer");
    for (int m = 0; m < 2; ++m)
      for (size_t p0 = 0; p0 < npair; p0 += chunk) {
        const size_t cnt = std::min(chunk, npair - p0);
        k_gather_half<<<blocks_for((long long)(cnt * nb4), 256), 256, 0, h->st>>>(cnt * nb4, nb4, w.G + p0 * 2 * nb4, m, tmp);
        h->launches++;
        CK(cudaMemcpyAsync(stage.p, tmp, cnt * nb4 * 16, cudaMemcpyDeviceToHost, h->st));
        CK(cudaStreamSynchronize(h->st));
        parallel_copy(dJdP + 2 * ((size_t)m * npair + p0) * nb4, stage.p, cnt * nb4 * 16);
      }
  }
  CK(cudaStreamSynchronize(h->st));
  unsigned int derr = 0;
  CK(cudaMemcpy(&derr, h->d_err, sizeof(derr), cudaMemcpyDeviceToHost));
  if (derr) {
    cudaMemset(h->d_err, 0, sizeof(derr));
    return fail(h, DMD_E_TIMEOUT, "a bounded device wait gave up (bulk copy did not complete)");
  }
  return DMD_OK;
}

}  // extern "C"

struct dmd_group {
  std::vector<dmd_handle*> m;
  int dev = 0;
  cudaStream_t st = nullptr;
  cudaGraphExec_t exec = nullptr;
  std::vector<cudaEvent_t> ev;  // [0] fork, [1..n] joins
};

extern "C" {

int dmd_group_create(dmd_handle* const* members, int n, dmd_group** out) {
  if (!members || n < 1 || !out) return DMD_E_ARG;
  *out = nullptr;
  for (int i = 0; i < n; ++i)
    if (!members[i] || members[i]->dev != members[0]->dev) return DMD_E_ARG;
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < i; ++j)
      if (members[i] == members[j]) return DMD_E_ARG;
  if (cudaSetDevice(members[0]->dev) != cudaSuccess) return DMD_E_CUDA;
  dmd_group* g = new dmd_group();
  g->m.assign(members, members + n);
  g->dev = members[0]->dev;
  bool ok = cudaStreamCreateWithFlags(&g->st, cudaStreamNonBlocking) == cudaSuccess;
  g->ev.assign(n + 1, nullptr);
  for (auto& e : g->ev) ok = ok && cudaEventCreateWithFlags(&e, cudaEventDisableTiming) == cudaSuccess;
  if (!ok) {
    dmd_group_destroy(g);
    return DMD_E_CUDA;
  }
  *out = g;
  return DMD_OK;
}

int dmd_group_destroy(dmd_group* g) {
  if (!g) return DMD_E_ARG;
  cudaSetDevice(g->dev);
  if (g->exec) cudaGraphExecDestroy(g->exec);
  for (auto e : g->ev)
    if (e) cudaEventDestroy(e);
  if (g->st) cudaStreamDestroy(g->st);
  delete g;
  return DMD_OK;
}

int dmd_group_rk4(dmd_group* g, double dt, int64_t nsteps) {
  if (!g || nsteps < 0 || !(dt == dt)) return DMD_E_ARG;
  if (nsteps == 0) return DMD_OK;
  dmd_handle* h0 = g->m[0];
  dmd_handle* h = h0;  // error messages go to the first member
  CK(cudaSetDevice(g->dev));
  for (dmd_handle* hm : g->m) {  // every member's stage times start from its own time
    const double tref[2] = {hm->t, dt};
    const long long zero = 0;
    if (cudaMemcpyAsync(hm->d_tref, tref, 16, cudaMemcpyHostToDevice, hm->st) != cudaSuccess ||
        cudaMemcpyAsync(hm->d_step, &zero, 8, cudaMemcpyHostToDevice, hm->st) != cudaSuccess ||
        cudaStreamSynchronize(hm->st) != cudaSuccess)
      return fail(hm, DMD_E_CUDA, "group: time reference upload");
  }
  if (!g->exec) {  // one step of every member as parallel branches of one graph
    std::vector<long long> l0;
    for (dmd_handle* hm : g->m) l0.push_back(hm->launches);
    CK(cudaStreamBeginCapture(g->st, cudaStreamCaptureModeThreadLocal));
    int rc = DMD_OK;
    cudaError_t e = cudaEventRecord(g->ev[0], g->st);
    for (size_t i = 0; i < g->m.size() && rc == DMD_OK && e == cudaSuccess; ++i) {
      dmd_handle* hm = g->m[i];
      e = cudaStreamWaitEvent(hm->st, g->ev[0], 0);
      if (e == cudaSuccess) rc = rk4_step_launches(hm);
      if (rc == DMD_OK && e == cudaSuccess) e = cudaEventRecord(g->ev[i + 1], hm->st);
      if (rc == DMD_OK && e == cudaSuccess) e = cudaStreamWaitEvent(g->st, g->ev[i + 1], 0);
    }
    cudaGraph_t graph = nullptr;
    const cudaError_t e2 = cudaStreamEndCapture(g->st, &graph);
    if (rc) {
      if (graph) cudaGraphDestroy(graph);
      return rc;
    }
    if (e != cudaSuccess || e2 != cudaSuccess) {
      if (graph) cudaGraphDestroy(graph);
      return fail(h, DMD_E_CUDA, std::string("group graph capture: ") + cudaGetErrorString(e != cudaSuccess ? e : e2));
    }
    e = cudaGraphInstantiate(&g->exec, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) return fail(h, DMD_E_CUDA, std::string("group graph instantiate: ") + cudaGetErrorString(e));
    for (size_t i = 0; i < g->m.size(); ++i) g->m[i]->launches = l0[i];  // counted when the graph runs
  }
  for (int64_t s = 0; s < nsteps; ++s) CK(cudaGraphLaunch(g->exec, g->st));
  CK(cudaStreamSynchronize(g->st));
  int rc = DMD_OK;
  for (dmd_handle* hm : g->m) {
    const long long per_step = hm->npair ? (hm->use_tc ? 21 : hm->use_cb ? 17 : 13) : 9;
    hm->launches += per_step * nsteps;
    hm->t = hm->t + (double)nsteps * dt;
    const int r = check_state(hm);
    if (r && !rc) rc = r;
  }
  return rc;
}

}  // extern "C"

namespace {
// waits on a phase that nothing completes: the bounded wait gives up and raises the flag
__global__ void k_wait_never(unsigned int* errflag, uint32_t polls) {
  __shared__ uint64_t bar;
  if (threadIdx.x == 0) {
    mbar_init(&bar, 1);
    fence_mbar_init();
  }
  __syncthreads();
  if (threadIdx.x == 0) mbar_wait_bounded(&bar, 0u, errflag, polls);
}
__global__ void k_set_one(unsigned int* p) { *p = 1u; }

// fused multiply-add throughput: 8 independent chains per thread, `iters` rounds; the sums are
// stored only when `sink` is set (never by the probe), which keeps the chains live
template <typename T>
__global__ void __launch_bounds__(256) k_fma_rate(int iters, T a, T b, T* sink) {
  T c[8];
#pragma unroll
  for (int i = 0; i < 8; ++i) c[i] = (T)(threadIdx.x + i);
#pragma unroll 1
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int r = 0; r < 16; ++r)
#pragma unroll
      for (int i = 0; i < 8; ++i) c[i] = fma(c[i], a, b);
  }
  if (sink) {
    T s = 0;
#pragma unroll
    for (int i = 0; i < 8; ++i) s += c[i];
    sink[blockIdx.x * blockDim.x + threadIdx.x] = s;
  }
}

// raw operators of a chunk of pairs ([pair][P1 | P2][nb^4]) += scale * (P1_add | P2_add), the additive
// operators of the chunk given as [P1: cnt][nb^4] then [P2: cnt][nb^4]
__global__ void k_praw_axpy(long long cnt, size_t nb4, const double2* __restrict__ add, double scale,
                            double2* __restrict__ raw) {
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  const long long n = cnt * (long long)nb4;
  if (i >= 2 * n) return;
  const int m = (int)(i / n);
  const long long r = i - m * n, j = r / (long long)nb4, e = r - j * (long long)nb4;
  double2& o = raw[(size_t)j * 2 * nb4 + (size_t)m * nb4 + e];
  const double2 a = add[i];
  o = mk2(__dadd_rn(o.x, __dmul_rn(a.x, scale)), __dadd_rn(o.y, __dmul_rn(a.y, scale)));
}

template <typename T>
int fma_rate(int device, double* tflops) {
  int nsm = 0;
  if (cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, device) != cudaSuccess) return DMD_E_CUDA;
  const int blocks = nsm * 8, threads = 256;
  const int iters = sizeof(T) == 8 ? 256 : 8192;  // ~20 ms (FP64) / ~10 ms (FP32) per launch on GB300
  cudaEvent_t e0, e1;
  if (cudaEventCreate(&e0) != cudaSuccess) return DMD_E_CUDA;
  if (cudaEventCreate(&e1) != cudaSuccess) {
    cudaEventDestroy(e0);
    return DMD_E_CUDA;
  }
  int rc = DMD_OK;
  float best = 0.f;
  for (int rep = 0; rep < 4 && rc == DMD_OK; ++rep) {  // the first launch warms up
    cudaEventRecord(e0);
    k_fma_rate<T><<<blocks, threads>>>(iters, (T)0.999999, (T)1e-7, (T*)nullptr);
    cudaEventRecord(e1);
    float ms = 0.f;
    if (cudaEventSynchronize(e1) != cudaSuccess || cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess) rc = DMD_E_CUDA;
    else if (rep > 0 && (best == 0.f || ms < best)) best = ms;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (rc != DMD_OK || best <= 0.f) return rc ? rc : DMD_E_CUDA;
  const double flops = 2.0 * blocks * threads * (double)iters * 16 * 8;
  *tflops = flops / (best * 1e-3) / 1e12;
  return DMD_OK;
}
}  // namespace

extern "C" {

int dmd_selftest_wait_timeout(int device, uint32_t polls, int* status) {
  if (!status || polls < 1 || polls > (1u << 20)) return DMD_E_ARG;
  *status = DMD_OK;
  if (cudaSetDevice(device) != cudaSuccess) return DMD_E_NODEV;
  unsigned int* d = nullptr;
  if (cudaMalloc((void**)&d, 2 * sizeof(unsigned int)) != cudaSuccess) return DMD_E_NOMEM;
  int rc = DMD_OK;
  unsigned int hv[2] = {0, 0};
  if (cudaMemset(d, 0, 2 * sizeof(unsigned int)) != cudaSuccess) rc = DMD_E_CUDA;
  if (rc == DMD_OK) {
    k_wait_never<<<1, 32>>>(d, polls);
    if (cudaDeviceSynchronize() != cudaSuccess) rc = DMD_E_CUDA;
  }
  if (rc == DMD_OK) {  // the context still works: a second kernel runs and writes
    k_set_one<<<1, 1>>>(d + 1);
    if (cudaMemcpy(hv, d, sizeof(hv), cudaMemcpyDeviceToHost) != cudaSuccess) rc = DMD_E_CUDA;
  }
  cudaFree(d);
  if (rc != DMD_OK) return rc;
  if (hv[1] != 1u) return DMD_E_CUDA;
  *status = (hv[0] & DMD_DEVERR_TIMEOUT) ? DMD_E_TIMEOUT : DMD_OK;
  return DMD_OK;
}

int dmd_add_operators(dmd_handle* h, const double* P1_add, const double* P2_add, double scale) {
  if (!h || !P1_add || !P2_add) return DMD_E_ARG;
  if (!h->use_cb || h->use_tc || h->lin || h->nrhs != 1 || !h->d_Praw || !h->d_dst || h->ee_on)
    return fail(h, DMD_E_ARG, "dmd_add_operators needs a handle made with DMD_FLAG_ADJOINT (or DMD_FLAG_EE without "
                              "an attached e-e model), nb = 2 or 4, a single state, not linearized");
  CK(cudaSetDevice(h->dev));
  CK(cudaStreamSynchronize(h->st));
  const size_t nb4 = (size_t)h->nb4;
  const long long chunk = std::max<long long>(1, std::min<long long>(h->npair, (128LL << 20) / (long long)(2 * nb4 * 16)));
  double2* tmp = nullptr;
  int rc;
  if ((rc = dalloc(h, &tmp, (size_t)chunk * 2 * nb4))) return rc;
  cudaError_t e = cudaSuccess;
  for (long long p0 = 0; p0 < h->npair && e == cudaSuccess; p0 += chunk) {
    const long long cnt = std::min<long long>(chunk, h->npair - p0);
    const size_t n = (size_t)cnt * nb4;
    e = cudaMemcpy(tmp, P1_add + 2 * (size_t)p0 * nb4, n * 16, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(tmp + n, P2_add + 2 * (size_t)p0 * nb4, n * 16, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) {
      k_praw_axpy<<<blocks_for((long long)(2 * n), 256), 256, 0, h->st>>>((long long)cnt, nb4, tmp, scale,
                                                                           h->d_Praw + 2 * (size_t)p0 * nb4);
      e = cudaGetLastError();
      if (e == cudaSuccess) e = cudaStreamSynchronize(h->st);
    }
  }
  cudaFree(tmp);
  h->padf_ok = 0;
  if (e != cudaSuccess) return fail(h, DMD_E_CUDA, std::string("dmd_add_operators: ") + cudaGetErrorString(e));
  // the stored form again from the updated operators (and, in the deviation forms, the constant term)
  const bool dev = deviation_form(h->prec);
  if (dev) CK(cudaMemsetAsync(h->d_acc0, 0, (size_t)h->nk * 2 * h->nb2 * sizeof(double2), h->st));
  const FillSrc fs = {h->d_Praw, nb4, 2 * nb4, nullptr, 0, 0};
  const unsigned g = blocks_for(h->npair, 128);
  if (h->nb == 2)
    k_cb_fill<2><<<g, 128, 0, h->st>>>(0, h->npair, fs, 0.0, (const CbDst*)h->d_dst, 0, h->prec, elem_bytes(h->prec),
                                       (unsigned char*)h->d_P, h->d_fref, dev ? (double*)h->d_acc0 : nullptr);
  else
    k_cb_fill<4><<<g, 128, 0, h->st>>>(0, h->npair, fs, 0.0, (const CbDst*)h->d_dst, 0, h->prec, elem_bytes(h->prec),
                                       (unsigned char*)h->d_P, h->d_fref, dev ? (double*)h->d_acc0 : nullptr);
  h->launches += 1 + (h->npair + chunk - 1) / chunk;
  CKL();
  CK(cudaStreamSynchronize(h->st));
  return DMD_OK;
}

int dmd_peak_fma(int device, int fp64, double* tflops) {
  if (!tflops) return DMD_E_ARG;
  *tflops = 0.0;
  if (cudaSetDevice(device) != cudaSuccess) return DMD_E_NODEV;
  return fp64 ? fma_rate<double>(device, tflops) : fma_rate<float>(device, tflops);
}

int dmd_autotune(dmd_handle* h, int evals, int* chosen) {
  if (!h || evals < 1) return DMD_E_ARG;
  CK(cudaSetDevice(h->dev));
  // candidate shapes of this handle's contraction
  std::vector<int> cand;
  int* knob = nullptr;
  if (h->use_cb && !h->use_tc && h->nrhs == 1 && h->prec == DMD_PREC_F64X && h->nb == 2) {
    cand = {0, 1, 2, 3, 4};
    knob = &h->pcfg;
  } else if (h->use_cb && !h->use_tc && h->nrhs == 1 && h->prec == DMD_PREC_F64 && h->nb == 2) {
    cand = {0, 1, 2, 3};
    knob = &h->pcfg64;
  } else if (h->use_cb && !h->use_tc && h->nrhs > 1 && h->prec == DMD_PREC_F32) {
    cand = {4, 8};
    knob = &h->brw;
  } else if (h->use_tc) {
    cand = {4, 3, 2};
    knob = &h->tcst;
  }
  if (!knob) {
    if (chosen) *chosen = 0;
    return DMD_OK;
  }
  cudaEvent_t a = nullptr, b = nullptr;
  CK(cudaEventCreate(&a));
  CK(cudaEventCreate(&b));
  const int keep = *knob;
  int best = keep, rc = DMD_OK;
  float best_ms = 1e30f;
  for (int c : cand) {
    *knob = c;
    if ((rc = rhs_plain(h, h->t, h->d_y, h->d_out))) break;  // warm-up
    cudaEventRecord(a, h->st);
    for (int i = 0; i < evals && rc == DMD_OK; ++i) rc = rhs_plain(h, h->t, h->d_y, h->d_out);
    cudaEventRecord(b, h->st);
    if (rc) break;
    if (cudaEventSynchronize(b) != cudaSuccess) {
      rc = fail(h, DMD_E_CUDA, "autotune timing");
      break;
    }
    float ms = 0.f;
    cudaEventElapsedTime(&ms, a, b);
    if (ms < best_ms) {
      best_ms = ms;
      best = c;
    }
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  *knob = rc ? keep : best;
  drop_graphs(h);  // the captured step holds the old kernels
  if (rc) return rc;
  if (chosen) *chosen = best;
  return check_state(h);
}

int dmd_pair_bytes(const dmd_handle* h, int64_t* n) {
  if (!h || !n) return DMD_E_ARG;
  *n = h->pair_bytes;
  return DMD_OK;
}

int dmd_launch_count(const dmd_handle* h, int64_t* n) {
  if (!h || !n) return DMD_E_ARG;
  *n = h->launches;
  return DMD_OK;
}

int dmd_sync(dmd_handle* h) {
  if (!h) return DMD_E_ARG;
  CK(cudaSetDevice(h->dev));
  CK(cudaStreamSynchronize(h->st));
  prof_harvest(h);
  return DMD_OK;
}

int dmd_pinned_alloc(size_t bytes, void** out) {
  if (!out) return DMD_E_ARG;
  *out = nullptr;
  cudaError_t e = cudaHostAlloc(out, bytes ? bytes : 1, cudaHostAllocDefault);
  if (e != cudaSuccess) return e == cudaErrorMemoryAllocation ? DMD_E_NOMEM : DMD_E_CUDA;
  return DMD_OK;
}

int dmd_pinned_free(void* p) {
  if (!p) return DMD_E_ARG;
  return cudaFreeHost(p) == cudaSuccess ? DMD_OK : DMD_E_CUDA;
}

int dmd_timer(dmd_handle* h, int op, double* ms) {
  if (!h || (op != 0 && op != 1)) return DMD_E_ARG;
  CK(cudaSetDevice(h->dev));
  for (auto& e : h->tev)
    if (!e) CK(cudaEventCreate(&e));
  if (op == 0) {
    CK(cudaEventRecord(h->tev[0], h->st));
    return DMD_OK;
  }
  CK(cudaEventRecord(h->tev[1], h->st));
  CK(cudaEventSynchronize(h->tev[1]));
  float f = 0;
  CK(cudaEventElapsedTime(&f, h->tev[0], h->tev[1]));
  if (ms) *ms = f;
  return DMD_OK;
}

int dmd_set_profiling(dmd_handle* h, int on) {
  if (!h) return DMD_E_ARG;
  CK(cudaSetDevice(h->dev));
  CK(cudaStreamSynchronize(h->st));
  prof_harvest(h);
  h->prof_on = on ? 1 : 0;
  if (on)
    for (int i = 0; i < 5; ++i) {
      h->prof_ms[i] = 0;
      h->prof_n[i] = 0;
    }
  return DMD_OK;
}

int dmd_ee_attach(dmd_handle* h, const dmd_ee_desc* ee) {
  if (!h || !ee) return DMD_E_ARG;
  if (!h->eek || !h->d_dst || !h->d_Praw) return fail(h, DMD_E_STATE, "the handle was not made with DMD_FLAG_EE");
  if (h->ee_on) return fail(h, DMD_E_STATE, "an e-e model is already attached");
  if (ee->nbw < h->nb || !ee->kvec || !ee->U || !ee->f || ee->kmesh[0] < 1 || ee->kmesh[1] < 1 || ee->kmesh[2] < 1 ||
      ee->formula < DMD_SCREEN_UNSCREENED || ee->formula > DMD_SCREEN_RPA || !(ee->degauss > 0) ||
      !(ee->ethr >= 0) || !(ee->cell_size > 0) || !(ee->nk_full > 0) || !(ee->temperature > 0) ||
      !(ee->eps_background >= 1) || !(ee->meff > 0) || ee->dynamic < 0 || ee->dynamic > 1 || !(ee->eppa >= 0) ||
      !(ee->smearing >= 0))
    return fail(h, DMD_E_ARG, "e-e model description");
  if (ee->dynamic && ee->formula != DMD_SCREEN_RPA)  // Scatt_Param.h:28-29
    return fail(h, DMD_E_ARG, "plasmon-pole screening needs the RPA formula (debye and Bechstedt are static)");
  if (!ee->dynamic && ee->two_freqs)
    return fail(h, DMD_E_ARG, "only for dynamic screening, dynamic_screening_ee_two_freqs can be true");
  CK(cudaSetDevice(h->dev));
  const int nk = h->nk, nb = h->nb;
  const size_t nmesh = (size_t)ee->kmesh[0] * ee->kmesh[1] * ee->kmesh[2];
  if (nmesh > ((size_t)1 << 31)) return fail(h, DMD_E_ARG, "k mesh too large for the mesh table");
  // mesh indices (kIndexMap::ikvec3, comm/kmap.cpp:15-23) and the mesh table; the first k-point of
  // an index wins, as std::map::insert keeps it (comm/kmap.h:22-28)
  std::vector<int4> kidx(nk);
  std::vector<int> kmap(nmesh, -1);
  for (int k = 0; k < nk; ++k) {
    int v[3];
    for (int d = 0; d < 3; ++d) {
      const double x = ee->kvec[3 * k + d];
      const double ki = x - std::floor(x);
      v[d] = (int)std::round(ee->kmesh[d] * ki);
      if (v[d] == ee->kmesh[d]) v[d] = 0;
      if (!(v[d] >= 0 && v[d] < ee->kmesh[d])) return fail(h, DMD_E_ARG, "k-point off the mesh table");
    }
    kidx[k] = make_int4(v[0], v[1], v[2], 0);
    int& slot = kmap[((size_t)v[0] * ee->kmesh[1] + v[1]) * ee->kmesh[2] + v[2]];
    if (slot < 0) slot = k;
  }
  std::vector<double> ew((size_t)nk * nb);
  CK(cudaMemcpy(ew.data(), h->d_ew, ew.size() * 8, cudaMemcpyDeviceToHost));
  // FP32 window energies relative to their minimum for the candidate test; the FP32 sum of four
  // of them is within 4 x 2^-24 x span of the exact one, so the margin keeps the test a superset
  double emin = ew[0], emax = ew[0];
  for (double v : ew) {
    emin = std::min(emin, v);
    emax = std::max(emax, v);
  }
  std::vector<float> ewf(ew.size());
  for (size_t i = 0; i < ew.size(); ++i) ewf[i] = (float)(ew[i] - emin);
  const double margin = 1e-6 * (emax - emin) + 1e-12;
  int rc;
  if ((rc = dalloc(h, &h->d_ee_kvec, (size_t)nk * 3)) || (rc = dalloc(h, &h->d_ee_kidx, (size_t)nk)) ||
      (rc = dalloc(h, &h->d_ee_kmap, nmesh)) || (rc = dalloc(h, &h->d_ee_U, (size_t)nk * ee->nbw * nb)) ||
      (rc = dalloc(h, &h->d_ee_ewf, (size_t)nk * nb)) || (rc = dalloc(h, &h->d_ee_f, (size_t)nk * nb)) ||
      (rc = dalloc(h, &h->d_ee_dm, (size_t)nk * h->nb2)) || (rc = dalloc(h, &h->d_ee_dm1, (size_t)nk * h->nb2)) ||
      (rc = dalloc(h, &h->d_ee_dmf, (size_t)nk * h->nb2)) || (rc = dalloc(h, &h->d_ee_dm1f, (size_t)nk * h->nb2)) ||
      (rc = dalloc(h, &h->d_ee_scr, 1)) || (rc = dalloc(h, &h->d_ee_Pee, (size_t)h->npair * 2 * h->nb4)))
    return rc;
  CK(cudaMemcpy(h->d_ee_kvec, ee->kvec, (size_t)nk * 3 * 8, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(h->d_ee_kidx, kidx.data(), (size_t)nk * sizeof(int4), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(h->d_ee_kmap, kmap.data(), nmesh * sizeof(int), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(h->d_ee_U, ee->U, (size_t)nk * ee->nbw * nb * 16, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(h->d_ee_ewf, ewf.data(), ewf.size() * sizeof(float), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(h->d_ee_f, ee->f, (size_t)nk * nb * 8, cudaMemcpyHostToDevice));
  CK(cudaMemset(h->d_ee_dm, 0, (size_t)nk * h->nb2 * 16));
  EeArgs& a = h->ee_args;
  memset(&a, 0, sizeof(a));
  a.nk = nk;
  a.npair = (int)h->npair;
  a.nbw = ee->nbw;
  for (int d = 0; d < 3; ++d) a.kmesh[d] = ee->kmesh[d];
  for (int i = 0; i < 9; ++i) a.GGT[i] = ee->GGT[i];
  a.ethr = ee->ethr;
  a.prefac_exp = -0.25 / std::pow(ee->degauss, 2);  // Lindblad (ElecElec_Model.h:33-34)
  a.prefac = 1. / (ee->degauss * std::sqrt(2. * M_PI)) / ee->nk_full;
  if (ee->antisymmetry) a.prefac *= 2;
  a.formula = ee->formula;
  a.antisym = ee->antisymmetry ? 1 : 0;
  a.kk = h->d_kkraw;
  a.kvec = h->d_ee_kvec;
  a.kidx = h->d_ee_kidx;
  a.kmap = h->d_ee_kmap;
  a.U = h->d_ee_U;
  a.ew = h->d_ew;
  a.ewf = h->d_ee_ewf;
  a.thr32 = (float)(ee->ethr + margin);
  a.scr = h->d_ee_scr;
  a.Pee = h->d_ee_Pee;
  // plasmon pole: eppa defaults to the plasma frequency of the set-up density (init_RPA,
  // Coulomb_Model.h:572-573), the smearing to 0.5 T except for Godby-Needs (:523)
  const double eppa = ee->eppa == 0 ? std::sqrt(4 * M_PI * ee->nfree / ee->meff / ee->eps_background) : ee->eppa;
  a.dynamic = ee->dynamic ? 1 : 0;
  a.two_freqs = ee->two_freqs ? 1 : 0;
  a.smearing = (ee->dynamic && ee->ppa_gn) ? ee->smearing : (ee->smearing <= 0 ? 0.5 * ee->temperature : ee->smearing);
  h->ee_eppa = eppa;
  h->ee_smear = a.smearing;
  h->ee_gn = ee->ppa_gn ? 1 : 0;
  h->ee_every = ee->every_rhs ? 1 : 0;
  h->ee_update = ee->update_screening ? 1 : 0;
  h->ee_nv = ee->nv;
  h->ee_scale = ee->scale;
  h->ee_nfree0 = ee->nfree;
  h->ee_nkfull = ee->nk_full;
  h->ee_cell = ee->cell_size;
  h->ee_eps = ee->eps_background;
  h->ee_T = ee->temperature;
  h->ee_meff = ee->meff;
  if (ee->formula == DMD_SCREEN_RPA) {  // the RPA table from the set-up occupations (+ plasmon-pole terms)
    double* qacc = nullptr;
    double* qacc1 = nullptr;  // Godby-Needs: the sums at i eppa
    unsigned int* qhit = nullptr;
    const bool gn = ee->dynamic && ee->ppa_gn;
    if ((rc = dalloc(h, &h->d_ee_vqtab, nmesh)) || (rc = dalloc(h, &qacc, nmesh)) || (rc = dalloc(h, &qhit, nmesh)) ||
        (gn && (rc = dalloc(h, &qacc1, 2 * nmesh))) ||
        (ee->dynamic && ((rc = dalloc(h, &h->d_ee_Aq, nmesh)) || (rc = dalloc(h, &h->d_ee_Eq2, nmesh))))) {
      cudaFree(qacc);
      cudaFree(qacc1);
      cudaFree(qhit);
      return rc;
    }
    a.vqtab = h->d_ee_vqtab;
    a.Aq = h->d_ee_Aq;
    a.Eq2 = h->d_ee_Eq2;
    cudaMemsetAsync(qacc, 0, nmesh * 8, h->st);
    cudaMemsetAsync(qhit, 0, nmesh * 4, h->st);
    if (qacc1) cudaMemsetAsync(qacc1, 0, 2 * nmesh * 8, h->st);
    const long long npp = (long long)nk * nk;
    if (nb == 2)
      k_ee_rpa_sum<2><<<blocks_for(npp, 256), 256, 0, h->st>>>(a, ee->temperature, h->d_ee_f, qacc, qhit, eppa, qacc1);
    else
      k_ee_rpa_sum<4><<<blocks_for(npp, 256), 256, 0, h->st>>>(a, ee->temperature, h->d_ee_f, qacc, qhit, eppa, qacc1);
    k_ee_rpa_table<<<blocks_for((long long)nmesh, 256), 256, 0, h->st>>>(
        a, 4 * M_PI / ee->eps_background / ee->cell_size, ee->nk_full, qacc, qhit, h->d_ee_vqtab, eppa, qacc1,
        h->d_ee_Aq, h->d_ee_Eq2);
    const cudaError_t e = cudaStreamSynchronize(h->st);
    cudaFree(qacc);
    cudaFree(qacc1);
    cudaFree(qhit);
    if (e != cudaSuccess) return fail(h, DMD_E_CUDA, std::string("RPA screening: ") + cudaGetErrorString(e));
    h->launches += 2;
  }
  h->ee_on = 1;
  if ((rc = ee_rebuild_nb(h, nullptr, time_value(h->t), true))) return rc;
  CK(cudaStreamSynchronize(h->st));
  drop_graphs(h);  // the captured step must include the update
  return DMD_OK;
}

int dmd_ee_update(dmd_handle* h) {
  if (!h) return DMD_E_ARG;
  if (!h->ee_on) return fail(h, DMD_E_STATE, "no e-e model attached");
  CK(cudaSetDevice(h->dev));
  int rc = ee_rebuild_nb(h, h->d_y, time_value(h->t), false);
  if (rc) return rc;
  CK(cudaStreamSynchronize(h->st));
  return DMD_OK;
}

}  // extern "C"

namespace {
// P_ee at the occupations d_f and P3..P6 of every pair (k_ee_p36), into d_p [4][npair][nb^4]
template <int NB>
int ee_linear_nb(dmd_handle* h, const double* d_f, double2* d_p) {
  constexpr int NB4 = NB * NB * NB * NB;
  EeArgs a = h->ee_args;
  a.dm = a.dm1 = nullptr;
  a.dmf = a.dm1f = nullptr;
  a.f = d_f;
  constexpr int WPC = ee_warps_per_cta(NB);
  const unsigned grid = (unsigned)((h->npair + WPC - 1) / WPC);
  if (h->prec == DMD_PREC_F64) {
    if (a.dynamic) k_ee_pairs<NB, EeF64, true><<<grid, 32 * WPC, 0, h->st>>>(a);
    else k_ee_pairs<NB, EeF64><<<grid, 32 * WPC, 0, h->st>>>(a);
  } else {
    if (a.dynamic) k_ee_pairs<NB, EeDF, true><<<grid, 32 * WPC, 0, h->st>>>(a);
    else k_ee_pairs<NB, EeDF><<<grid, 32 * WPC, 0, h->st>>>(a);
  }
  const size_t n = (size_t)h->npair * NB4;
  k_ee_p36<NB><<<(unsigned)h->npair, NB == 4 ? 256 : 32, 0, h->st>>>(a, d_f, d_p, d_p + n, d_p + 2 * n, d_p + 3 * n);
  h->launches += 2;
  CKL();
  return DMD_OK;
}
}  // namespace

extern "C" {

int dmd_ee_linear_terms(dmd_handle* h, const double* f_eq, double nfree, double* P1ee, double* P2ee, double* P3,
                        double* P4, double* P5, double* P6) {
  if (!h || !f_eq) return DMD_E_ARG;
  if (!h->ee_on) return fail(h, DMD_E_STATE, "no e-e model attached");
  if (h->ee_args.dynamic)
    return fail(h, DMD_E_ARG, "the linearized e-e terms are restated with static screening only");
  if (h->npair == 0) return DMD_OK;
  CK(cudaSetDevice(h->dev));
  const size_t nb4 = (size_t)h->nb4, np = (size_t)h->npair;
  double* d_f = nullptr;
  double2* d_p = nullptr;
  int rc;
  if ((rc = dalloc(h, &d_f, (size_t)h->nk * h->nb)) || (rc = dalloc(h, &d_p, 4 * np * nb4))) {
    cudaFree(d_f);
    return rc;
  }
  auto done = [&](int r) {
    cudaFree(d_f);
    cudaFree(d_p);
    return r;
  };
  if (cudaMemcpy(d_f, f_eq, (size_t)h->nk * h->nb * 8, cudaMemcpyHostToDevice) != cudaSuccess)
    return done(fail(h, DMD_E_CUDA, "dmd_ee_linear_terms: upload f"));
  // the screening constants of density nfree (coulomb_model::init(f_eq) when the model updates it)
  k_ee_screen<<<1, 256, 0, h->st>>>(h->nk, h->nb, h->ee_nv, nullptr, 0, nfree, h->ee_nkfull, h->ee_cell, h->ee_eps,
                                    h->ee_T, h->ee_meff, h->d_ee_scr);
  rc = h->nb == 2 ? ee_linear_nb<2>(h, d_f, d_p) : ee_linear_nb<4>(h, d_f, d_p);
  // the attach-time screening again
  k_ee_screen<<<1, 256, 0, h->st>>>(h->nk, h->nb, h->ee_nv, nullptr, 0, h->ee_nfree0, h->ee_nkfull, h->ee_cell,
                                    h->ee_eps, h->ee_T, h->ee_meff, h->d_ee_scr);
  if (rc) return done(rc);
  if (cudaStreamSynchronize(h->st) != cudaSuccess) return done(fail(h, DMD_E_CUDA, "dmd_ee_linear_terms"));
  std::vector<double2> buf(np * 2 * nb4);
  if (cudaMemcpy(buf.data(), h->d_ee_Pee, buf.size() * 16, cudaMemcpyDeviceToHost) != cudaSuccess)
    return done(fail(h, DMD_E_CUDA, "dmd_ee_linear_terms: read P_ee"));
  for (size_t p = 0; p < np; ++p) {
    if (P1ee) memcpy(P1ee + 2 * p * nb4, &buf[p * 2 * nb4], nb4 * 16);
    if (P2ee) memcpy(P2ee + 2 * p * nb4, &buf[(p * 2 + 1) * nb4], nb4 * 16);
  }
  double* outs[4] = {P3, P4, P5, P6};
  for (int m = 0; m < 4; ++m)
    if (outs[m] && cudaMemcpy(outs[m], d_p + m * np * nb4, np * nb4 * 16, cudaMemcpyDeviceToHost) != cudaSuccess)
      return done(fail(h, DMD_E_CUDA, "dmd_ee_linear_terms: read P3..P6"));
  return done(DMD_OK);
}

int dmd_ee_read(dmd_handle* h, double* P1ee, double* P2ee, double* nfree) {
  if (!h) return DMD_E_ARG;
  if (!h->ee_on) return fail(h, DMD_E_STATE, "no e-e model attached");
  CK(cudaSetDevice(h->dev));
  CK(cudaStreamSynchronize(h->st));
  const size_t nb4 = (size_t)h->nb4, np = (size_t)h->npair;
  if (P1ee || P2ee) {
    std::vector<double2> buf(np * 2 * nb4);
    CK(cudaMemcpy(buf.data(), h->d_ee_Pee, buf.size() * 16, cudaMemcpyDeviceToHost));
    for (size_t p = 0; p < np; ++p)
      for (int m = 0; m < 2; ++m) {
        double* o = m == 0 ? P1ee : P2ee;
        if (!o) continue;
        memcpy(o + 2 * p * nb4, &buf[(p * 2 + m) * nb4], nb4 * 16);
      }
  }
  if (nfree) {
    EeScreen c;
    CK(cudaMemcpy(&c, h->d_ee_scr, sizeof(c), cudaMemcpyDeviceToHost));
    *nfree = c.nfree;
  }
  return DMD_OK;
}

int dmd_profile_get(const dmd_handle* h, int cls, double* total_ms, int64_t* n) {
  if (!h || cls < 0 || cls > 4) return DMD_E_ARG;
  if (total_ms) *total_ms = h->prof_ms[cls];
  if (n) *n = h->prof_n[cls];
  return DMD_OK;
}

}  // extern "C"
