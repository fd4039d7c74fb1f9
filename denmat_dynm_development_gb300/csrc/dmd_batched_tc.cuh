// Batched form of the k-pair contraction on the tensor cores (tcgen05), nb = 2.
//
// With many states sharing P the contraction is a GEMM. Every stored pair (k1, k2) is kept twice, as
// directed operators (row <- column): (k1 <- k2) with A = Q1, B = Q2 and, when the pair carries the
// reverse term, (k2 <- k1) with A = conj(Q2), B = conj(Q1) (Q1, Q2: the Hermitian-coordinate
// operators of dmd_pairs_cb.cuh). Then for every row k
//   X'_k[a] = sum_c sum_j A_kc[a][j] r_c[j],      Y'_k[j] = sum_c sum_a B_kc[a][j] s_c[a]
// and no reverse sums remain. Rows (energy-rank positions) are grouped in tiles of TR = 16, columns
// in groups of CG = 8; a tile's operators over one column group form a dense block (zeros where a
// row and a column have no pair; rows of an energy window pair with nearly the same columns, so the
// blocks are nearly full). For a tile and up to 128 states one CTA computes
//   D_X[q][(r, a, re|im)] = sum_(c, j) R[q][(c, j)] * BX[(c, j)][(r, a, re|im)]
//   D_Y[q][(r, j, re|im)] = sum_(c, a) S[q][(c, a)] * BY[(c, a)][(r, j, re|im)]
// (M = 128 states, N = 16 rows x 4 x 2 = 128, K = 8 columns x 4 = 32 per group) as tcgen05 MMAs
// accumulating in tensor memory over all of the tile's column groups, then writes each row's sums
// once: no atomics. Operands are bf16 hi + lo splits (x = hi + lo, 16 significant bits); the
// product keeps hi*hi + hi*lo + lo*hi. Operand blocks are laid out in HBM exactly as the MMA reads
// them (K-major, no swizzle: core matrices of 8 rows x 16 B), so one bulk copy per block fills a
// pipeline stage: thread 0 produces, thread 32 issues MMAs, all four warps read TMEM at the end.
#pragma once
#include <cuda_bf16.h>

#include "dmd_common.cuh"
#include "dmd_tc.cuh"
#include "dmd_tma.cuh"

namespace dmd {

struct TcTile {
  int32_t g0, g1;  // column groups [g0, g1)
  int64_t boff;    // index of the tile's first operator block
};

constexpr int TC_TR = 16, TC_CG = 8, TC_K = 32, TC_N = 128, TC_M = 128;
constexpr int TC_PLANE = 4096;                     // bf16 per plane (128 x 32)
constexpr int TC_BLOCK = 4 * TC_PLANE;             // bf16 per block: 4 planes
constexpr uint32_t TC_BLOCK_BYTES = 2 * TC_BLOCK;  // 32 KB
constexpr int TC_NST = 3;                          // pipeline stages of (coordinate block, operator block)

// element (row, kk) of a 128 x 32 K-major plane: core matrices [row / 8][kk / 8] of 8 x 8
__host__ __device__ __forceinline__ int tc_ci(int row, int kk) {
  return (((row >> 3) * 4 + (kk >> 3)) << 6) + ((row & 7) << 3) + (kk & 7);
}

// coordinates (FP32, [part][q][pos][2 NB2] as written by k_prep_herm) -> coordinate blocks
// [part][group][mblock][r_hi, r_lo, s_hi, s_lo][128 x 32]; entries of padding states stay zero.
// Part 1 (anti-Hermitian) is packed only when *gate is set.
__global__ void k_pack_tc(int nk, int nrhs, int ngroups, int nmb, const float* __restrict__ rs,
                          uint16_t* __restrict__ A, const unsigned int* __restrict__ gate) {
  const size_t idx = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  const int part = blockIdx.y;
  if (part == 1 && *gate == 0u) return;
  const size_t per = (size_t)nrhs * nk * 8;
  if (idx >= per) return;
  const int e = (int)(idx % 8), p = (int)((idx / 8) % nk), q = (int)(idx / ((size_t)8 * nk));
  const float v = rs[(size_t)part * per + idx];
  const __nv_bfloat16 hi = __float2bfloat16_rn(v);
  const __nv_bfloat16 lo = __float2bfloat16_rn(__fsub_rn(v, __bfloat162float(hi)));
  const int g = p / TC_CG, kk = (p % TC_CG) * 4 + (e & 3), mb = q / TC_M, m = q % TC_M;
  uint16_t* blk = A + (((size_t)part * ngroups + g) * nmb + mb) * TC_BLOCK + (e < 4 ? 0 : 2 * TC_PLANE);
  blk[tc_ci(m, kk)] = __bfloat16_as_ushort(hi);
  blk[TC_PLANE + tc_ci(m, kk)] = __bfloat16_as_ushort(lo);
}

// IMAG: the anti-Hermitian pass (sums times i, added); otherwise acc = acc0 + sums (stored)
template <bool IMAG>
__global__ void __launch_bounds__(128, 1) k_pairs_tc(const TcTile* __restrict__ tiles, int ntiles,
                                                     const uint16_t* __restrict__ B, const uint16_t* __restrict__ A,
                                                     int nmb, int nrhs, int nk, const double2* __restrict__ acc0,
                                                     double2* __restrict__ acc, size_t astride,
                                                     const unsigned int* __restrict__ gate,
                                                     unsigned int* __restrict__ errflag) {
  extern __shared__ __align__(1024) unsigned char smem[];
  if (gate && *gate == 0u) return;
  // the CTAs of one tile (all state blocks) are adjacent, so its operator blocks are read from HBM once
  const int t = blockIdx.x / nmb, mb = blockIdx.x % nmb;
  if (t >= ntiles) return;
  const TcTile tile = tiles[t];
  const int nch = tile.g1 - tile.g0;
  uint64_t* full = (uint64_t*)(smem + TC_NST * 2 * TC_BLOCK_BYTES);
  uint64_t* empty = full + TC_NST;
  uint64_t* done = empty + TC_NST;
  uint32_t* tslot = (uint32_t*)(done + 1);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (threadIdx.x == 0) {
    for (int s = 0; s < TC_NST; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    mbar_init(done, 1);
    fence_mbar_init();
  }
  if (warp == 0) {
    tc_alloc(tslot, 256);  // D_X in columns [0, 128), D_Y in [128, 256)
    tc_relinquish();
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tslot;
  if (nch > 0) {
    int issued = 0;
    if (threadIdx.x == 0) {  // producer: coordinate block + operator block per column group
      const uint64_t pol_a = policy_evict_last(), pol_b = policy_evict_first();
      for (int i = 0; i < nch; ++i) {
        const int s = i % TC_NST;
        if (i >= TC_NST && !mbar_wait_bounded(&empty[s], (uint32_t)((i / TC_NST - 1) & 1), errflag)) break;
        unsigned char* st = smem + (size_t)s * 2 * TC_BLOCK_BYTES;
        mbar_arrive_expect_tx(&full[s], 2 * TC_BLOCK_BYTES);
        bulk_g2s(st, A + ((size_t)(tile.g0 + i) * nmb + mb) * TC_BLOCK, TC_BLOCK_BYTES, &full[s], pol_a);
        bulk_g2s(st + TC_BLOCK_BYTES, B + (size_t)(tile.boff + i) * TC_BLOCK, TC_BLOCK_BYTES, &full[s], pol_b);
        ++issued;
      }
    } else if (threadIdx.x == 32) {  // MMA issuer
      constexpr uint32_t idesc = tc_idesc_bf16(TC_M, TC_N);
      constexpr uint32_t LBO = 128, SBO = 512, PL = 2 * TC_PLANE;  // bytes: K-adjacent, M/N-adjacent core matrices; plane
      for (int i = 0; i < nch; ++i) {
        const int s = i % TC_NST;
        if (!mbar_wait_bounded(&full[s], (uint32_t)((i / TC_NST) & 1), errflag)) break;
        tc_fence_after();
        const uint32_t a0 = smem_u32(smem + (size_t)s * 2 * TC_BLOCK_BYTES), b0 = a0 + TC_BLOCK_BYTES;
#pragma unroll
        for (int ks = 0; ks < 2; ++ks) {  // K = 32 as two MMAs of K = 16 (two core matrices apart)
          const uint32_t ko = ks * 2 * LBO;
          const uint32_t accum = (i | ks) != 0;  // the tile's first MMA overwrites the accumulator
          // X: R x BX (planes r_hi, r_lo / x_hi, x_lo)
          tc_mma(tmem, tc_desc(a0 + ko, LBO, SBO), tc_desc(b0 + ko, LBO, SBO), idesc, accum);
          tc_mma(tmem, tc_desc(a0 + ko, LBO, SBO), tc_desc(b0 + PL + ko, LBO, SBO), idesc, 1);
          tc_mma(tmem, tc_desc(a0 + PL + ko, LBO, SBO), tc_desc(b0 + ko, LBO, SBO), idesc, 1);
          // Y: S x BY (planes s_hi, s_lo / y_hi, y_lo)
          tc_mma(tmem + 128, tc_desc(a0 + 2 * PL + ko, LBO, SBO), tc_desc(b0 + 2 * PL + ko, LBO, SBO), idesc, accum);
          tc_mma(tmem + 128, tc_desc(a0 + 2 * PL + ko, LBO, SBO), tc_desc(b0 + 3 * PL + ko, LBO, SBO), idesc, 1);
          tc_mma(tmem + 128, tc_desc(a0 + 3 * PL + ko, LBO, SBO), tc_desc(b0 + 2 * PL + ko, LBO, SBO), idesc, 1);
        }
        tc_commit(&empty[s]);  // the stage is free once these MMAs have read it
      }
      tc_commit(done);  // arrives when every MMA issued above has completed (also after a failure)
    }
    // all MMAs complete before TMEM is read (bounded; a timeout sets the flag)
    mbar_wait_bounded(done, 0, errflag);
    if (threadIdx.x == 0)  // no bulk copy into this CTA's shared memory outlives it (all done unless a wait gave up)
      for (int j = issued > TC_NST ? issued - TC_NST : 0; j < issued; ++j)
        mbar_wait_bounded(&full[j % TC_NST], (uint32_t)((j / TC_NST) & 1), errflag);
  }
  __syncwarp();  // the producer and issuer lanes rejoin their warps before the warp-wide TMEM loads
  tc_fence_after();
  // epilogue: thread (warp w, lane l) owns state q = 128 mb + 32 w + l = TMEM lane 32 w + l
  const int q = mb * TC_M + warp * 32 + lane;
  const uint32_t lane_addr = tmem + ((uint32_t)(warp * 32) << 16);
  for (int cb = 0; cb < 8; ++cb) {  // 8 x 32 columns: D_X then D_Y
    float v[32];
    if (nch > 0) {
      tc_ld32(lane_addr + cb * 32, v);
    } else {
#pragma unroll
      for (int i = 0; i < 32; ++i) v[i] = 0.f;
    }
    if (q >= nrhs) continue;
    // columns cb*32 .. cb*32+31 = 4 rows x (4 elements x re|im) of X' (cb < 4) or Y' (cb >= 4)
    const int half = cb >> 2;  // 0: X', 1: Y'
#pragma unroll
    for (int rr = 0; rr < 4; ++rr) {
      const int r = (cb & 3) * 4 + rr, p = t * TC_TR + r;
      if (p >= nk) continue;
      double2* dst = acc + (size_t)q * astride + (size_t)p * 8 + half * 4;
#pragma unroll
      for (int a = 0; a < 4; ++a) {
        const double re = v[rr * 8 + 2 * a], im = v[rr * 8 + 2 * a + 1];
        if (IMAG) {
          const double2 o = dst[a];
          dst[a] = mk2(o.x - im, o.y + re);
        } else {
          const double2 c = acc0 ? acc0[(size_t)p * 8 + half * 4 + a] : mk2(0.0, 0.0);
          dst[a] = mk2(c.x + re, c.y + im);
        }
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) tc_dealloc(tmem, 256);
}

}  // namespace dmd
