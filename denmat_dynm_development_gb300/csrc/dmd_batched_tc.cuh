// Batched form of the k-pair contraction on the tensor cores (tcgen05), nb = 2 and nb = 4.
//
// With many states sharing P the contraction is a GEMM. Every stored pair (k1, k2) is kept twice, as
// directed operators (row <- column): (k1 <- k2) with A = Q1, B = Q2 and, when the pair carries the
// reverse term, (k2 <- k1) with A = conj(Q2), B = conj(Q1) (Q1, Q2: the Hermitian-coordinate
// operators of dmd_pairs_cb.cuh). Then for every row k
//   X'_k[a] = sum_c sum_j A_kc[a][j] r_c[j],      Y'_k[j] = sum_c sum_a B_kc[a][j] s_c[a]
// and no reverse sums remain. The batched form runs in the deviation form, where s = -r (or s = 0 in
// the linearized form), so both sums contract the same coordinates: Y'_k[j] = -sum B_kc[a][j] r_c[a].
// Rows (energy-rank positions) are grouped in tiles of TR = 64 / nb^2 (16 for nb = 2, 4 for nb = 4),
// columns in groups of CG = 32 / nb^2 (8, 2); a tile's operators over one column group form a dense
// block (zeros where a row and a column have no pair; rows of an energy window pair with nearly the
// same columns, so the blocks are nearly full). For a tile and up to 128 states one CTA computes
//   D[q][n] = sum_(c, j) R[q][(c, j)] * B[(c, j)][n],  n < 128: (r, a, re|im) of X', n >= 128: (r, j, re|im) of -Y'
// (M = 128 states, N = 256, K = CG columns x nb^2 = 32 per group) as tcgen05 MMAs accumulating in tensor
// memory over all of the tile's column groups, then writes each row's sums once (FP32, as the
// tensor memory holds them): no atomics.
// Operands are bf16 hi + lo splits (x = hi + lo, 16 significant bits); the product keeps
// hi*hi + hi*lo + lo*hi. Every operand row holds [hi (32) | lo (32)] = 128 bytes, so a tile is a
// 128-byte-swizzled K-major tile and the three products are MMAs over K slices paired through
// descriptor offsets (hi: +0, +32 B; lo: +64, +96 B). Operand blocks are laid out in HBM exactly as
// the MMA reads them (swizzle included), so two bulk copies fill a pipeline stage. Warp 0 (one lane)
// produces, warp 1 (one lane) issues MMAs, the other lanes of both warps park at __syncwarp (a lane
// polling an mbarrier would hold up the working lane of its warp), and all four warps write the sums
// through shared memory in 512-byte rows.
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

constexpr int TC_K = 32, TC_N = 128, TC_M = 128;
// rows per tile and columns per group for nb2 = nb^2 coordinates per k-point
__host__ __device__ constexpr int tc_tr(int nb2) { return 64 / nb2; }
__host__ __device__ constexpr int tc_cg(int nb2) { return 32 / nb2; }
constexpr int TC_PLANE = 8192;                     // bf16 per 128-row tile (128 rows x [hi 32 | lo 32])
constexpr int TC_BLOCK = 2 * TC_PLANE;             // bf16 per operator block: X rows, then Y rows (256)
constexpr int TC_ABLOCK = TC_PLANE;                // bf16 per coordinate block: R (128 states)
constexpr uint32_t TC_BLOCK_BYTES = 2 * TC_BLOCK;  // 32 KB
constexpr uint32_t TC_ABLOCK_BYTES = 2 * TC_ABLOCK;  // 16 KB
constexpr uint32_t TC_STAGE_BYTES = TC_ABLOCK_BYTES + TC_BLOCK_BYTES;
constexpr int TC_NST = 4;                          // pipeline stages of (coordinate block, operator block)
// dynamic shared memory of a CTA with nst stages (2 stages leave room for 2 CTAs per SM)
__host__ __device__ constexpr size_t tc_smem_bytes(int nst) { return (size_t)nst * TC_STAGE_BYTES + 1024 + 128; }
constexpr size_t TC_SMEM_BYTES = tc_smem_bytes(TC_NST);

// element (row, kk) of a tile: kk < 32 the hi part, kk + 32 the lo part of K index kk
__host__ __device__ __forceinline__ int tc_ci(int row, int kk) { return tc_sw128(row, kk); }

// r coordinates (FP32, [part][q][pos][2 NB2] as written by k_prep_herm, the first NB2 of each 2 NB2)
// -> coordinate blocks [part][group][mblock][128 x (hi 32 | lo 32)]; entries of padding states stay
// zero. Part 1 (anti-Hermitian) is packed only when *gate is set.
template <int NB>
__global__ void k_pack_tc(int nk, int nrhs, int ngroups, int nmb, const float* __restrict__ rs,
                          uint16_t* __restrict__ A, const unsigned int* __restrict__ gate) {
  constexpr int NB2 = NB * NB, CG = tc_cg(NB2);
  const size_t idx = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  const int part = blockIdx.y;
  if (part == 1 && *gate == 0u) return;
  const size_t per = (size_t)nrhs * nk * NB2;
  if (idx >= per) return;
  const int e = (int)(idx % NB2), p = (int)((idx / NB2) % nk), q = (int)(idx / ((size_t)NB2 * nk));
  const float v = rs[(size_t)part * 2 * per + ((size_t)q * nk + p) * 2 * NB2 + e];
  const __nv_bfloat16 hi = __float2bfloat16_rn(v);
  const __nv_bfloat16 lo = __float2bfloat16_rn(__fsub_rn(v, __bfloat162float(hi)));
  const int g = p / CG, kk = (p % CG) * NB2 + e, mb = q / TC_M, m = q % TC_M;
  uint16_t* blk = A + (((size_t)part * ngroups + g) * nmb + mb) * TC_ABLOCK;
  blk[tc_ci(m, kk)] = __bfloat16_as_ushort(hi);
  blk[tc_ci(m, kk + 32)] = __bfloat16_as_ushort(lo);
}

// IMAG: the anti-Hermitian pass (sums times i, added); otherwise acc = sums (stored). acc is FP32,
// [state][position][X' (NB2) | Y' (NB2)], astride float2 per state. ysign: -1 (Y' = -D_Y, s = -r) or 0
// (linearized form, s = 0).
template <bool IMAG, int NST = TC_NST, int NB = 2>
__global__ void __launch_bounds__(128, 1) k_pairs_tc(const TcTile* __restrict__ tiles, int ntiles,
                                                     const uint16_t* __restrict__ B, const uint16_t* __restrict__ A,
                                                     int nmb, int nrhs, int nk, float2* __restrict__ acc,
                                                     size_t astride, float ysign,
                                                     const unsigned int* __restrict__ gate,
                                                     unsigned int* __restrict__ errflag) {
  extern __shared__ __align__(128) unsigned char smem_raw[];
  if (gate && *gate == 0u) return;
  // swizzled operand tiles start on 1024-byte boundaries (1 KB of slack is allocated)
  unsigned char* smem = smem_raw + ((1024u - (smem_u32(smem_raw) & 1023u)) & 1023u);
  // the CTAs of one tile (all state blocks) are adjacent, so its operator blocks are read from HBM once
  const int t = blockIdx.x / nmb, mb = blockIdx.x % nmb;
  if (t >= ntiles) return;
  const TcTile tile = tiles[t];
  const int nch = tile.g1 - tile.g0;
  uint64_t* full = (uint64_t*)(smem + NST * TC_STAGE_BYTES);
  uint64_t* empty = full + NST;
  uint64_t* done = empty + NST;
  uint32_t* tslot = (uint32_t*)(done + 1);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (threadIdx.x == 0) {
    for (int s = 0; s < NST; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    mbar_init(done, 1);
    fence_mbar_init();
  }
  if (warp == 0) {
    tc_alloc(tslot, 256);  // D: X' in columns [0, 128), -Y' in [128, 256)
    tc_relinquish();
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tslot;
  if (nch > 0) {
    if (warp == 0) {
      if (lane == 0) {  // producer: coordinate block + operator block per column group
        const uint64_t pol_a = policy_evict_last(), pol_b = policy_evict_first();
        int issued = 0;
        for (int i = 0; i < nch; ++i) {
          const int s = i % NST;
          if (i >= NST && !mbar_wait_bounded(&empty[s], (uint32_t)((i / NST - 1) & 1), errflag)) break;
          unsigned char* st = smem + (size_t)s * TC_STAGE_BYTES;
          mbar_arrive_expect_tx(&full[s], TC_STAGE_BYTES);
          bulk_g2s(st, A + ((size_t)(tile.g0 + i) * nmb + mb) * TC_ABLOCK, TC_ABLOCK_BYTES, &full[s], pol_a);
          bulk_g2s(st + TC_ABLOCK_BYTES, B + (size_t)(tile.boff + i) * TC_BLOCK, TC_BLOCK_BYTES, &full[s], pol_b);
          ++issued;
        }
        mbar_wait_bounded(done, 0, errflag);
        // no bulk copy into this CTA's shared memory outlives it (all landed unless a wait gave up)
        for (int j = issued > NST ? issued - NST : 0; j < issued; ++j)
          mbar_wait_bounded(&full[j % NST], (uint32_t)((j / NST) & 1), errflag);
      }
      __syncwarp();
    } else if (warp == 1) {
      if (lane == 0) {  // MMA issuer
        constexpr uint32_t idesc = tc_idesc_bf16(TC_M, 2 * TC_N);
        constexpr uint32_t SBO = 1024, LO = 64;  // bytes: 8-row atoms; hi -> lo slice of a row
        for (int i = 0; i < nch; ++i) {
          const int s = i % NST;
          if (!mbar_wait_bounded(&full[s], (uint32_t)((i / NST) & 1), errflag)) break;
          tc_fence_after();
          const uint32_t a0 = smem_u32(smem + (size_t)s * TC_STAGE_BYTES), b0 = a0 + TC_ABLOCK_BYTES;
#pragma unroll
          for (int ks = 0; ks < 2; ++ks) {  // K = 32 as two MMAs of K = 16 (32 bytes of the row apart)
            const uint32_t ko = ks * 32;
            const uint32_t accum = (i | ks) != 0;  // the tile's first MMA overwrites the accumulator
            tc_mma(tmem, tc_desc_sw128(a0 + ko, SBO), tc_desc_sw128(b0 + ko, SBO), idesc, accum);  // hi x hi
            tc_mma(tmem, tc_desc_sw128(a0 + LO + ko, SBO), tc_desc_sw128(b0 + ko, SBO), idesc, 1);  // lo x hi
            tc_mma(tmem, tc_desc_sw128(a0 + ko, SBO), tc_desc_sw128(b0 + LO + ko, SBO), idesc, 1);  // hi x lo
          }
          tc_commit(&empty[s]);  // the stage is free once these MMAs have read it
        }
        tc_commit(done);  // arrives when every MMA issued above has completed (also after a failure)
      }
      __syncwarp();
    }
    // all MMAs complete before TMEM is read (bounded; a timeout sets the flag)
    mbar_wait_bounded(done, 0, errflag);
  }
  tc_fence_after();
  // epilogue: TMEM lane 32 w + l holds state q = 128 mb + 32 w + l. 32 TMEM columns hold RPC rows of
  // the tile (4 for nb = 2, 1 for nb = 4) x NB2 elements x (re, im); per such chunk a thread writes its
  // state's RPC x 2 NB2 sums into shared memory (a row of 33 float2 per state), then the warp stores
  // each state's 256 contiguous bytes with one coalesced instruction.
  constexpr int NB2 = NB * NB, RPC = 16 / NB2, TR = tc_tr(NB2);
  float2* wsm = (float2*)smem + (size_t)warp * 32 * 33;
  const int qb = mb * TC_M + warp * 32;
  const uint32_t lane_addr = tmem + ((uint32_t)(warp * 32) << 16);
  for (int rq = 0; rq < 4; ++rq) {
    float vx[32], vy[32];
    if (nch > 0) {
      tc_ld32(lane_addr + rq * 32, vx);
      tc_ld32(lane_addr + 128 + rq * 32, vy);
    } else {
#pragma unroll
      for (int i = 0; i < 32; ++i) vx[i] = vy[i] = 0.f;
    }
    float2* my = wsm + lane * 33;
#pragma unroll
    for (int rr = 0; rr < RPC; ++rr)
#pragma unroll
      for (int a = 0; a < NB2; ++a) {
        my[rr * 2 * NB2 + a] = make_float2(vx[rr * 2 * NB2 + 2 * a], vx[rr * 2 * NB2 + 2 * a + 1]);
        my[rr * 2 * NB2 + NB2 + a] =
            make_float2(ysign * vy[rr * 2 * NB2 + 2 * a], ysign * vy[rr * 2 * NB2 + 2 * a + 1]);
      }
    __syncwarp();
    // lane l covers row p0 + l / (2 NB2), element l % (2 NB2) of every state of the warp
    const int p = t * TR + rq * RPC + lane / (2 * NB2);
    if (p < nk) {
      for (int j = 0; j < 32 && qb + j < nrhs; ++j) {
        const float2 v = wsm[j * 33 + lane];
        float2* dst = acc + (size_t)(qb + j) * astride + (size_t)p * 2 * NB2 + lane % (2 * NB2);
        if (IMAG) {
          const float2 o = *dst;
          *dst = make_float2(o.x - v.y, o.y + v.x);
        } else {
          *dst = v;
        }
      }
    }
    __syncwarp();
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) tc_dealloc(tmem, 256);
}

}  // namespace dmd
