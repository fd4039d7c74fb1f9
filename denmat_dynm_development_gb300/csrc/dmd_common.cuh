// Shared device helpers for the Lindblad RHS kernels (sm_103a).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#define DMD_MAX_NBDM 8

struct cplx {
  double x, y;
};

__host__ __device__ __forceinline__ double2 mk2(double x, double y) { double2 r; r.x = x; r.y = y; return r; }

// Complex arithmetic written with explicit round-to-nearest intrinsics where the reference's operation
// order matters (no FMA contraction), so state updates round exactly like the FP64 CPU code.
__device__ __forceinline__ double2 cmul_rn(double2 a, double2 b) {
  return mk2(__dsub_rn(__dmul_rn(a.x, b.x), __dmul_rn(a.y, b.y)), __dadd_rn(__dmul_rn(a.x, b.y), __dmul_rn(a.y, b.x)));
}
__device__ __forceinline__ double2 cadd_rn(double2 a, double2 b) { return mk2(__dadd_rn(a.x, b.x), __dadd_rn(a.y, b.y)); }
__device__ __forceinline__ double2 csub_rn(double2 a, double2 b) { return mk2(__dsub_rn(a.x, b.x), __dsub_rn(a.y, b.y)); }
__device__ __forceinline__ double2 cscale_rn(double s, double2 a) { return mk2(__dmul_rn(a.x, s), __dmul_rn(a.y, s)); }
__device__ __forceinline__ double2 cconj(double2 a) { return mk2(a.x, -a.y); }

// fused forms for the bandwidth kernels
__device__ __forceinline__ double2 cfma(double2 a, double2 b, double2 c) {  // c + a*b
  return mk2(fma(a.x, b.x, fma(-a.y, b.y, c.x)), fma(a.x, b.y, fma(a.y, b.x, c.y)));
}
__device__ __forceinline__ double2 cfma_conja(double2 a, double2 b, double2 c) {  // c + conj(a)*b
  return mk2(fma(a.x, b.x, fma(a.y, b.y, c.x)), fma(a.x, b.y, fma(-a.y, b.x, c.y)));
}

__device__ __forceinline__ double2 ccis(double x) {
  double s, c;
  sincos(x, &s, &c);
  return mk2(c, s);
}
