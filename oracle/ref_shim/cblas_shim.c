/* Reference-semantics complex BLAS used by the oracle (test infrastructure only).
 *
 * cblas_zgemm : C = alpha*op(A)*op(B) + beta*C
 * cblas_zhemm : C = alpha*A*B + beta*C (Left) or alpha*B*A + beta*C (Right), A Hermitian and
 *               only the triangle named by Uplo is read; the imaginary parts of A's diagonal are
 *               taken as zero (BLAS Level-3 definition of ZHEMM).
 *
 * The reference calls these through comm/mymatrix.cpp:73-86 (row-major). Each output element is
 * a dot product accumulated from zero in increasing inner index, then scaled; the oracle's own
 * restatement calls the same two functions, so the shim-built reference and the restatement agree
 * bit for bit. Compile with -ffp-contract=off so the order of rounding is the same on every host.
 */
#include <stdlib.h>
#include <stdio.h>
#include "gsl/gsl_cblas.h"

typedef struct { double x, y; } zc;

static inline zc zmul(zc a, zc b) { zc r; r.x = a.x * b.x - a.y * b.y; r.y = a.x * b.y + a.y * b.x; return r; }
static inline zc zadd(zc a, zc b) { zc r; r.x = a.x + b.x; r.y = a.y + b.y; return r; }
static inline zc zconj(zc a) { a.y = -a.y; return a; }

static inline zc elem(const zc* M, int ld, int i, int j, int rowmajor) {
  return rowmajor ? M[(size_t)i * ld + j] : M[(size_t)j * ld + i];
}

static inline zc op_elem(const zc* M, int ld, int i, int j, enum CBLAS_TRANSPOSE t, int rowmajor) {
  if (t == CblasNoTrans) return elem(M, ld, i, j, rowmajor);
  zc v = elem(M, ld, j, i, rowmajor);
  return t == CblasConjTrans ? zconj(v) : v;
}

void cblas_zgemm(enum CBLAS_ORDER Order, enum CBLAS_TRANSPOSE TransA, enum CBLAS_TRANSPOSE TransB,
                 int M, int N, int K, const void* alpha, const void* A, int lda, const void* B, int ldb,
                 const void* beta, void* C, int ldc) {
  const zc al = *(const zc*)alpha, be = *(const zc*)beta;
  const zc *a = (const zc*)A, *b = (const zc*)B;
  zc* c = (zc*)C;
  int rm = Order == CblasRowMajor;
  for (int i = 0; i < M; ++i)
    for (int j = 0; j < N; ++j) {
      zc s = {0.0, 0.0};
      for (int l = 0; l < K; ++l) s = zadd(s, zmul(op_elem(a, lda, i, l, TransA, rm), op_elem(b, ldb, l, j, TransB, rm)));
      zc* cij = rm ? &c[(size_t)i * ldc + j] : &c[(size_t)j * ldc + i];
      if (be.x == 0.0 && be.y == 0.0) *cij = zmul(al, s);
      else *cij = zadd(zmul(al, s), zmul(be, *cij));
    }
}

static inline zc herm_elem(const zc* A, int lda, int i, int l, enum CBLAS_UPLO uplo, int rm) {
  if (i == l) { zc d = elem(A, lda, i, i, rm); d.y = 0.0; return d; }
  int stored = (uplo == CblasUpper) ? (i < l) : (i > l);
  return stored ? elem(A, lda, i, l, rm) : zconj(elem(A, lda, l, i, rm));
}

void cblas_zhemm(enum CBLAS_ORDER Order, enum CBLAS_SIDE Side, enum CBLAS_UPLO Uplo, int M, int N,
                 const void* alpha, const void* A, int lda, const void* B, int ldb, const void* beta,
                 void* C, int ldc) {
  const zc al = *(const zc*)alpha, be = *(const zc*)beta;
  const zc *a = (const zc*)A, *b = (const zc*)B;
  zc* c = (zc*)C;
  int rm = Order == CblasRowMajor;
  for (int i = 0; i < M; ++i)
    for (int j = 0; j < N; ++j) {
      zc s = {0.0, 0.0};
      if (Side == CblasLeft)
        for (int l = 0; l < M; ++l) s = zadd(s, zmul(herm_elem(a, lda, i, l, Uplo, rm), elem(b, ldb, l, j, rm)));
      else
        for (int l = 0; l < N; ++l) s = zadd(s, zmul(elem(b, ldb, i, l, rm), herm_elem(a, lda, l, j, Uplo, rm)));
      zc* cij = rm ? &c[(size_t)i * ldc + j] : &c[(size_t)j * ldc + i];
      if (be.x == 0.0 && be.y == 0.0) *cij = zmul(al, s);
      else *cij = zadd(zmul(al, s), zmul(be, *cij));
    }
}
