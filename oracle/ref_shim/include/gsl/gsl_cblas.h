/* CBLAS subset used by the reference DMD sources (comm/mymatrix.cpp:73-86: cblas_zgemm and
 * cblas_zhemm, row-major). Oracle build infrastructure only; the definitions live in
 * oracle/ref_shim/cblas_shim.c and follow the BLAS Level-3 definitions
 * C = alpha*op(A)*op(B) + beta*C and C = alpha*A*B + beta*C (A Hermitian, one triangle read). */
#ifndef ORACLE_SHIM_GSL_CBLAS_H
#define ORACLE_SHIM_GSL_CBLAS_H
#include <stddef.h>
#ifdef __cplusplus
extern "C" {
#endif
enum CBLAS_ORDER { CblasRowMajor = 101, CblasColMajor = 102 };
enum CBLAS_TRANSPOSE { CblasNoTrans = 111, CblasTrans = 112, CblasConjTrans = 113 };
enum CBLAS_UPLO { CblasUpper = 121, CblasLower = 122 };
enum CBLAS_DIAG { CblasNonUnit = 131, CblasUnit = 132 };
enum CBLAS_SIDE { CblasLeft = 141, CblasRight = 142 };
typedef enum CBLAS_ORDER CBLAS_ORDER;
typedef enum CBLAS_TRANSPOSE CBLAS_TRANSPOSE;
typedef enum CBLAS_UPLO CBLAS_UPLO;
typedef enum CBLAS_DIAG CBLAS_DIAG;
typedef enum CBLAS_SIDE CBLAS_SIDE;

void cblas_zgemm(enum CBLAS_ORDER Order, enum CBLAS_TRANSPOSE TransA, enum CBLAS_TRANSPOSE TransB,
                 int M, int N, int K, const void* alpha, const void* A, int lda, const void* B, int ldb,
                 const void* beta, void* C, int ldc);
void cblas_zhemm(enum CBLAS_ORDER Order, enum CBLAS_SIDE Side, enum CBLAS_UPLO Uplo, int M, int N,
                 const void* alpha, const void* A, int lda, const void* B, int ldb, const void* beta,
                 void* C, int ldc);
#ifdef __cplusplus
}
#endif
#endif
