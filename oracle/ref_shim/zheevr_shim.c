/* Hermitian eigensolver standing in for LAPACK zheevr_ in the oracle build (test
 * infrastructure only). The reference calls it through diagonalize() (comm/mymatrix.cpp:5-36)
 * for small band blocks: the observable "entropy_bloch" (observable.h:241) and the b^2 spin-mixing
 * diagnostics. None of them feed the right-hand side.
 *
 * Method: cyclic complex Jacobi rotations. For each off-diagonal h_pq = r e^{i phi} the unitary
 * U = diag(1, e^{-i phi}) * [[c, s], [-s, c]] zeroes h_pq, with t = sgn(th)/(|th| + sqrt(th^2+1)),
 * th = (h_qq - h_pp)/(2r), c = 1/sqrt(1+t^2), s = t c (Jacobi's method for symmetric matrices
 * applied after removing the phase). Eigenvalues are returned in ascending order with their
 * column-major eigenvectors, as JOBZ='V', RANGE='A' asks.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

typedef struct { double x, y; } zc;
static inline zc zm(zc a, zc b) { zc r = {a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x}; return r; }
static inline zc za(zc a, zc b) { zc r = {a.x + b.x, a.y + b.y}; return r; }
static inline zc zj(zc a) { a.y = -a.y; return a; }

void zheevr_(char* jobz, char* range, char* uplo, int* N, zc* A, int* lda, double* vl, double* vu, int* il, int* iu,
             double* abstol, int* M, double* W, zc* Z, int* ldz, int* isuppz, zc* work, int* lwork, double* rwork,
             int* lrwork, int* iwork, int* liwork, int* info) {
  (void)range; (void)vl; (void)vu; (void)il; (void)iu; (void)abstol; (void)isuppz; (void)work; (void)lwork;
  (void)rwork; (void)lrwork; (void)iwork; (void)liwork;
  const int n = *N;
  const int up = (*uplo == 'U' || *uplo == 'u');
  zc* H = (zc*)malloc(sizeof(zc) * (size_t)n * n);
  zc* V = (zc*)malloc(sizeof(zc) * (size_t)n * n);
  if (!H || !V) { free(H); free(V); *info = -99; return; }
  /* H[i*n+j], full Hermitian, from the referenced triangle of column-major A */
  for (int j = 0; j < n; ++j)
    for (int i = 0; i < n; ++i) {
      int stored = up ? (i <= j) : (i >= j);
      zc a = stored ? A[(size_t)j * *lda + i] : zj(A[(size_t)i * *lda + j]);
      if (i == j) a.y = 0.0;
      H[(size_t)i * n + j] = a;
      V[(size_t)i * n + j].x = (i == j) ? 1.0 : 0.0;
      V[(size_t)i * n + j].y = 0.0;
    }
  for (int sweep = 0; sweep < 100; ++sweep) {
    double off = 0.0, diag = 0.0;
    for (int i = 0; i < n; ++i)
      for (int j = 0; j < n; ++j) {
        zc h = H[(size_t)i * n + j];
        if (i == j) diag += h.x * h.x; else off += h.x * h.x + h.y * h.y;
      }
    if (off <= 1e-32 * (diag > 0 ? diag : 1.0)) break;
    for (int p = 0; p < n - 1; ++p)
      for (int q = p + 1; q < n; ++q) {
        zc hpq = H[(size_t)p * n + q];
        double r = hypot(hpq.x, hpq.y);
        if (r == 0.0) continue;
        zc eph = {hpq.x / r, hpq.y / r};           /* e^{i phi} */
        double th = (H[(size_t)q * n + q].x - H[(size_t)p * n + p].x) / (2.0 * r);
        double t = (th >= 0 ? 1.0 : -1.0) / (fabs(th) + sqrt(th * th + 1.0));
        double c = 1.0 / sqrt(1.0 + t * t), s = t * c;
        zc emi = zj(eph);                           /* e^{-i phi} */
        zc Upp = {c, 0.0}, Upq = {s, 0.0};
        zc Uqp = {-s * emi.x, -s * emi.y}, Uqq = {c * emi.x, c * emi.y};
        for (int k = 0; k < n; ++k) {               /* H <- H U */
          zc hkp = H[(size_t)k * n + p], hkq = H[(size_t)k * n + q];
          H[(size_t)k * n + p] = za(zm(hkp, Upp), zm(hkq, Uqp));
          H[(size_t)k * n + q] = za(zm(hkp, Upq), zm(hkq, Uqq));
          zc vkp = V[(size_t)k * n + p], vkq = V[(size_t)k * n + q];
          V[(size_t)k * n + p] = za(zm(vkp, Upp), zm(vkq, Uqp));
          V[(size_t)k * n + q] = za(zm(vkp, Upq), zm(vkq, Uqq));
        }
        for (int k = 0; k < n; ++k) {               /* H <- U^dag H */
          zc hpk = H[(size_t)p * n + k], hqk = H[(size_t)q * n + k];
          H[(size_t)p * n + k] = za(zm(zj(Upp), hpk), zm(zj(Uqp), hqk));
          H[(size_t)q * n + k] = za(zm(zj(Upq), hpk), zm(zj(Uqq), hqk));
        }
        H[(size_t)p * n + q].x = H[(size_t)p * n + q].y = 0.0;
        H[(size_t)q * n + p].x = H[(size_t)q * n + p].y = 0.0;
        H[(size_t)p * n + p].y = 0.0;
        H[(size_t)q * n + q].y = 0.0;
      }
  }
  int* idx = (int*)malloc(sizeof(int) * (size_t)n);
  for (int i = 0; i < n; ++i) idx[i] = i;
  for (int i = 1; i < n; ++i) {                     /* insertion sort, ascending */
    int v = idx[i], j = i - 1;
    while (j >= 0 && H[(size_t)idx[j] * n + idx[j]].x > H[(size_t)v * n + v].x) { idx[j + 1] = idx[j]; --j; }
    idx[j + 1] = v;
  }
  for (int j = 0; j < n; ++j) {
    W[j] = H[(size_t)idx[j] * n + idx[j]].x;
    if (*jobz == 'V' || *jobz == 'v')
      for (int i = 0; i < n; ++i) Z[(size_t)j * *ldz + i] = V[(size_t)i * n + idx[j]];
  }
  *M = n;
  *info = 0;
  free(idx); free(H); free(V);
}
