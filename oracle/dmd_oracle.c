/* ORACLE -- CPU restatement of DMD's Lindblad density-matrix right-hand side and steppers.
 *
 * TEST INFRASTRUCTURE ONLY. Imported solely by tests/, __graft_entry__.smoke() and bench.py's
 * CPU-baseline leg, always as the checker; never part of the product path.
 *
 * Pinned against the reference: tests/golden/ holds vectors produced by the reference's own
 * sources (src_v4.5.7, compiled unmodified against oracle/ref_shim by oracle/Makefile.ref) and the
 * CPU tests check this file against them. The complex BLAS calls go through the same
 * cblas_zgemm/cblas_zhemm definitions (oracle/ref_shim/cblas_shim.c) as that build.
 *
 * Every function follows the reference statement by statement; file:line citations are relative
 * to the reference tree. complex128 arrays are interleaved (re, im) doubles, k-major, then
 * row-major nb x nb.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include "gsl/gsl_cblas.h"
#include "gsl/gsl_errno.h"
#include "gsl/gsl_odeiv2.h"

typedef struct { double x, y; } zc;

static inline zc zmk(double x, double y) { zc r = {x, y}; return r; }
static inline zc zmul(zc a, zc b) { return zmk(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x); }
static inline zc zadd(zc a, zc b) { return zmk(a.x + b.x, a.y + b.y); }
static inline zc zsub(zc a, zc b) { return zmk(a.x - b.x, a.y - b.y); }
static inline zc zconj(zc a) { return zmk(a.x, -a.y); }
static inline zc zscale(double s, zc a) { return zmk(a.x * s, a.y * s); } /* complex*double (scalar.h:96) */
static inline zc zcis(double x) { return zmk(cos(x), sin(x)); }          /* cis (scalar.h:122-125) */

/* ---------------------------------------------------------------------------------------------
 * System description (what DMD holds in electronphonon / singdenmat_k after setup).
 * ------------------------------------------------------------------------------------------- */
typedef struct {
  int nk;            /* elec->nk */
  int nb_dm;         /* elec->nb_dm: bands of the density matrix */
  int bstart, bend;  /* electronphonon::bStart/bEnd relative to bStart_dm (ElectronPhonon.cpp:143) */
  int64_t npair;     /* nkpair_glob (single rank: nkpair_proc) */
  const uint64_t* k1st;
  const uint64_t* k2nd;
  const zc* P1;      /* [npair][nb^4], already scaled and with e-imp folded (ElectronPhonon.cpp:209-253, 44-113) */
  const zc* P2;
  const double* e_dm;  /* [nk][nb_dm] */
  double prefac_eph;   /* 2*pi/nk_full (ElectronPhonon.h:61) */
  const zc* Hcoh;      /* [nk][nb_dm^2] or NULL (DenMat.cpp:7-28) */
  int picture_schrodinger; /* alg.picture == "schrodinger" */
  int expt;            /* alg.expt */
  const zc* ddmdt_eq;  /* [nk][nb^2] window, NULL unless alg.ddmdteq */
  int scatt_enable;    /* alg.scatt_enable */
  int linear;          /* alg.linearize: P1, P2 hold Lscij, Lscji (ElectronPhonon_linear.cpp) */
  const double* f_lin; /* [nk][nb] window f_eq of the linearization */
} orc_sys;

/* workspace for one RHS evaluation */
typedef struct {
  zc *dm, *dm1, *ddmdt_eph, *Pdm, *dm1P, *P1t, *P2t, *P1n, *P2n, *coh, *dmx, *dm1x, *ddmx, *ddmdt;
} orc_ws;

static void* xmalloc(size_t n) { void* p = calloc(n ? n : 1, 1); if (!p) abort(); return p; }

orc_ws* orc_ws_new(const orc_sys* s) {
  orc_ws* w = (orc_ws*)xmalloc(sizeof(orc_ws));
  const int nb = s->bend - s->bstart, nb2 = nb * nb, nb4 = nb2 * nb2, nd2 = s->nb_dm * s->nb_dm;
  w->dm = (zc*)xmalloc(sizeof(zc) * s->nk * nb2);
  w->dm1 = (zc*)xmalloc(sizeof(zc) * s->nk * nb2);
  w->ddmdt_eph = (zc*)xmalloc(sizeof(zc) * s->nk * nb2);
  w->Pdm = (zc*)xmalloc(sizeof(zc) * s->nk * nb2);
  w->dm1P = (zc*)xmalloc(sizeof(zc) * s->nk * nb2);
  w->P1t = (zc*)xmalloc(sizeof(zc) * nb4);
  w->P2t = (zc*)xmalloc(sizeof(zc) * nb4);
  w->P1n = (zc*)xmalloc(sizeof(zc) * nb4);
  w->P2n = (zc*)xmalloc(sizeof(zc) * nb4);
  w->coh = (zc*)xmalloc(sizeof(zc) * s->nk * nd2);
  w->dmx = (zc*)xmalloc(sizeof(zc) * s->nk * nd2);
  w->dm1x = (zc*)xmalloc(sizeof(zc) * s->nk * nd2);
  w->ddmx = (zc*)xmalloc(sizeof(zc) * s->nk * nd2);
  w->ddmdt = (zc*)xmalloc(sizeof(zc) * s->nk * nd2);
  return w;
}

void orc_ws_free(orc_ws* w) {
  if (!w) return;
  zc* p[] = {w->dm, w->dm1, w->ddmdt_eph, w->Pdm, w->dm1P, w->P1t, w->P2t, w->P1n, w->P2n, w->coh, w->dmx, w->dm1x, w->ddmx, w->ddmdt};
  for (size_t i = 0; i < sizeof(p) / sizeof(p[0]); ++i) free(p[i]);
  free(w);
}

/* zgemm_interface(C, A, B, m, n, k, alpha, beta) -- comm/mymatrix.cpp:82-86 (row-major, no trans) */
static void zgemm_mnk(zc* C, const zc* A, const zc* B, int m, int n, int k, zc alpha, zc beta) {
  cblas_zgemm(CblasRowMajor, CblasNoTrans, CblasNoTrans, m, n, k, &alpha, A, k, B, n, &beta, C, n);
}
/* zhemm_interface(C, left, A, B, n, alpha, beta) -- comm/mymatrix.cpp:73-76 (upper triangle) */
static void zhemm_n(zc* C, int left, const zc* A, const zc* B, int n, zc alpha, zc beta) {
  cblas_zhemm(CblasRowMajor, left ? CblasLeft : CblasRight, CblasUpper, n, n, &alpha, A, n, B, n, &beta, C, n);
}

/* compute_Pt -- evolve_eph.cpp:169-187 */
static void compute_Pt(int nb, double t, const double* ek, const double* ekp, const zc* P, zc* Pt, int minus) {
  for (int i1 = 0; i1 < nb; i1++) {
    int n1 = i1 * nb;
    for (int i2 = 0; i2 < nb; i2++) {
      int n12 = (n1 + i2) * nb;
      for (int i3 = 0; i3 < nb; i3++) {
        int n123 = (n12 + i3) * nb;
        for (int i4 = 0; i4 < nb; i4++) {
          if (!minus) Pt[n123 + i4] = zmul(P[n123 + i4], zcis((ek[i1] - ekp[i3] - ek[i2] + ekp[i4]) * t));
          else Pt[n123 + i4] = zmul(P[n123 + i4], zcis((ek[i3] - ekp[i1] - ek[i4] + ekp[i2]) * t));
        }
      }
    }
  }
}

/* The rank-local pair loop of electronphonon::evolve (evolve_eph.cpp:49-135) over pairs [p0, p1)
 * (one MPI rank's contiguous slice, mymp::distribute_var mymp.cpp:8-36), accumulating into Pdm and
 * dm1P (summode, dense P, expt or not; no valley filtering: the default alg.only_intra/intervalley =
 * false and fewer than two valleys keep every pair, evolve_eph.cpp:52-58). e is [nk][nb]. */
void orc_pairs_partial(const orc_sys* s, const double* e, double t, const zc* dm, const zc* dm1, int64_t p0, int64_t p1,
                       zc* Pdm, zc* dm1P) {
  const int nb = s->bend - s->bstart, nb2 = nb * nb, nb4 = nb2 * nb2;
  const zc c1 = zmk(1, 0);
  zc *P1t = (zc*)xmalloc(sizeof(zc) * nb4), *P2t = (zc*)xmalloc(sizeof(zc) * nb4);
  zc *P1n = (zc*)xmalloc(sizeof(zc) * nb4), *P2n = (zc*)xmalloc(sizeof(zc) * nb4);
  for (int64_t ip = p0; ip < p1; ip++) {
    const int ik = (int)s->k1st[ip], ikp = (int)s->k2nd[ip];
    const zc* P1 = s->P1 + (size_t)ip * nb4;
    const zc* P2 = s->P2 + (size_t)ip * nb4;
    if (!s->expt) {
      /* axbyc(P1t, P1, nb^4): y = x */
      memcpy(P1t, P1, sizeof(zc) * nb4);
      memcpy(P2t, P2, sizeof(zc) * nb4);
    } else {
      compute_Pt(nb, t, e + (size_t)ik * nb, e + (size_t)ikp * nb, P1, P1t, 0);
      compute_Pt(nb, t, e + (size_t)ik * nb, e + (size_t)ikp * nb, P2, P2t, 1);
    }
    zgemm_mnk(Pdm + (size_t)ik * nb2, P1t, dm + (size_t)ikp * nb2, nb2, 1, nb2, c1, c1);
    zgemm_mnk(dm1P + (size_t)ik * nb2, dm1 + (size_t)ikp * nb2, P2t, 1, nb2, nb2, c1, c1);
    if (ik < ikp) {
      for (int i = 0; i < nb4; i++) { P2n[i] = zconj(P1t[i]); P1n[i] = zconj(P2t[i]); }
      zgemm_mnk(Pdm + (size_t)ikp * nb2, P1n, dm + (size_t)ik * nb2, nb2, 1, nb2, c1, c1);
      zgemm_mnk(dm1P + (size_t)ikp * nb2, dm1 + (size_t)ik * nb2, P2n, 1, nb2, nb2, c1, c1);
    }
  }
  free(P1t); free(P2t); free(P1n); free(P2n);
}

/* The per-k finish of electronphonon::evolve after the allreduce (evolve_eph.cpp:140-162). */
void orc_evolve_finish(const orc_sys* s, const double* e, double t, const zc* dm, const zc* dm1, const zc* Pdm,
                       const zc* dm1P, zc* ddmdt_eph, int compute_eq) {
  const int nk = s->nk, nb = s->bend - s->bstart, nb2 = nb * nb;
  const zc c1 = zmk(1, 0), cm1 = zmk(-1, 0), c0 = zmk(0, 0);
  zc* contrib = (zc*)xmalloc(sizeof(zc) * nb2);
  for (int ik = 0; ik < nk; ik++) {
    memset(contrib, 0, sizeof(zc) * nb2);
    zhemm_n(contrib, 1, dm1 + (size_t)ik * nb2, Pdm + (size_t)ik * nb2, nb, c1, c0);
    zhemm_n(contrib, 0, dm + (size_t)ik * nb2, dm1P + (size_t)ik * nb2, nb, cm1, c1);
    for (int i = 0; i < nb; i++)
      for (int j = 0; j < nb; j++)
        ddmdt_eph[(size_t)ik * nb2 + i * nb + j] = zscale(s->prefac_eph * 0.5, zadd(contrib[i * nb + j], zconj(contrib[j * nb + i])));
  }
  free(contrib);
  if (!compute_eq && s->ddmdt_eq) {
    for (int ik = 0; ik < nk; ik++)
      for (int i = 0; i < nb; i++)
        for (int j = 0; j < nb; j++) {
          zc* o = &ddmdt_eph[(size_t)ik * nb2 + i * nb + j];
          const zc q = s->ddmdt_eq[(size_t)ik * nb2 + i * nb + j];
          if (i == j || s->picture_schrodinger) *o = zsub(*o, q);
          else *o = zsub(*o, zmul(q, zcis((e[(size_t)ik * nb + i] - e[(size_t)ik * nb + j]) * t)));
        }
  }
}

/* electronphonon::evolve -- evolve_eph.cpp:34-166 on a single rank */
void orc_evolve(const orc_sys* s, orc_ws* w, const double* e, double t, const zc* dm, const zc* dm1, zc* ddmdt_eph, int compute_eq) {
  const int nk = s->nk, nb = s->bend - s->bstart, nb2 = nb * nb;
  memset(ddmdt_eph, 0, sizeof(zc) * nk * nb2);
  memset(w->Pdm, 0, sizeof(zc) * nk * nb2);
  memset(w->dm1P, 0, sizeof(zc) * nk * nb2);
  orc_pairs_partial(s, e, t, dm, dm1, 0, s->npair, w->Pdm, w->dm1P);
  /* the rank-local sums are complete on a single rank (mymp allreduce, evolve_eph.cpp:137) */
  orc_evolve_finish(s, e, t, dm, dm1, w->Pdm, w->dm1P, ddmdt_eph, compute_eq);
}

/* trunc_copy_arraymat -- comm/mymatrix.cpp:134-144 */
static void trunc_copy(zc* A, const zc* B, int n1, int n2, int bs, int be) {
  const int nb = be - bs;
  for (int i1 = 0; i1 < n1; i1++)
    for (int b1 = 0; b1 < nb; b1++)
      for (int b2 = 0; b2 < nb; b2++) A[(size_t)i1 * nb * nb + b1 * nb + b2] = B[(size_t)i1 * n2 * n2 + (b1 + bs) * n2 + b2 + bs];
}

/* electronphonon::compute_ddmdt -- evolve_eph_linear.cpp:44-51 */
static void lin_compute_ddmdt(const orc_sys* s, int nb, const zc* dmkp, const zc* lsc, zc* ddmdtk) {
  const int nb2 = nb * nb;
  zc contrib[16];
  memset(contrib, 0, sizeof(contrib));
  zgemm_mnk(contrib, lsc, dmkp, nb2, 1, nb2, zmk(1, 0), zmk(0, 0));
  for (int i = 0; i < nb; i++)
    for (int j = 0; j < nb; j++)
      ddmdtk[i * nb + j] = zadd(ddmdtk[i * nb + j], zscale(s->prefac_eph * 0.5, zadd(contrib[i * nb + j], zconj(contrib[j * nb + i]))));
}

/* electronphonon::evolve_linear -- evolve_eph_linear.cpp:3-42 on a single rank; dm is the window
 * copy, modified in place (dm_ii -= f_eq) as the reference does */
static void orc_evolve_linear(const orc_sys* s, const double* e, double t, zc* dm, zc* ddmdt_eph) {
  const int nk = s->nk, nb = s->bend - s->bstart, nb2 = nb * nb, nb4 = nb2 * nb2;
  for (int ik = 0; ik < nk; ik++)
    for (int i = 0; i < nb; i++) dm[(size_t)ik * nb2 + i * nb + i].x -= s->f_lin[(size_t)ik * nb + i];
  memset(ddmdt_eph, 0, sizeof(zc) * (size_t)nk * nb2);
  zc* Lsct = (zc*)xmalloc(sizeof(zc) * nb4);
  for (int64_t ip = 0; ip < s->npair; ip++) {
    const int ik = (int)s->k1st[ip], ikp = (int)s->k2nd[ip];
    const zc* Lij = s->P1 + (size_t)ip * nb4;
    const zc* Lji = s->P2 + (size_t)ip * nb4;
    if (!s->expt) {
      lin_compute_ddmdt(s, nb, dm + (size_t)ikp * nb2, Lij, ddmdt_eph + (size_t)ik * nb2);
      if (ik < ikp) lin_compute_ddmdt(s, nb, dm + (size_t)ik * nb2, Lji, ddmdt_eph + (size_t)ikp * nb2);
    } else {
      compute_Pt(nb, t, e + (size_t)ik * nb, e + (size_t)ikp * nb, Lij, Lsct, 0);
      lin_compute_ddmdt(s, nb, dm + (size_t)ikp * nb2, Lsct, ddmdt_eph + (size_t)ik * nb2);
      if (ik < ikp) {
        compute_Pt(nb, t, e + (size_t)ikp * nb, e + (size_t)ik * nb, Lji, Lsct, 0);
        lin_compute_ddmdt(s, nb, dm + (size_t)ik * nb2, Lsct, ddmdt_eph + (size_t)ikp * nb2);
      }
    }
  }
  free(Lsct);
}

/* Linear operators from one source of P (ElectronPhonon_linear.cpp:147-225): for every pair,
 * add_Lscii_from_P1_P2 then add_Lscij_from_P1_P2 (fac2 = false). f is the window f_eq [nk][nb]. */
void orc_lsc_add(int nk, int nb, int64_t npair, const uint64_t* k1, const uint64_t* k2, const zc* P1, const zc* P2,
                 const double* f, zc* Lscii, zc* Lij, zc* Lji) {
  const int nb2 = nb * nb, nb4 = nb2 * nb2;
  (void)nk;
  for (int64_t p = 0; p < npair; p++) {
    const int ik = (int)k1[p], jk = (int)k2[p];
    const zc* P1p = P1 + (size_t)p * nb4;
    const zc* P2p = P2 + (size_t)p * nb4;
    zc* Li = Lscii + (size_t)ik * nb4;
    zc* Lj = Lscii + (size_t)jk * nb4;
    for (int i1 = 0; i1 < nb; i1++)
      for (int i2 = 0; i2 < nb; i2++) {
        const int i12 = i1 * nb + i2, n12 = i12 * nb2;
        for (int ib = 0; ib < nb; ib++) {
          const int nbv = (ib * nb + i2) * nb2, iab = i1 * nb + ib, i12ab = n12 + iab;
          for (int i3 = 0; i3 < nb; i3++) {
            const int ib233 = nbv + i3 * nb + i3;
            Li[i12ab] = zsub(Li[i12ab], zscale(f[(size_t)jk * nb + i3], P1p[ib233]));
            if (jk > ik) Lj[i12ab] = zsub(Lj[i12ab], zscale(f[(size_t)ik * nb + i3], zconj(P2p[ib233])));
          }
        }
        for (int ia = 0; ia < nb; ia++) {
          const int i1a = i1 * nb + ia, iab = ia * nb + i2, i12ab = n12 + iab;
          for (int i3 = 0; i3 < nb; i3++) {
            const int i331a = (i3 * nb + i3) * nb2 + i1a;
            Li[i12ab] = zsub(Li[i12ab], zscale(1 - f[(size_t)jk * nb + i3], P2p[i331a]));
            if (jk > ik) Lj[i12ab] = zsub(Lj[i12ab], zscale(1 - f[(size_t)ik * nb + i3], zconj(P1p[i331a])));
          }
        }
      }
    zc* Lijp = Lij + (size_t)p * nb4;
    zc* Ljip = Lji + (size_t)p * nb4;
    for (int i1 = 0; i1 < nb; i1++)
      for (int i2 = 0; i2 < nb; i2++) {
        const int i12 = i1 * nb + i2, n12 = i12 * nb2;
        for (int ia = 0; ia < nb; ia++)
          for (int ib = 0; ib < nb; ib++) {
            const int iab = ia * nb + ib, i12ab = n12 + iab, iab12 = iab * nb2 + i12;
            zc c = zadd(zscale(1 - f[(size_t)ik * nb + i1], P1p[i12ab]), zscale(f[(size_t)ik * nb + i2], P2p[iab12]));
            Lijp[i12ab] = zadd(Lijp[i12ab], c);
            c = zadd(zscale(1 - f[(size_t)jk * nb + i1], zconj(P2p[i12ab])), zscale(f[(size_t)jk * nb + i2], zconj(P1p[iab12])));
            Ljip[i12ab] = zadd(Ljip[i12ab], c);
          }
      }
  }
}

/* set_Lsc's last step (ElectronPhonon_linear.cpp:23-30): Lscii joins the diagonal pairs */
void orc_lsc_diag(int nb, int64_t npair, const uint64_t* k1, const uint64_t* k2, const zc* Lscii, zc* Lij, zc* Lji) {
  const int nb4 = nb * nb * nb * nb;
  for (int64_t p = 0; p < npair; p++) {
    if (k1[p] != k2[p]) continue;
    const zc* x = Lscii + (size_t)k1[p] * nb4;
    for (int e = 0; e < nb4; e++) {
      Lij[(size_t)p * nb4 + e] = zadd(Lij[(size_t)p * nb4 + e], zadd(x[e], zmk(0, 0)));
      Lji[(size_t)p * nb4 + e] = zadd(Lji[(size_t)p * nb4 + e], zadd(x[e], zmk(0, 0)));
    }
  }
}

/* electronphonon::evolve_driver -- evolve_eph.cpp:21-32 (window copy, evolve, set_mat back;
 * set_mat's column loop starts at i0 = bStart, comm/mymatrix.cpp:114-119, and i0 = j0 here) */
void orc_evolve_driver(const orc_sys* s, orc_ws* w, double t, const zc* dm_x, const zc* dm1_x, zc* ddmdt_x) {
  const int nk = s->nk, nd = s->nb_dm, bs = s->bstart, be = s->bend, nb = be - bs;
  double* e = (double*)xmalloc(sizeof(double) * nk * nb);
  for (int ik = 0; ik < nk; ik++)
    for (int b = 0; b < nb; b++) e[ik * nb + b] = s->e_dm[(size_t)ik * nd + bs + b]; /* trunc_alloccopy_array (ElectronPhonon.h:79) */
  trunc_copy(w->dm, dm_x, nk, nd, bs, be);
  trunc_copy(w->dm1, dm1_x, nk, nd, bs, be);
  if (s->linear) orc_evolve_linear(s, e, t, w->dm, w->ddmdt_eph);
  else orc_evolve(s, w, e, t, w->dm, w->dm1, w->ddmdt_eph, 0);
  memset(ddmdt_x, 0, sizeof(zc) * nk * nd * nd);
  for (int ik = 0; ik < nk; ik++)
    for (int i = bs; i < be; i++)
      for (int j = bs; j < be; j++) ddmdt_x[(size_t)ik * nd * nd + i * nd + j] = w->ddmdt_eph[(size_t)ik * nb * nb + (i - bs) * nb + j - bs];
  free(e);
}

/* singdenmat_k::evolve_coh -- DenMat.cpp:29-55 (single rank: nk_proc = nk, ik0 = 0) */
void orc_evolve_coh(const orc_sys* s, orc_ws* w, double t, const zc* dm, zc* out) {
  const int nk = s->nk, nb = s->nb_dm, nb2 = nb * nb;
  const zc c1 = zmk(1, 0), cm1 = zmk(-1, 0), c0 = zmk(0, 0), cmi = zmk(0, -1);
  zc* Hbuf = (zc*)xmalloc(sizeof(zc) * nb2);
  zc* Ht = Hbuf;
  memset(out, 0, sizeof(zc) * nk * nb2);
  for (int ik = 0; ik < nk; ik++) {
    const zc* dmk = dm + (size_t)ik * nb2;
    zc* o = out + (size_t)ik * nb2;
    const double* ek = s->e_dm + (size_t)ik * nb;
    if (s->Hcoh) {
      const zc* Hk = s->Hcoh + (size_t)ik * nb2;
      if (!s->picture_schrodinger) {
        for (int i = 0; i < nb; i++)
          for (int j = 0; j < nb; j++) Ht[i * nb + j] = (i == j) ? Hk[i * nb + j] : zmul(Hk[i * nb + j], zcis((ek[i] - ek[j]) * t));
      } else {
        memcpy(Ht, Hk, sizeof(zc) * nb2); /* Hcoh already holds H + diag(e) (DenMat.cpp:20-24) */
      }
      zhemm_n(o, 0, Ht, dmk, nb, c1, c0);   /* dm * H   (Right) */
      zhemm_n(o, 1, Ht, dmk, nb, c1, cm1);  /* H * dm - dm * H */
      for (int i = 0; i < nb2; i++) o[i] = zmul(o[i], cmi);
    } else if (s->picture_schrodinger) {
      /* commutator_mat_diag(C, e, dm, nb, cmi) (comm/mymatrix.cpp:230-235 with mat_diag_mult
       * :173-199): C = dm_ij e_j; C = -C + e_i dm_ij; C *= -i */
      for (int i = 0; i < nb; i++)
        for (int j = 0; j < nb; j++) {
          const zc d = dmk[i * nb + j];
          const zc a = zmk(-(d.x * ek[j]), -(d.y * ek[j]));
          o[i * nb + j] = zmul(zadd(a, zmul(zmk(ek[i], 0), d)), cmi);
        }
    }
  }
  free(Hbuf);
}

/* dm_dynamics::compute -- DensityMatrix_Dynamics.h:243-278 (no laser, no phenomenological term,
 * not semiclassical): ddmdt = coherent + scattering on the state dm; 1 - dm per set_oneminusdm
 * (DenMat.cpp:249-261). */
void orc_compute(const orc_sys* s, orc_ws* w, double t, const zc* dm, zc* ddmdt) {
  const int nk = s->nk, nb = s->nb_dm, nb2 = nb * nb;
  for (int ik = 0; ik < nk; ik++)
    for (int i = 0; i < nb; i++)
      for (int j = 0; j < nb; j++) {
        const zc v = dm[(size_t)ik * nb2 + i * nb + j];
        w->dm1x[(size_t)ik * nb2 + i * nb + j] = (i == j) ? zsub(zmk(1, 0), v) : zmk(-v.x, -v.y);
      }
  memset(ddmdt, 0, sizeof(zc) * nk * nb2);
  if (s->picture_schrodinger || s->Hcoh) {
    orc_evolve_coh(s, w, t, dm, w->coh);
    for (size_t i = 0; i < (size_t)nk * nb2; i++) ddmdt[i] = zadd(ddmdt[i], w->coh[i]);
  }
  if (s->scatt_enable) {
    orc_evolve_driver(s, w, t, dm, w->dm1x, w->ddmx);
    for (size_t i = 0; i < (size_t)nk * nb2; i++) ddmdt[i] = zadd(ddmdt[i], w->ddmx[i]);
  }
}

/* func -- DensityMatrix_Dynamics.h:358-369 with copy_complex_from_real / copy_real_from_complex
 * (comm/ODE.h:6-15): y and dydt are interleaved (re, im). */
typedef struct { const orc_sys* s; orc_ws* w; unsigned long ncalls; } orc_ctx;

int orc_func(double t, const double y[], double dydt[], void* params) {
  orc_ctx* c = (orc_ctx*)params;
  c->ncalls++;
  orc_compute(c->s, c->w, t, (const zc*)y, (zc*)dydt);
  return GSL_SUCCESS;
}

/* observable "sx/sy/sz" for bands [bs, be) -- observable.h:356-366 (general branch) and
 * 412-429 (totals): tot = prefac * sum_k sum_{i in [bs,be)} sum_b Re[o_ib(t) (dm_bi - f_i delta_ib)]
 * with o_ib(t) = o_ib * cis((e_i - e_b) t) off the diagonal in the interaction picture, and
 * tot_amp the same without the phase. prefac = 1/(nk_full * cell_size_cmd) (observable.h:54). */
void orc_measure(int nk, int nb, int bs, int be, const zc* obs /*[nk][nb^2] one direction*/, size_t obs_kstride,
                 const double* f, const double* e, double t, int picture_schrodinger, const zc* dm, double prefac,
                 double* tot_out, double* amp_out) {
  double tot = 0, tot_amp = 0;
  for (int ik = 0; ik < nk; ik++)
    for (int i = bs; i < be; i++) {
      double ob = 0, ob_amp = 0;
      for (int b = 0; b < nb; b++) {
        const zc ob_kib = obs[(size_t)ik * obs_kstride + i * nb + b];
        const zc ob_kib_t = (i == b || picture_schrodinger) ? ob_kib : zmul(ob_kib, zcis((e[(size_t)ik * nb + i] - e[(size_t)ik * nb + b]) * t));
        zc dm_kbi = dm[(size_t)ik * nb * nb + b * nb + i];
        if (i == b) dm_kbi = zsub(dm_kbi, zmk(f[(size_t)ik * nb + i], 0));
        ob += zmul(ob_kib_t, dm_kbi).x;
        ob_amp += zmul(ob_kib, dm_kbi).x;
      }
      tot += ob;
      tot_amp += ob_amp;
    }
  *tot_out = tot * prefac;
  *amp_out = tot_amp * prefac;
}

/* electron::compute_dm_Bpert_1st -- electron.cpp:62-98 (needL = false): dm = f + dfde * (Bpert . S)
 * with the interaction-picture phase at t0 off the diagonal. */
void orc_dm_bpert(int nk, int nb, const zc* s /*[nk][3][nb^2]*/, const double* e, const double* f, double temperature,
                  const double* Bpert, double t0, int picture_schrodinger, zc* dm_out) {
  const double degthr = 1e-8;
  for (int ik = 0; ik < nk; ik++) {
    zc* d = dm_out + (size_t)ik * nb * nb;
    const zc* sk = s + (size_t)ik * 3 * nb * nb;
    for (int i = 0; i < nb; i++)
      for (int j = i; j < nb; j++) {
        zc H1 = zadd(zadd(zscale(Bpert[0], sk[i * nb + j]), zscale(Bpert[1], sk[nb * nb + i * nb + j])), zscale(Bpert[2], sk[2 * nb * nb + i * nb + j]));
        double dfde;
        const double *ek = e + (size_t)ik * nb, *fk = f + (size_t)ik * nb;
        if (fabs(ek[i] - ek[j]) < degthr) {
          double favg = 0.5 * (fk[i] + fk[j]);
          dfde = favg * (favg - 1.) / temperature;
        } else {
          dfde = (fk[i] - fk[j]) / (ek[i] - ek[j]);
        }
        d[i * nb + j] = zscale(dfde, H1);
        if (i != j && !picture_schrodinger) d[i * nb + j] = zmul(d[i * nb + j], zcis((ek[i] - ek[j]) * t0));
        if (i < j) d[j * nb + i] = zconj(d[i * nb + j]);
      }
    for (int i = 0; i < nb; i++) d[i * nb + i] = zadd(d[i * nb + i], zmk(f[(size_t)ik * nb + i], 0));
  }
}

/* singdenmat_k::init_dm(complex**) -- DenMat.cpp:65-81: Hermitian part of dm0 */
void orc_init_dm(int nk, int nb, const zc* dm0, zc* dm) {
  for (int ik = 0; ik < nk; ik++)
    for (int i = 0; i < nb; i++)
      for (int j = 0; j < nb; j++)
        dm[(size_t)ik * nb * nb + i * nb + j] = zscale(0.5, zadd(dm0[(size_t)ik * nb * nb + i * nb + j], zconj(dm0[(size_t)ik * nb * nb + j * nb + i])));
}

/* electron::set_H_BS -- electron.cpp:19-42 (no g-factor distribution, no Bso, needL = false):
 * H = B . S; then singdenmat_k::init_Hcoh (DenMat.cpp:7-28) adds diag(e) in the Schrodinger picture. */
void orc_H_BS(int nk, int nb, const zc* s, const double* B, const double* e, int picture_schrodinger, zc* H) {
  for (int ik = 0; ik < nk; ik++)
    for (int ij = 0; ij < nb * nb; ij++) {
      const zc* sk = s + (size_t)ik * 3 * nb * nb;
      /* vec3_dot_vec3array(vm, v, m, n): vm = v[0]*m[0] + v[1]*m[1] + v[2]*m[2] */
      H[(size_t)ik * nb * nb + ij] = zadd(zadd(zscale(B[0], sk[ij]), zscale(B[1], sk[nb * nb + ij])), zscale(B[2], sk[2 * nb * nb + ij]));
    }
  if (picture_schrodinger)
    for (int ik = 0; ik < nk; ik++)
      for (int i = 0; i < nb; i++) H[(size_t)ik * nb * nb + i * nb + i].x += e[(size_t)ik * nb + i];
}

/* ---------------------------------------------------------------------------------------------
 * Steppers.
 * ------------------------------------------------------------------------------------------- */

/* Classic fixed-step RK4 calling func (the oracle driver's mode; DMD itself offers RKF45 and
 * Euler). y_{n+1} = y_n + h/6 (k1 + 2 k2 + 2 k3 + k4), stages at t, t+h/2, t+h/2, t+h.
 * After every `every` steps the S observable of direction idir is recorded (if obs != NULL). */
typedef struct {
  const zc* obs; size_t obs_kstride; const double* f; double prefac; int bs, be;
} orc_meas;

int orc_rk4(const orc_sys* s, double t0, double h, long nsteps, double* y, long every, const orc_meas* m, double* rec /* [nsteps/every][3] t,tot,amp */) {
  const size_t n2 = (size_t)2 * s->nk * s->nb_dm * s->nb_dm;
  orc_ws* w = orc_ws_new(s);
  orc_ctx c = {s, w, 0};
  double *k1 = (double*)xmalloc(n2 * 8), *k2 = (double*)xmalloc(n2 * 8), *k3 = (double*)xmalloc(n2 * 8), *k4 = (double*)xmalloc(n2 * 8), *yt = (double*)xmalloc(n2 * 8);
  const double hh = 0.5 * h, h6 = h / 6.0;
  long irec = 0;
  for (long st = 0; st < nsteps; ++st) {
    const double t = t0 + (double)st * h;
    orc_func(t, y, k1, &c);
    for (size_t i = 0; i < n2; ++i) yt[i] = y[i] + hh * k1[i];
    orc_func(t + hh, yt, k2, &c);
    for (size_t i = 0; i < n2; ++i) yt[i] = y[i] + hh * k2[i];
    orc_func(t + hh, yt, k3, &c);
    for (size_t i = 0; i < n2; ++i) yt[i] = y[i] + h * k3[i];
    orc_func(t + h, yt, k4, &c);
    for (size_t i = 0; i < n2; ++i) y[i] = y[i] + h6 * (k1[i] + 2.0 * k2[i] + 2.0 * k3[i] + k4[i]);
    if (m && rec && every > 0 && (st + 1) % every == 0) {
      const double t1 = t0 + (double)(st + 1) * h;
      double tot, amp;
      orc_measure(s->nk, s->nb_dm, m->bs, m->be, m->obs, m->obs_kstride, m->f, s->e_dm, t1, s->picture_schrodinger, (const zc*)y, m->prefac, &tot, &amp);
      rec[3 * irec + 0] = t1; rec[3 * irec + 1] = tot; rec[3 * irec + 2] = amp;
      ++irec;
    }
  }
  free(k1); free(k2); free(k3); free(k4); free(yt);
  orc_ws_free(w);
  return 0;
}

/* DMD's evolve_gsl loop (DensityMatrix_Dynamics.h:189-225) without laser / scattering updates:
 * the GSL driver (oracle/gsl_rkf45.c) advances to ti = t0 + it*tstep for it = 1..nout and S is
 * recorded after each output interval. Returns the GSL status; ncalls_out[it-1] holds the RHS
 * evaluations of each interval (ode.ncalls). */
int orc_rkf45(const orc_sys* s, double t0, double tend, double tstep, double hstart, double hmin, double hmax, double epsabs,
              double* y, const orc_meas* m, double* rec, long* ncalls_out, long max_out) {
  const size_t n2 = (size_t)2 * s->nk * s->nb_dm * s->nb_dm;
  orc_ws* w = orc_ws_new(s);
  orc_ctx c = {s, w, 0};
  gsl_odeiv2_system sys = {orc_func, 0, n2, &c};
  gsl_odeiv2_driver* d = gsl_odeiv2_driver_alloc_y_new(&sys, gsl_odeiv2_step_rkf45, hstart, epsabs, 0.0);
  gsl_odeiv2_driver_set_hmin(d, hmin);
  gsl_odeiv2_driver_set_hmax(d, hmax);
  double t = t0, ti = t0;
  int status = GSL_SUCCESS;
  long it = 1;
  for (; t < tend && it <= max_out; it += 1) {
    ti += tstep;
    c.ncalls = 0;
    status = gsl_odeiv2_driver_apply(d, &t, ti, y);
    if (status != GSL_SUCCESS) break;
    if (ncalls_out) ncalls_out[it - 1] = (long)c.ncalls;
    if (m && rec) {
      double tot, amp;
      orc_measure(s->nk, s->nb_dm, m->bs, m->be, m->obs, m->obs_kstride, m->f, s->e_dm, t, s->picture_schrodinger, (const zc*)y, m->prefac, &tot, &amp);
      rec[3 * (it - 1) + 0] = t; rec[3 * (it - 1) + 1] = tot; rec[3 * (it - 1) + 2] = amp;
    }
  }
  gsl_odeiv2_driver_free(d);
  orc_ws_free(w);
  return status;
}

/* Euler step -- singdenmat_k::update_dm_euler (DenMat.cpp:236-248) after compute(t). */
int orc_euler(const orc_sys* s, double t0, double h, long nsteps, double* y) {
  const int nk = s->nk, nb = s->nb_dm, nb2 = nb * nb;
  orc_ws* w = orc_ws_new(s);
  double t = t0;
  for (long st = 0; st < nsteps; ++st, t += h) { /* sdmk->t += dt_current() (DensityMatrix_Dynamics.h:232) */
    orc_compute(s, w, t, (const zc*)y, w->ddmdt);
    zc* dm = (zc*)y;
    for (int ik = 0; ik < nk; ik++)
      for (int i = 0; i < nb; i++)
        for (int j = 0; j < nb; j++)
          dm[(size_t)ik * nb2 + i * nb + j] = zadd(dm[(size_t)ik * nb2 + i * nb + j],
              zscale(0.5 * h, zadd(w->ddmdt[(size_t)ik * nb2 + i * nb + j], zconj(w->ddmdt[(size_t)ik * nb2 + j * nb + i]))));
  }
  orc_ws_free(w);
  return 0;
}

/* one-call wrappers used through ctypes */
void orc_rhs(const orc_sys* s, double t, const double* y, double* dydt) {
  orc_ws* w = orc_ws_new(s);
  orc_compute(s, w, t, (const zc*)y, (zc*)dydt);
  orc_ws_free(w);
}

void orc_rhs_parts(const orc_sys* s, double t, const double* y, double* ddmdt_eph, double* ddmdt_coh) {
  orc_ws* w = orc_ws_new(s);
  const int nk = s->nk, nb = s->nb_dm, nb2 = nb * nb;
  const zc* dm = (const zc*)y;
  for (int ik = 0; ik < nk; ik++)
    for (int i = 0; i < nb; i++)
      for (int j = 0; j < nb; j++) {
        const zc v = dm[(size_t)ik * nb2 + i * nb + j];
        w->dm1x[(size_t)ik * nb2 + i * nb + j] = (i == j) ? zsub(zmk(1, 0), v) : zmk(-v.x, -v.y);
      }
  orc_evolve_driver(s, w, t, dm, w->dm1x, (zc*)ddmdt_eph);
  if (s->Hcoh || s->picture_schrodinger) orc_evolve_coh(s, w, t, dm, (zc*)ddmdt_coh);
  else memset(ddmdt_coh, 0, sizeof(zc) * nk * nb2);
  orc_ws_free(w);
}

size_t orc_sys_size(void) { return sizeof(orc_sys); }

/* electron::fermi (electron.h:119-124) over an array, with the C library's exp */
void orc_fermi(double T, double mu, const double* e, double* f, size_t n) {
  for (size_t i = 0; i < n; i++) {
    const double ebyt = (e[i] - mu) / T;
    if (ebyt < -46) f[i] = 1;
    else if (ebyt > 46) f[i] = 0;
    else f[i] = 1. / (exp(ebyt) + 1);
  }
}

/* Multi-rank form of func (the reference's MPI decomposition, main.cpp:66 + evolve_eph.cpp:137):
 * orc_window_in builds the window dm / 1-dm (evolve_driver's trunc_copy) and e; each rank runs
 * orc_pairs_partial on its slice; the sums are added (the allreduce) and orc_rhs_from_partials
 * finishes, adds the coherent term and writes dydt. */
void orc_window_in(const orc_sys* s, const double* y, double* e_w, double* dm_w, double* dm1_w) {
  const int nk = s->nk, nd = s->nb_dm, bs = s->bstart, be = s->bend, nb = be - bs, nd2 = nd * nd;
  const zc* dm = (const zc*)y;
  zc* dm1x = (zc*)xmalloc(sizeof(zc) * (size_t)nk * nd2);
  for (int ik = 0; ik < nk; ik++)
    for (int i = 0; i < nd; i++)
      for (int j = 0; j < nd; j++) {
        const zc v = dm[(size_t)ik * nd2 + i * nd + j];
        dm1x[(size_t)ik * nd2 + i * nd + j] = (i == j) ? zsub(zmk(1, 0), v) : zmk(-v.x, -v.y);
      }
  for (int ik = 0; ik < nk; ik++)
    for (int b = 0; b < nb; b++) e_w[ik * nb + b] = s->e_dm[(size_t)ik * nd + bs + b];
  trunc_copy((zc*)dm_w, dm, nk, nd, bs, be);
  trunc_copy((zc*)dm1_w, dm1x, nk, nd, bs, be);
  free(dm1x);
}

void orc_rhs_from_partials(const orc_sys* s, double t, const double* y, const double* e_w, const double* dm_w,
                           const double* dm1_w, const double* Pdm, const double* dm1P, double* dydt) {
  const int nk = s->nk, nd = s->nb_dm, bs = s->bstart, be = s->bend, nb = be - bs, nd2 = nd * nd, nb2 = nb * nb;
  orc_ws* w = orc_ws_new(s);
  zc* out = (zc*)dydt;
  memset(out, 0, sizeof(zc) * (size_t)nk * nd2);
  if (s->picture_schrodinger || s->Hcoh) {
    orc_evolve_coh(s, w, t, (const zc*)y, w->coh);
    for (size_t i = 0; i < (size_t)nk * nd2; i++) out[i] = zadd(out[i], w->coh[i]);
  }
  orc_evolve_finish(s, e_w, t, (const zc*)dm_w, (const zc*)dm1_w, (const zc*)Pdm, (const zc*)dm1P, w->ddmdt_eph, 0);
  for (int ik = 0; ik < nk; ik++)
    for (int i = bs; i < be; i++)
      for (int j = bs; j < be; j++)
        out[(size_t)ik * nd2 + i * nd + j] = zadd(out[(size_t)ik * nd2 + i * nd + j], w->ddmdt_eph[(size_t)ik * nb2 + (i - bs) * nb + j - bs]);
  orc_ws_free(w);
}

/* ------------------------------------------------------------------------------------------------
 * Chemical potential and the equilibrium drift (set-up, once per run)
 * ---------------------------------------------------------------------------------------------- */
static double fermi1(double T, double mu, double e) { /* electron::fermi, electron.h:119-124 */
  const double ebyt = (e - mu) / T;
  if (ebyt < -46) return 1;
  else if (ebyt > 46) return 0;
  else return 1. / (exp(ebyt) + 1);
}
static int isgn(double v) { return (0. < v) - (v < 0.); } /* sgn, electron.cpp:3-5 / DenMat.cpp:3-5 */

/* electron::compute_nfree -- electron.cpp:578-596 (one rank; e is [nk][nb], valence bands [0, nv)) */
double orc_compute_nfree(int isHole, double T, double mu, const double* e, int nk, int nb, int nv) {
  const int b0 = isHole ? 0 : nv, b1 = isHole ? nv : nb;
  double r = 0.;
  for (int ik = 0; ik < nk; ik++)
    for (int i = b0; i < b1; i++) {
      const double f = fermi1(T, mu, e[(size_t)ik * nb + i]);
      if (!isHole) r += f;
      else r += (f - 1.);
    }
  return r;
}

/* electron::find_mu by bisection -- electron.cpp:537-572. The impurity-level carriers
 * (Scatt_Param.h:82-94) are zero without partially ionised impurities, the only case accepted. */
double orc_find_mu_bisect(double carrier_bvk, int is_excess, double T, double emin, double emax, const double* e,
                          int nk, int nb, int nv) {
  const int isHole = carrier_bvk < 0;
  double lo = emin, hi = emax, result = 0, cnew;
  int niter = 0;
  while (niter < 200) {
    niter++;
    result = 0.5 * (lo + hi);
    if (is_excess)
      cnew = orc_compute_nfree(1, T, result, e, nk, nb, nv) + 0. + orc_compute_nfree(0, T, result, e, nk, nb, nv) + 0.;
    else
      cnew = orc_compute_nfree(isHole, T, result, e, nk, nb, nv) + 0.;
    const double error = cnew - carrier_bvk;
    if (fabs(error) < 1e-12) return result;
    if (cnew > carrier_bvk) hi = result;
    else lo = result;
  }
  return result;
}

/* singdenmat_k::compute_nfree_eq -- DenMat.cpp:198-225 (e = e_dm [nk][nb], bands [b0, b1)) */
static double nfree_eq(int isHole, double T, double mu, const double* e, int nk, int nb, int b0, int b1) {
  double r = 0.;
  for (int ik = 0; ik < nk; ik++)
    for (int i = b0; i < b1; i++) {
      const double f = fermi1(T, mu, e[(size_t)ik * nb + i]);
      if (!isHole) r += f;
      else r += (f - 1.);
    }
  return r;
}

/* singdenmat_k::find_mu -- DenMat.cpp:150-197 (damped search from mu0) */
double orc_find_mu_eq(int isHole, double carrier_bvk, double T, double mu0, const double* e, int nk, int nb, int b0,
                      int b1) {
  double result = mu0, damp = 0.7, dmu = 5e-6;
  double eoo = 1., eo = 1., excess, cnew;
  int step = 0;
  while (1) {
    cnew = nfree_eq(isHole, T, result, e, nk, nb, b0, b1) + 0.;
    excess = cnew - carrier_bvk;
    if (fabs(excess) > 1e-14) {
      if (fabs(excess) > fabs(eo) || fabs(excess) > fabs(eoo)) dmu *= damp;
      result -= isgn(excess) * dmu;
      if (step > 0 && isgn(excess) == isgn(eo)) {
        const double ratio = cnew / carrier_bvk;
        if (ratio < 1e-9) result -= (double)(isgn(excess) * 10) * T;
        else if (ratio < 1e-4) result -= (double)(isgn(excess) * 3) * T;
        else if (ratio < 0.1) result -= isgn(excess) * 0.7 * T;
      }
      if (dmu < 1e-16) break;
      eoo = eo;
      eo = excess;
      step++;
      if (step > 1e4) break;
    } else
      break;
  }
  return result;
}

/* elecimpParam::carrier_bvk_ex -- Scatt_Param.h:63-68. gs[0..2] = carrier_bvk_gs, ne_bvk_gs, nh_bvk_gs
 * (electron.h:155-157); nimp = number of impurity densities. Returns 0 in *ok for the combination the
 * reference leaves undefined (carrier_bvk_gs == 0 with impurities). */
double orc_carrier_bvk_ex(int isHole, double n_bvk_ex, int nimp, const double* gs, int* ok) {
  *ok = 1;
  if (nimp == 0 || (gs[0] > 0 && isHole) || (gs[0] < 0 && !isHole)) return n_bvk_ex;
  if (gs[0] < 0 && isHole) return gs[0] + (n_bvk_ex - gs[2]);
  if (gs[0] > 0 && !isHole) return gs[0] + (n_bvk_ex - gs[1]);
  *ok = 0;
  return n_bvk_ex;
}

/* singdenmat_k::set_dm_eq -- DenMat.cpp:97-148 with compute_f (DenMat.h:74-83): the chemical
 * potentials that keep the carrier numbers of dm, and the occupations f_eq [nk][nb_dm].
 * mu[0..1] in: mue, muh start values; out: the found ones. Returns 0, or -1 for the undefined case. */
int orc_set_dm_eq(int nk, int nb, int nv, const zc* dm, double T, const double* e, int nimp, const double* gs,
                  int debug, double* mu, double* f_eq) {
  for (int pass = 0; pass < 2; pass++) {
    const int isHole = pass == 1;
    if (!isHole && !(nb > nv)) continue;
    if (isHole && !(nv > 0)) continue;
    const int b0 = isHole ? 0 : nv, b1 = isHole ? nv : nb;
    double nfree_bvk = 0.;
    for (int ik = 0; ik < nk; ik++)
      for (int i = b0; i < b1; i++) {
        if (!isHole) nfree_bvk += dm[(size_t)ik * nb * nb + i * nb + i].x;
        else nfree_bvk += (dm[(size_t)ik * nb * nb + i * nb + i].x - 1.);
      }
    int ok;
    const double target = orc_carrier_bvk_ex(isHole, nfree_bvk, nimp, gs, &ok);
    if (!ok) return -1;
    double m = orc_find_mu_eq(isHole, target, T, mu[pass], e, nk, nb, b0, b1);
    if (debug) m = mu[pass];
    mu[pass] = m;
  }
  for (int ik = 0; ik < nk; ik++) {
    for (int i = 0; i < nv; i++) f_eq[(size_t)ik * nb + i] = fermi1(T, mu[1], e[(size_t)ik * nb + i]);
    for (int i = nv; i < nb; i++) f_eq[(size_t)ik * nb + i] = fermi1(T, mu[0], e[(size_t)ik * nb + i]);
  }
  return 0;
}

/* electronphonon::compute_ddmdt_eq -- evolve_eph.cpp:3-19: the scattering term at t = 0 of the
 * diagonal state f_eq (1 - f_eq on the diagonal of dm1, zeros elsewhere), window [bstart, bend).
 * s->ddmdt_eq must be NULL (it is still all zeros in the reference when this runs). */
void orc_compute_ddmdt_eq(const orc_sys* s, const double* f_eq, double* ddmdt_eq) {
  const int nk = s->nk, nd = s->nb_dm, nd2 = nd * nd, bs = s->bstart, be = s->bend, nb = be - bs;
  orc_ws* w = orc_ws_new(s);
  zc* dm = (zc*)xmalloc(sizeof(zc) * (size_t)nk * nd2);
  zc* dm1 = (zc*)xmalloc(sizeof(zc) * (size_t)nk * nd2);
  zc* out = (zc*)xmalloc(sizeof(zc) * (size_t)nk * nd2);
  for (int ik = 0; ik < nk; ik++)
    for (int i = 0; i < nd; i++) {
      dm[(size_t)ik * nd2 + i * nd + i] = zmk(f_eq[(size_t)ik * nd + i], 0);
      dm1[(size_t)ik * nd2 + i * nd + i] = zmk(1 - f_eq[(size_t)ik * nd + i], 0);
    }
  orc_evolve_driver(s, w, 0., dm, dm1, out);
  trunc_copy((zc*)ddmdt_eq, out, nk, nd, bs, be);
  (void)nb;
  free(dm); free(dm1); free(out);
  orc_ws_free(w);
}
