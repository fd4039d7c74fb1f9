/* ORACLE -- CPU restatement of DMD's Lindblad density-matrix right-hand side and steppers.
 *
 * TEST INFRASTRUCTURE ONLY. Imported solely by tests/, __graft_entry__.smoke() and bench.py's
 * CPU-baseline leg, always as the side the GPU results are compared with (or timed beside); never
 * part of the product path.
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
#define _GNU_SOURCE /* sincos (glibc), as scalar.h's cis calls it */
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
/* a / b: complex(a.x b.x + a.y b.y, a.y b.x - a.x b.y) / b.norm(), the division by a double a
 * multiplication by its reciprocal (scalar.h:98-101) */
static inline zc zdiv(zc a, zc b) {
  const double r = 1.0 / (b.x * b.x + b.y * b.y);
  return zmk((a.x * b.x + a.y * b.y) * r, (a.y * b.x - a.x * b.y) * r);
}

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
  struct orc_ee* ee;   /* e-e model rebuilt from rho on every RHS (eeMode Pee_update, freq < 0), or NULL */
  int sparse;          /* alg.sparseP: P kept as sparse_mat per pair and contracted by sparse_zgemm */
  double thr_sparse;   /* alg.thr_sparseP */
} orc_sys;

/* e-e scattering model (ElecElec_Model.h) with static screening (Coulomb_Model.h:394-688):
 * what electronphonon holds for eeMode = Pee_update. P1, P2 of the system point at P1eff, P2eff. */
typedef struct orc_ee {
  int nb, nbw;             /* window bands; Wannier functions (elec->nb_wannier) */
  const double* kvec;      /* [nk][3] fractional (electron.cpp:134-146) */
  int kmesh[3];
  const zc* U;             /* [nk][nbw][nb] (electron.cpp:388-410) */
  double GGT[9];           /* lattice.h:41-42 */
  double cell_size, nk_full, T, eps, meff;
  int formula;             /* 0 unscreened, 1 debye, 2 Bechstedt, 3 RPA, 4 lindhard (clp.scrFormula) */
  double nfree;            /* clp.nfreetot: the screening density */
  int update_screening;    /* clp.update: nfree from rho at each rebuild (Coulomb_Model.h:533-553) */
  int nv;                  /* coul_model->nv: window bands below it count holes */
  double degauss, ethr;    /* eep.degauss; param->degauss * ndegauss */
  int antisym;             /* eep.antisymmetry */
  double scale;            /* scale_ee */
  int inside;              /* rebuild before every RHS evaluation */
  const zc* P1base;        /* [npair][nb^4]: P_eph (+ P_eimp) */
  const zc* P2base;
  zc* P1eff;               /* P_base + scale P_ee: the operators the RHS uses */
  zc* P2eff;
  zc* P1ee;                /* the last P_ee (prefactor included, scale not) */
  zc* P2ee;
  const double* f_setup;   /* [nk][nb] window occupations of the set-up (coul_model->f): static RPA */
  double* vq_rpa;          /* [n0 n1 n2] static RPA / Lindhard vq by the q mesh index (orc_ee_rpa_table) */
  int dynamic;             /* clp.dynamic: 0 "static", 1 "ppa" (plasmon-pole approximation) */
  int ppa_gn;              /* clp.ppamodel: 1 "gn" (Godby-Needs), 0 "hl" (Hybertsen-Louie) */
  double eppa;             /* clp.eppa after init_RPA (the plasma frequency when given as 0) */
  double smearing;         /* clp.smearing after Coulomb_Model.h:523 (0.5 T when <= 0, except gn) */
  int two_freqs;           /* clp.dynamic_screening_ee_two_freqs */
  zc* Aq_ppa;              /* [n0 n1 n2] by q mesh index: eps^-1(w) = 1 + A / (w^2 - E^2) (:855-874) */
  zc* Eq2_ppa;
} orc_ee;

void orc_ee_rebuild(struct orc_ee* ee, const orc_sys* s, double t, const double* y);

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

/* sparse_mat::sparse (comm/sparse_matrix.h:57-69): the elements with abs(A) = sqrt(norm) > thr, row-major */
static int sparse_of(const zc* A, int n2, double thr, zc* sv, int* si, int* sj) {
  int ns = 0;
  for (int i = 0; i < n2; i++)
    for (int j = 0; j < n2; j++) {
      const zc a = A[i * n2 + j];
      if (sqrt(a.x * a.x + a.y * a.y) > thr) {
        sv[ns] = a;
        si[ns] = i;
        sj[ns] = j;
        ns++;
      }
    }
  return ns;
}

/* compute_sPt (evolve_eph.cpp:194-203): the phase of every stored element; ij2i / ij2j split the
 * operator's row (i1 i2) and column (i3 i4) indices */
static void compute_sPt(int nb, double t, const double* ek, const double* ekp, const zc* sv, const int* si,
                        const int* sj, int ns, zc* st, int minus) {
  for (int is = 0; is < ns; is++) {
    const int i = si[is] / nb, j = si[is] % nb, k = sj[is] / nb, l = sj[is] % nb;
    if (!minus) st[is] = zmul(sv[is], zcis((ek[i] - ekp[k] - ek[j] + ekp[l]) * t));
    else st[is] = zmul(sv[is], zcis((ek[k] - ekp[i] - ek[l] + ekp[j]) * t));
  }
}

/* sparse_zgemm (comm/sparse_matrix.cpp:6-40) with alpha = beta = 1 for the two shapes the evolve
 * loop uses: left (m = nb^2, n = 1): c[i] += s b[j]; right (m = 1, n = nb^2): c[j] += b[i] s. The
 * c *= beta pass over the whole output is kept. */
static void sparse_zgemm_v(zc* c, int left, const zc* sv, const int* si, const int* sj, int ns, const zc* b, int n2) {
  const zc one = zmk(1, 0);
  for (int i = 0; i < n2; i++) c[i] = zmul(c[i], one);
  if (left)
    for (int is = 0; is < ns; is++) c[si[is]] = zadd(c[si[is]], zmul(sv[is], b[sj[is]]));
  else
    for (int is = 0; is < ns; is++) c[sj[is]] = zadd(c[sj[is]], zmul(b[si[is]], sv[is]));
}

/* The sparse branch of the pair loop (alg.sparseP, evolve_eph.cpp:67-82): P1 and P2 of every pair as
 * sparse_mat (built from the dense operators with thr_sparseP, ElectronPhonon.cpp:115-130), phases per
 * element, sparse GEMVs, and for k < k' the conjugated elements of P2 / P1 on the k' side. */
static void orc_pairs_sparse(const orc_sys* s, const double* e, double t, const zc* dm, const zc* dm1, int64_t p0,
                             int64_t p1, zc* Pdm, zc* dm1P) {
  const int nb = s->bend - s->bstart, nb2 = nb * nb, nb4 = nb2 * nb2;
  zc *s1 = (zc*)xmalloc(sizeof(zc) * nb4), *s2 = (zc*)xmalloc(sizeof(zc) * nb4);
  zc *t1 = (zc*)xmalloc(sizeof(zc) * nb4), *t2 = (zc*)xmalloc(sizeof(zc) * nb4);
  zc *n1 = (zc*)xmalloc(sizeof(zc) * nb4), *n2 = (zc*)xmalloc(sizeof(zc) * nb4);
  int *i1 = (int*)xmalloc(sizeof(int) * nb4), *j1 = (int*)xmalloc(sizeof(int) * nb4);
  int *i2 = (int*)xmalloc(sizeof(int) * nb4), *j2 = (int*)xmalloc(sizeof(int) * nb4);
  for (int64_t ip = p0; ip < p1; ip++) {
    const int ik = (int)s->k1st[ip], ikp = (int)s->k2nd[ip];
    const int ns1 = sparse_of(s->P1 + (size_t)ip * nb4, nb2, s->thr_sparse, s1, i1, j1);
    const int ns2 = sparse_of(s->P2 + (size_t)ip * nb4, nb2, s->thr_sparse, s2, i2, j2);
    if (!s->expt) {
      memcpy(t1, s1, sizeof(zc) * ns1);
      memcpy(t2, s2, sizeof(zc) * ns2);
    } else {
      compute_sPt(nb, t, e + (size_t)ik * nb, e + (size_t)ikp * nb, s1, i1, j1, ns1, t1, 0);
      compute_sPt(nb, t, e + (size_t)ik * nb, e + (size_t)ikp * nb, s2, i2, j2, ns2, t2, 1);
    }
    sparse_zgemm_v(Pdm + (size_t)ik * nb2, 1, t1, i1, j1, ns1, dm + (size_t)ikp * nb2, nb2);
    sparse_zgemm_v(dm1P + (size_t)ik * nb2, 0, t2, i2, j2, ns2, dm1 + (size_t)ikp * nb2, nb2);
    if (ik < ikp) {
      for (int q = 0; q < ns2; q++) n1[q] = zconj(t2[q]); /* sm1_next = conj(smat2_time) */
      for (int q = 0; q < ns1; q++) n2[q] = zconj(t1[q]); /* sm2_next = conj(smat1_time) */
      sparse_zgemm_v(Pdm + (size_t)ikp * nb2, 1, n1, i2, j2, ns2, dm + (size_t)ik * nb2, nb2);
      sparse_zgemm_v(dm1P + (size_t)ikp * nb2, 0, n2, i1, j1, ns1, dm1 + (size_t)ik * nb2, nb2);
    }
  }
  free(s1); free(s2); free(t1); free(t2); free(n1); free(n2); free(i1); free(j1); free(i2); free(j2);
}

/* The rank-local pair loop of electronphonon::evolve (evolve_eph.cpp:49-135) over pairs [p0, p1)
 * (one MPI rank's contiguous slice, mymp::distribute_var mymp.cpp:8-36), accumulating into Pdm and
 * dm1P (summode, dense P, expt or not; no valley filtering: the default alg.only_intra/intervalley =
 * false and fewer than two valleys keep every pair, evolve_eph.cpp:52-58). e is [nk][nb]. */
void orc_pairs_partial(const orc_sys* s, const double* e, double t, const zc* dm, const zc* dm1, int64_t p0, int64_t p1,
                       zc* Pdm, zc* dm1P) {
  if (s->sparse) {
    orc_pairs_sparse(s, e, t, dm, dm1, p0, p1, Pdm, dm1P);
    return;
  }
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
 * add_Lscii_from_P1_P2 then add_Lscij_from_P1_P2 (fac2 = false; the e-e source with the exchange
 * term passes fac2 = true, ElectronPhonon_linear.cpp:84). f is the window f_eq [nk][nb]. */
void orc_lsc_add2(int nk, int nb, int64_t npair, const uint64_t* k1, const uint64_t* k2, const zc* P1, const zc* P2,
                  const double* f, zc* Lscii, zc* Lij, zc* Lji, int fac2);
void orc_lsc_add(int nk, int nb, int64_t npair, const uint64_t* k1, const uint64_t* k2, const zc* P1, const zc* P2,
                 const double* f, zc* Lscii, zc* Lij, zc* Lji) {
  orc_lsc_add2(nk, nb, npair, k1, k2, P1, P2, f, Lscii, Lij, Lji, 0);
}
void orc_lsc_add2(int nk, int nb, int64_t npair, const uint64_t* k1, const uint64_t* k2, const zc* P1, const zc* P2,
                  const double* f, zc* Lscii, zc* Lij, zc* Lji, int fac2) {
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
            Lijp[i12ab] = zadd(Lijp[i12ab], fac2 ? zscale(2, c) : c);
            c = zadd(zscale(1 - f[(size_t)jk * nb + i1], zconj(P2p[i12ab])), zscale(f[(size_t)jk * nb + i2], zconj(P1p[iab12])));
            Ljip[i12ab] = zadd(Ljip[i12ab], fac2 ? zscale(2, c) : c);
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

/* ---------------------------------------------------------------------------------------------
 * e-e model (eeMode = Pee_update)
 * ------------------------------------------------------------------------------------------- */

/* wrap to [-0.5, 0.5) -- comm/kmap.h:6-15 */
static void ee_wrap(const double* x, double* r) {
  for (int d = 0; d < 3; d++) {
    r[d] = x[d];
    r[d] -= floor(0.5 + r[d]);
    if (fabs(r[d] - 0.5) < 1e-6) r[d] = -0.5;
  }
}

/* GGT.metric_length_squared(wrap(q)) -- comm/matrix3.h:119-121 */
static double ee_q2(const orc_ee* ee, const double* q) {
  double v[3];
  ee_wrap(q, v);
  const double* m = ee->GGT;
  return v[0] * v[0] * m[0] + v[1] * v[1] * m[4] + v[2] * v[2] * m[8] +
         2 * (v[0] * v[1] * m[1] + v[0] * v[2] * m[2] + v[1] * v[2] * m[5]);
}

/* screening constants of coulomb_model::init_model (Coulomb_Model.h:555-569) for density n */
typedef struct { double prefac_vq, prefac_vq_bare, qscr2_debye, fac0, fac2, fac4; } ee_scr;

static ee_scr ee_screen(const orc_ee* ee, double n) {
  ee_scr c;
  c.prefac_vq = 4 * M_PI / ee->eps / ee->cell_size;  /* Coulomb_Model.h:423-424 */
  c.prefac_vq_bare = 4 * M_PI / ee->cell_size;
  const double kF = pow(3 * M_PI * M_PI * n, 1. / 3.);
  const double kF2 = kF * kF;
  const double EF = kF2 / 2. / ee->meff;
  const double qTF2 = 6 * M_PI * n / ee->eps / EF;
  c.fac0 = 1. / (ee->eps - 1);
  c.fac2 = 1. / qTF2;
  c.fac4 = 3. / 4. / kF2 / qTF2;
  c.qscr2_debye = 4 * M_PI * n / ee->eps / ee->T;
  return c;
}

static void ee_ikvec3(const orc_ee* ee, const double* k, int* v);

/* coulomb_model::vq, static branches (Coulomb_Model.h:632-660) */
static double ee_vq(const orc_ee* ee, const ee_scr* c, const double* q) {
  const double q2 = ee_q2(ee, q);
  if (ee->formula >= 3) { /* vq_RPA[q2iq(q)][0].real() (Coulomb_Model.h:662-666) */
    if (q2 < 1e-20) return 0.0;
    int v[3];
    ee_ikvec3(ee, q, v);
    return ee->vq_rpa[((size_t)v[0] * ee->kmesh[1] + v[1]) * ee->kmesh[2] + v[2]];
  }
  if (ee->formula == 0) return q2 < 1e-20 ? 0.0 : c->prefac_vq / q2;
  if (ee->formula == 1) return c->prefac_vq / (c->qscr2_debye + q2);
  if (q2 < 1e-20) return 0.0;
  const double epsq = 1 + 1. / (c->fac0 + c->fac2 * q2 + c->fac4 * q2 * q2);
  return c->prefac_vq_bare / epsq / q2;
}

/* coulomb_model::vq(q, w) with dynamic = ppa (Coulomb_Model.h:659-687): RPA / Lindhard only (the
 * reference refuses the other formulas with dynamic screening); w = 0 gives the static value
 * vq_RPA[iq][0].real(); otherwise (prefac_vq + A / (cw^2 - E^2)) / |q|^2 with cw = |w| + i smearing,
 * conjugated for w < 0 (eps(q, -w) = eps(q, w)^*) */
static zc ee_vq_dyn(const orc_ee* ee, const ee_scr* c, const double* q, double w) {
  const double q2 = ee_q2(ee, q);
  int v[3];
  ee_ikvec3(ee, q, v);
  const size_t m = ((size_t)v[0] * ee->kmesh[1] + v[1]) * ee->kmesh[2] + v[2];
  if (q2 < 1e-20) return zmk(0, 0);
  if (w == 0) return zmk(ee->vq_rpa[m], 0);
  const zc cw = zmk(fabs(w), ee->smearing);
  const zc t = zdiv(ee->Aq_ppa[m], zsub(zmk(cw.x * cw.x - cw.y * cw.y, cw.y * cw.x + cw.x * cw.y), ee->Eq2_ppa[m]));
  const double rq = 1.0 / q2;
  const zc r = zmk((t.x + c->prefac_vq) * rq, t.y * rq);
  return w < 0 ? zconj(r) : r;
}

/* the interaction factor of one mee element (ElecElec_Model.h:96-110, 124-135): vq(q, w) at the mean
 * energy transfer w = 0.5 (wa + wb), or with the two-frequency option sqrt(|vq(q, wa)| |vq(q, wb)|)
 * cis of the mean phase */
static zc ee_vq_elem(const orc_ee* ee, const ee_scr* c, const double* q, double wa, double wb, double wmean) {
  if (!ee->two_freqs) return ee_vq_dyn(ee, c, q, wmean);
  const zc va = ee_vq_dyn(ee, c, q, wa), vb = ee_vq_dyn(ee, c, q, wb);
  const double vabs = sqrt(sqrt(va.x * va.x + va.y * va.y) * sqrt(vb.x * vb.x + vb.y * vb.y));
  const double varg = 0.5 * (atan2(va.y, va.x) + atan2(vb.y, vb.x));
  double sn, cs;
  sincos(varg, &sn, &cs);
  return zmk(cs * vabs, sn * vabs);
}

/* kIndexMap::ikvec3 -- comm/kmap.cpp:15-23 */
static void ee_ikvec3(const orc_ee* ee, const double* k, int* v) {
  for (int d = 0; d < 3; d++) {
    const double ki = k[d] - floor(k[d]);
    v[d] = (int)round(ee->kmesh[d] * ki);
    if (v[d] == ee->kmesh[d]) v[d] = 0;
  }
}

/* kIndexMap::findk (comm/kmap.cpp:3-10): the map from mesh indices to k as a dense table over the
 * mesh, the first k-point of an index kept as std::map::insert keeps it (comm/kmap.h:22-28) */
static int ee_findk(const orc_ee* ee, const int* table, const double* k) {
  int v[3];
  ee_ikvec3(ee, k, v);
  return table[((size_t)v[0] * ee->kmesh[1] + v[1]) * ee->kmesh[2] + v[2]];
}

/* elecelec_model::calc_ovlp -- ElecElec_Model.h:72-80: ovlp = U_ik^dagger U_jk (nb x nb), times
 * vq(k_ik - k_jk) when asked */
static void ee_ovlp(const orc_ee* ee, const ee_scr* c, zc* ovlp, zc* Uih, int ik, int jk, int with_vq) {
  const int nb = ee->nb, nbw = ee->nbw;
  const zc* Ui = ee->U + (size_t)ik * nbw * nb;
  for (int i = 0; i < nb; i++) /* hermite(a, h, m = nbw, n = nb): h[i*m + j] = conj(a[j*n + i]) */
    for (int j = 0; j < nbw; j++) Uih[i * nbw + j] = zconj(Ui[j * nb + i]);
  zgemm_mnk(ovlp, Uih, ee->U + (size_t)jk * nbw * nb, nb, nb, nbw, zmk(1, 0), zmk(0, 0));
  if (!with_vq) return;
  double q[3];
  for (int d = 0; d < 3; d++) q[d] = ee->kvec[3 * ik + d] - ee->kvec[3 * jk + d];
  const zc vq = zmk(ee_vq(ee, c, q), 0);
  for (int i = 0; i < nb * nb; i++) ovlp[i] = zmul(vq, ovlp[i]); /* axbyc(ovlp, nullptr, n, c0, vq) */
}

/* coulomb_model's static RPA / Lindhard screening (Coulomb_Model.h:690-736 calc_qscr2_static_RPA,
 * 819-826 calc_vq_RPA, static): the q set of qIndexMap::build (comm/kmap.h:43-56: every k_i - k_j, first
 * occurrence of a mesh index), then for each q in that order and each k in order with k - q on the
 * set, dfde |<k|k-q>|^2 summed (Lindhard: b1 = b2, no overlap), times prefac_vq / nk_full, and
 * vq = prefac_vq / (|q|^2 + qscr2) with scalar.h's complex division. Stored by q mesh index. */
void orc_ee_rpa_table(orc_ee* ee, int nk, const double* e /* [nk][nb] */) {
  const int nb = ee->nb;
  const size_t nmesh = (size_t)ee->kmesh[0] * ee->kmesh[1] * ee->kmesh[2];
  int* table = (int*)xmalloc(sizeof(int) * nmesh);
  for (size_t i = 0; i < nmesh; i++) table[i] = -1;
  for (int ik = 0; ik < nk; ik++) {
    int v[3];
    ee_ikvec3(ee, ee->kvec + 3 * ik, v);
    int* slot = &table[((size_t)v[0] * ee->kmesh[1] + v[1]) * ee->kmesh[2] + v[2]];
    if (*slot < 0) *slot = ik;
  }
  /* qvec in qIndexMap::build order: wrap(k_ik - k_jk), the first of each mesh index */
  int* qseen = (int*)xmalloc(sizeof(int) * nmesh);
  for (size_t i = 0; i < nmesh; i++) qseen[i] = -1;
  double* qvec = (double*)xmalloc(sizeof(double) * 3 * (size_t)nk * nk);
  size_t nq = 0;
  for (int ik = 0; ik < nk; ik++)
    for (int jk = 0; jk < nk; jk++) {
      double d[3], q[3];
      for (int x = 0; x < 3; x++) d[x] = ee->kvec[3 * ik + x] - ee->kvec[3 * jk + x];
      ee_wrap(d, q);
      int v[3];
      ee_ikvec3(ee, q, v);
      const size_t m = ((size_t)v[0] * ee->kmesh[1] + v[1]) * ee->kmesh[2] + v[2];
      if (qseen[m] < 0) {
        qseen[m] = (int)nq;
        memcpy(qvec + 3 * nq, q, sizeof(q));
        nq++;
      }
    }
  ee_scr c = ee_screen(ee, ee->nfree);
  zc* Uih = (zc*)xmalloc(sizeof(zc) * nb * ee->nbw);
  zc* ovlp = (zc*)xmalloc(sizeof(zc) * nb * nb);
  for (size_t iq = 0; iq < nq; iq++) {
    const double* q = qvec + 3 * iq;
    zc sum = zmk(0, 0);
    for (int ik = 0; ik < nk; ik++) {
      double kj[3];
      for (int x = 0; x < 3; x++) kj[x] = ee->kvec[3 * ik + x] - q[x];
      const int jk = ee_findk(ee, table, kj);
      if (jk < 0) continue;
      ee_ovlp(ee, &c, ovlp, Uih, ik, jk, 0);
      for (int b1 = 0; b1 < nb; b1++)
        for (int b2 = 0; b2 < nb; b2++) {
          if (ee->formula == 4 && b1 != b2) continue;
          const double de = e[ik * nb + b1] - e[jk * nb + b2];
          zc dfde;
          if (sqrt(de * de + 0.0 * 0.0) < 1e-8) { /* abs(complex) (scalar.h:103) */
            const double favg = 0.5 * (ee->f_setup[ik * nb + b1] + ee->f_setup[jk * nb + b2]);
            dfde = zmk((1 - favg) * favg / ee->T, 0);
          } else { /* complex(f_j - f_i, 0) / complex(de, 0) (scalar.h:99) */
            const double fd = ee->f_setup[jk * nb + b2] - ee->f_setup[ik * nb + b1];
            const double nrm = de * de + 0.0 * 0.0, r = 1.0 / nrm;
            dfde = zmk((fd * de + 0.0 * 0.0) * r, (0.0 * de - fd * 0.0) * r);
          }
          if (ee->formula == 3) {
            const double n2 = ovlp[b1 * nb + b2].x * ovlp[b1 * nb + b2].x + ovlp[b1 * nb + b2].y * ovlp[b1 * nb + b2].y;
            sum = zadd(sum, zmk(dfde.x * n2, dfde.y * n2));
          } else {
            sum = zadd(sum, dfde);
          }
        }
    }
    sum = zmul(zmk(c.prefac_vq / ee->nk_full, 0), sum);
    const double q2 = ee_q2(ee, q);
    /* complex(prefac_vq, 0) / (q2 + qscr2) */
    const double dx = q2 + sum.x, dy = sum.y;
    const double r = 1.0 / (dx * dx + dy * dy);
    int v[3];
    ee_ikvec3(ee, q, v);
    const size_t m = ((size_t)v[0] * ee->kmesh[1] + v[1]) * ee->kmesh[2] + v[2];
    ee->vq_rpa[m] = (c.prefac_vq * dx + 0.0 * dy) * r;
    if (!ee->dynamic) continue;
    /* plasmon pole (Coulomb_Model.h:780-874): Godby-Needs needs the sums at w = i eppa as well */
    zc sum1 = zmk(0, 0);
    if (ee->ppa_gn) {
      for (int ik = 0; ik < nk; ik++) {
        double kj[3];
        for (int x = 0; x < 3; x++) kj[x] = ee->kvec[3 * ik + x] - q[x];
        const int jk = ee_findk(ee, table, kj);
        if (jk < 0) continue;
        ee_ovlp(ee, &c, ovlp, Uih, ik, jk, 0);
        for (int b1 = 0; b1 < nb; b1++)
          for (int b2 = 0; b2 < nb; b2++) {
            if (ee->formula == 4 && b1 != b2) continue;
            /* de = e_i - e_j - i eppa; dfde = complex(f_j - f_i, 0) / de */
            const zc de = zmk(e[ik * nb + b1] - e[jk * nb + b2], -ee->eppa);
            const zc dfde = zdiv(zmk(ee->f_setup[jk * nb + b2] - ee->f_setup[ik * nb + b1], 0), de);
            if (ee->formula == 3) {
              const double n2 = ovlp[b1 * nb + b2].x * ovlp[b1 * nb + b2].x + ovlp[b1 * nb + b2].y * ovlp[b1 * nb + b2].y;
              sum1 = zadd(sum1, zmk(dfde.x * n2, dfde.y * n2));
            } else {
              sum1 = zadd(sum1, dfde);
            }
          }
      }
      sum1 = zmul(zmk(c.prefac_vq / ee->nk_full, 0), sum1);
    }
    if (q2 < 1e-20) continue; /* Gamma skipped: A = E^2 = 0 */
    const double wp2 = ee->eppa * ee->eppa;
    if (!ee->ppa_gn) { /* Hybertsen-Louie */
      ee->Aq_ppa[m] = zmk(c.prefac_vq * wp2, 0);
      const zc t = zdiv(zmk(q2, 0), sum);
      ee->Eq2_ppa[m] = zmk((t.x + 1) * wp2, t.y * wp2);
    } else { /* Godby-Needs */
      const double rq = 1.0 / q2;
      const zc eps0inv = zdiv(zmk(1, 0), zmk(sum.x * rq + 1, sum.y * rq));
      const zc epspinv = zdiv(zmk(1, 0), zmk(sum1.x * rq + 1, sum1.y * rq));
      /* wp2 (1 - epspinv) / (epspinv - eps0inv); 1 - z is -z + 1 */
      ee->Eq2_ppa[m] = zdiv(zmk((-epspinv.x + 1) * wp2, -epspinv.y * wp2), zsub(epspinv, eps0inv));
      ee->Aq_ppa[m] = zmul(zmk((-eps0inv.x + 1) * c.prefac_vq, -eps0inv.y * c.prefac_vq), ee->Eq2_ppa[m]);
    }
  }
  free(table); free(qseen); free(qvec); free(Uih); free(ovlp);
}

/* elecelec_model::calc_P for every stored pair (ElecElec_Model.h:186-262, static screening,
 * Lindblad, not linearized). dm, dm1: window [nk][nb^2] in the Schrodinger picture, or NULL for the
 * equilibrium occupations f ([nk][nb] window). Out: P1ee, P2ee [npair][nb^4] (prefactor included). */
void orc_ee_P(const orc_ee* ee, const orc_sys* s, const zc* dm, const zc* dm1, const double* f, double nfree,
              zc* P1out, zc* P2out) {
  const int nk = s->nk, nb = ee->nb, nb2 = nb * nb, nb4 = nb2 * nb2, nd = s->nb_dm, bs = s->bstart;
  const ee_scr c = ee_screen(ee, nfree);
  double* e = (double*)xmalloc(sizeof(double) * nk * nb);
  for (int ik = 0; ik < nk; ik++)
    for (int b = 0; b < nb; b++) e[ik * nb + b] = s->e_dm[(size_t)ik * nd + bs + b];
  const size_t nmesh = (size_t)ee->kmesh[0] * ee->kmesh[1] * ee->kmesh[2];
  int* table = (int*)xmalloc(sizeof(int) * nmesh);
  for (size_t i = 0; i < nmesh; i++) table[i] = -1;
  for (int ik = 0; ik < nk; ik++) {
    int v[3];
    ee_ikvec3(ee, ee->kvec + 3 * ik, v);
    int* slot = &table[((size_t)v[0] * ee->kmesh[1] + v[1]) * ee->kmesh[2] + v[2]];
    if (*slot < 0) *slot = ik;
  }
  zc *Uih = (zc*)xmalloc(sizeof(zc) * nb * ee->nbw), *o12 = (zc*)xmalloc(sizeof(zc) * nb2),
     *o34 = (zc*)xmalloc(sizeof(zc) * nb2), *o14 = (zc*)xmalloc(sizeof(zc) * nb2), *o32 = (zc*)xmalloc(sizeof(zc) * nb2),
     *mee = (zc*)xmalloc(sizeof(zc) * nb4), *mex = (zc*)xmalloc(sizeof(zc) * nb4), *A = (zc*)xmalloc(sizeof(zc) * nb4),
     *A1rho = (zc*)xmalloc(sizeof(zc) * nb2), *A1rhobar = (zc*)xmalloc(sizeof(zc) * nb2),
     *mtmp = (zc*)xmalloc(sizeof(zc) * nb2), *P1 = (zc*)xmalloc(sizeof(zc) * nb4), *P2 = (zc*)xmalloc(sizeof(zc) * nb4);
  double* delta = (double*)xmalloc(sizeof(double) * nb4);
  const double prefac_gauss = 1. / (ee->degauss * sqrt(2. * M_PI));
  const double prefac_exp = -0.25 / pow(ee->degauss, 2); /* Lindblad: prefac_exp_ld */
  for (int64_t ip = 0; ip < s->npair; ip++) {
    const int ik1 = (int)s->k1st[ip], ik2 = (int)s->k2nd[ip];
    zc* P1o = P1out + (size_t)ip * nb4;
    zc* P2o = P2out + (size_t)ip * nb4;
    if (ik1 == ik2 && !ee->antisym) {
      memset(P1o, 0, sizeof(zc) * nb4);
      memset(P2o, 0, sizeof(zc) * nb4);
      continue;
    }
    memset(P1, 0, sizeof(zc) * nb4);
    memset(P2, 0, sizeof(zc) * nb4);
    ee_ovlp(ee, &c, o12, Uih, ik1, ik2, !ee->dynamic);
    double q12[3];
    for (int d = 0; d < 3; d++) q12[d] = ee->kvec[3 * ik1 + d] - ee->kvec[3 * ik2 + d];
    for (int ik3 = 0; ik3 < nk; ik3++) {
      if (ee->antisym && ik1 == ik2 && ik2 == ik3) continue;
      double k4v[3];
      for (int d = 0; d < 3; d++) k4v[d] = ee->kvec[3 * ik1 + d] + ee->kvec[3 * ik3 + d] - ee->kvec[3 * ik2 + d];
      const int ik4 = ee_findk(ee, table, k4v);
      if (ik4 < 0) continue;
      /* calc_delta (ElecElec_Model.h:164-184) */
      int conserved = 0;
      const double *e1 = e + ik1 * nb, *e2 = e + ik2 * nb, *e3 = e + ik3 * nb, *e4 = e + ik4 * nb;
      for (int i1 = 0; i1 < nb; i1++)
        for (int i2 = 0; i2 < nb; i2++)
          for (int i3 = 0; i3 < nb; i3++)
            for (int i4 = 0; i4 < nb; i4++) {
              const int i1234 = ((i1 * nb + i2) * nb + i3) * nb + i4;
              const double de = e1[i1] - e2[i2] + e3[i3] - e4[i4];
              if (fabs(de) < ee->ethr) {
                delta[i1234] = exp(prefac_exp * pow(de, 2));
                conserved = 1;
              } else {
                delta[i1234] = 0;
              }
            }
      if (!conserved) continue;
      /* calc_ovlps (ElecElec_Model.h:64-71; ovlp12 kept from above) and calc_mee / calc_mee_ex */
      ee_ovlp(ee, &c, o34, Uih, ik3, ik4, 0);
      if (ee->antisym) {
        ee_ovlp(ee, &c, o14, Uih, ik1, ik4, !ee->dynamic);
        ee_ovlp(ee, &c, o32, Uih, ik3, ik2, 0);
      }
      double q14[3];
      for (int d = 0; d < 3; d++) q14[d] = ee->kvec[3 * ik1 + d] - ee->kvec[3 * ik4 + d];
      for (int i1 = 0; i1 < nb; i1++)
        for (int i2 = 0; i2 < nb; i2++)
          for (int i3 = 0; i3 < nb; i3++)
            for (int i4 = 0; i4 < nb; i4++) {
              const int i1234 = ((i1 * nb + i2) * nb + i3) * nb + i4;
              mee[i1234] = zmul(o12[i1 * nb + i2], o34[i3 * nb + i4]);
              if (ee->dynamic) /* calc_mee: mee *= vq(k1 - k2, w) */
                mee[i1234] = zmul(mee[i1234], ee_vq_elem(ee, &c, q12, e1[i1] - e2[i2], e4[i4] - e3[i3],
                                                        0.5 * (e1[i1] - e2[i2] + e4[i4] - e3[i3])));
              if (ee->antisym) {
                mex[i1234] = zmul(o14[i1 * nb + i4], o32[i3 * nb + i2]);
                if (ee->dynamic) /* calc_mee_ex multiplies mee (not mee_ex) by vq(k1 - k4, w_ex) */
                  mee[i1234] = zmul(mee[i1234], ee_vq_elem(ee, &c, q14, e1[i1] - e4[i4], e2[i2] - e3[i3],
                                                          0.5 * (e1[i1] - e4[i4] + e2[i2] - e3[i3])));
              }
            }
      if (ee->antisym) /* axbyc(mee, mee_ex, n, -0.5, 0.5): mee = -0.5 mee_ex + 0.5 mee */
        for (int i = 0; i < nb4; i++) mee[i] = zadd(zmul(zmk(-0.5, 0), mex[i]), zmul(zmk(0.5, 0), mee[i]));
      for (int i = 0; i < nb4; i++) A[i] = zscale(delta[i], mee[i]); /* A2 = delta mee; A1 = A2 (Lindblad) */
      /* P1ee, P2ee accumulation (ElecElec_Model.h:199-240) */
      for (int i1 = 0; i1 < nb; i1++)
        for (int i3 = 0; i3 < nb; i3++) {
          const zc* Ab = A + (size_t)(i1 * nb + i3) * nb2;
          const zc* Abar = A + (size_t)(i3 * nb + i1) * nb2;
          if (!dm) { /* calc_A1f, calc_A1fbar */
            const double *f3 = f + (size_t)ik3 * nb, *f4 = f + (size_t)ik4 * nb;
            for (int i = 0; i < nb; i++)
              for (int j = 0; j < nb; j++) {
                A1rho[i * nb + j] = zscale(f4[j], zscale(1 - f3[i], Ab[i * nb + j]));
                A1rhobar[i * nb + j] = zscale(1 - f4[j], zscale(f3[i], Abar[i * nb + j]));
              }
          } else { /* calc_A1rho: dmleft * A1 * dmright (two zhemm) */
            zhemm_n(mtmp, 0, dm + (size_t)ik4 * nb2, Ab, nb, zmk(1, 0), zmk(0, 0));
            zhemm_n(A1rho, 1, dm1 + (size_t)ik3 * nb2, mtmp, nb, zmk(1, 0), zmk(0, 0));
            zhemm_n(mtmp, 0, dm1 + (size_t)ik4 * nb2, Abar, nb, zmk(1, 0), zmk(0, 0));
            zhemm_n(A1rhobar, 1, dm + (size_t)ik3 * nb2, mtmp, nb, zmk(1, 0), zmk(0, 0));
          }
          for (int i2 = 0; i2 < nb; i2++)
            for (int i4 = 0; i4 < nb; i4++) {
              const int i1234 = ((i1 * nb + i2) * nb + i3) * nb + i4;
              const int n24 = (i2 * nb + i4) * nb2, n42 = (i4 * nb + i2) * nb2;
              for (int i6 = 0; i6 < nb; i6++)
                for (int i8 = 0; i8 < nb; i8++) {
                  const int i68 = i6 * nb + i8;
                  P1[i1234] = zadd(P1[i1234], zmul(A1rho[i68], zconj(A[n24 + i68])));
                  P2[i1234] = zadd(P2[i1234], zmul(A1rhobar[i68], zconj(A[n42 + i68])));
                }
            }
        }
    }
    zc prefac = zmk(prefac_gauss / ee->nk_full, 0);
    if (ee->antisym) prefac = zmk(prefac.x * 2, prefac.y * 2);
    for (int i = 0; i < nb4; i++) {
      P1o[i] = zmul(prefac, P1[i]);
      P2o[i] = zmul(prefac, P2[i]);
    }
  }
  free(e); free(table); free(Uih); free(o12); free(o34); free(o14); free(o32); free(mee); free(mex); free(A);
  free(A1rho); free(A1rhobar); free(mtmp); free(P1); free(P2); free(delta);
}

/* elecelec_model::calc_A (ElecElec_Model.h:144-162) on k-points (q1, q2, q3, q4) with calc_ovlp12:
 * calc_delta over e[q1][i1] - e[q2][i2] + e[q3][i3] - e[q4][i4] (:164-184), calc_ovlps (:64-71),
 * calc_mee and, with the exchange term, calc_mee_ex and mee = (mee - mee_ex)/2 (:81-138). Lindblad:
 * A1 = A2 = delta mee. Returns 0 when no band combination conserves energy. */
static int ee_calc_A(const orc_ee* ee, const ee_scr* c, const double* e, int q1, int q2, int q3, int q4, zc* Uih,
                     zc* o12, zc* o34, zc* o14, zc* o32, double* delta, zc* mee, zc* mex, zc* A) {
  const int nb = ee->nb, nb4 = nb * nb * nb * nb;
  const double prefac_exp = -0.25 / pow(ee->degauss, 2);
  int conserved = 0;
  for (int i1 = 0; i1 < nb; i1++)
    for (int i2 = 0; i2 < nb; i2++)
      for (int i3 = 0; i3 < nb; i3++)
        for (int i4 = 0; i4 < nb; i4++) {
          const int i1234 = ((i1 * nb + i2) * nb + i3) * nb + i4;
          const double de = e[q1 * nb + i1] - e[q2 * nb + i2] + e[q3 * nb + i3] - e[q4 * nb + i4];
          if (fabs(de) < ee->ethr) {
            delta[i1234] = exp(prefac_exp * pow(de, 2));
            conserved = 1;
          } else {
            delta[i1234] = 0;
          }
        }
  if (!conserved) return 0;
  ee_ovlp(ee, c, o12, Uih, q1, q2, 1);
  ee_ovlp(ee, c, o34, Uih, q3, q4, 0);
  if (ee->antisym) {
    ee_ovlp(ee, c, o14, Uih, q1, q4, 1);
    ee_ovlp(ee, c, o32, Uih, q3, q2, 0);
  }
  for (int i1 = 0; i1 < nb; i1++)
    for (int i2 = 0; i2 < nb; i2++)
      for (int i3 = 0; i3 < nb; i3++)
        for (int i4 = 0; i4 < nb; i4++) {
          const int i1234 = ((i1 * nb + i2) * nb + i3) * nb + i4;
          mee[i1234] = zmul(o12[i1 * nb + i2], o34[i3 * nb + i4]);
          if (ee->antisym) mex[i1234] = zmul(o14[i1 * nb + i4], o32[i3 * nb + i2]);
        }
  if (ee->antisym)
    for (int i = 0; i < nb4; i++) mee[i] = zadd(zmul(zmk(-0.5, 0), mex[i]), zmul(zmk(0.5, 0), mee[i]));
  for (int i = 0; i < nb4; i++) A[i] = zscale(delta[i], mee[i]);
  return 1;
}

/* elecelec_model::calc_P3P4 and calc_P5P6 (ElecElec_Model_linear.cpp:3-112) for every stored pair
 * (k1, ka) at the occupations f (window [nk][nb]: the f_eq of the linearization) with screening
 * density nfree. P3, P4 are left zero with the exchange term (the reference skips them then). */
void orc_ee_P3P6(const orc_ee* ee, const orc_sys* s, const double* f, double nfree, zc* P3out, zc* P4out, zc* P5out,
                 zc* P6out) {
  const int nk = s->nk, nb = ee->nb, nb2 = nb * nb, nb4 = nb2 * nb2, nd = s->nb_dm, bs = s->bstart;
  const ee_scr c = ee_screen(ee, nfree);
  double* e = (double*)xmalloc(sizeof(double) * nk * nb);
  for (int ik = 0; ik < nk; ik++)
    for (int b = 0; b < nb; b++) e[ik * nb + b] = s->e_dm[(size_t)ik * nd + bs + b];
  const size_t nmesh = (size_t)ee->kmesh[0] * ee->kmesh[1] * ee->kmesh[2];
  int* table = (int*)xmalloc(sizeof(int) * nmesh);
  for (size_t i = 0; i < nmesh; i++) table[i] = -1;
  for (int ik = 0; ik < nk; ik++) {
    int v[3];
    ee_ikvec3(ee, ee->kvec + 3 * ik, v);
    int* slot = &table[((size_t)v[0] * ee->kmesh[1] + v[1]) * ee->kmesh[2] + v[2]];
    if (*slot < 0) *slot = ik;
  }
  zc *Uih = (zc*)xmalloc(sizeof(zc) * nb * ee->nbw), *o12 = (zc*)xmalloc(sizeof(zc) * nb2),
     *o34 = (zc*)xmalloc(sizeof(zc) * nb2), *o14 = (zc*)xmalloc(sizeof(zc) * nb2), *o32 = (zc*)xmalloc(sizeof(zc) * nb2),
     *mee = (zc*)xmalloc(sizeof(zc) * nb4), *mex = (zc*)xmalloc(sizeof(zc) * nb4), *A = (zc*)xmalloc(sizeof(zc) * nb4),
     *A1rho = (zc*)xmalloc(sizeof(zc) * nb2), *A1rhobar = (zc*)xmalloc(sizeof(zc) * nb2);
  double* delta = (double*)xmalloc(sizeof(double) * nb4);
  const double prefac_gauss = 1. / (ee->degauss * sqrt(2. * M_PI));
  zc prefac = zmk(prefac_gauss / ee->nk_full, 0);
  if (ee->antisym) prefac = zmk(prefac.x * 2, prefac.y * 2);
  for (int64_t ip = 0; ip < s->npair; ip++) {
    const int ik1 = (int)s->k1st[ip], ika = (int)s->k2nd[ip];
    zc* P3 = P3out + (size_t)ip * nb4;
    zc* P4 = P4out + (size_t)ip * nb4;
    zc* P5 = P5out + (size_t)ip * nb4;
    zc* P6 = P6out + (size_t)ip * nb4;
    memset(P3, 0, sizeof(zc) * nb4);
    memset(P4, 0, sizeof(zc) * nb4);
    memset(P5, 0, sizeof(zc) * nb4);
    memset(P6, 0, sizeof(zc) * nb4);
    if (!ee->antisym) {
      /* calc_P3P4: k4 = k1 + k3 - ka, A(k1, k4, k3, ka) */
      for (int ik3 = 0; ik3 < nk; ik3++) {
        if (ika == ik3 && !ee->antisym) continue;
        if (ee->antisym && ika == ik3 && ik1 == ika) continue;
        double k4v[3];
        for (int d = 0; d < 3; d++) k4v[d] = ee->kvec[3 * ik1 + d] + ee->kvec[3 * ik3 + d] - ee->kvec[3 * ika + d];
        const int ik4 = ee_findk(ee, table, k4v);
        if (ik4 < 0) continue;
        if (!ee_calc_A(ee, &c, e, ik1, ik4, ik3, ika, Uih, o12, o34, o14, o32, delta, mee, mex, A)) continue;
        const double *f3 = f + (size_t)ik3 * nb, *f4 = f + (size_t)ik4 * nb;
        for (int i1 = 0; i1 < nb; i1++)
          for (int ia = 0; ia < nb; ia++) {
            for (int i4 = 0; i4 < nb; i4++) {
              const int n14 = (i1 * nb + i4) * nb2;
              for (int i3 = 0; i3 < nb; i3++) {
                const int i43 = i4 * nb + i3, i143a = n14 + i3 * nb + ia;
                A1rho[i43] = zscale(f4[i4], zscale(1 - f3[i3], A[i143a]));
                A1rhobar[i43] = zscale(1 - f4[i4], zscale(f3[i3], A[i143a]));
              }
            }
            for (int i2 = 0; i2 < nb; i2++) {
              const int n12 = (i1 * nb + i2) * nb2;
              for (int ib = 0; ib < nb; ib++) {
                const int i12ab = n12 + ia * nb + ib;
                for (int i4 = 0; i4 < nb; i4++) {
                  const int n24 = (i2 * nb + i4) * nb2;
                  for (int i3 = 0; i3 < nb; i3++) {
                    const int i43 = i4 * nb + i3, i243b = n24 + i3 * nb + ib;
                    P3[i12ab] = zadd(P3[i12ab], zmul(A1rho[i43], zconj(A[i243b])));
                    P4[i12ab] = zadd(P4[i12ab], zmul(A1rhobar[i43], zconj(A[i243b])));
                  }
                }
              }
            }
          }
      }
      for (int i = 0; i < nb4; i++) {
        P3[i] = zmul(prefac, P3[i]);
        P4[i] = zmul(prefac, P4[i]);
      }
    }
    /* calc_P5P6: k4 = k1 + ka - k3, A(k1, k3, ka, k4) */
    for (int ik3 = 0; ik3 < nk; ik3++) {
      if (ik1 == ik3 && !ee->antisym) continue;
      if (ee->antisym && ik1 == ik3 && ika == ik3) continue;
      double k4v[3];
      for (int d = 0; d < 3; d++) k4v[d] = ee->kvec[3 * ik1 + d] + ee->kvec[3 * ika + d] - ee->kvec[3 * ik3 + d];
      const int ik4 = ee_findk(ee, table, k4v);
      if (ik4 < 0) continue;
      if (!ee_calc_A(ee, &c, e, ik1, ik3, ika, ik4, Uih, o12, o34, o14, o32, delta, mee, mex, A)) continue;
      const double *f3 = f + (size_t)ik3 * nb, *f4 = f + (size_t)ik4 * nb;
      for (int i1 = 0; i1 < nb; i1++)
        for (int ib = 0; ib < nb; ib++) {
          for (int i3 = 0; i3 < nb; i3++) {
            const int n13 = (i1 * nb + i3) * nb2;
            for (int i4 = 0; i4 < nb; i4++) {
              const int i34 = i3 * nb + i4, i13b4 = n13 + ib * nb + i4;
              A1rho[i34] = zscale(f4[i4], zscale(f3[i3], A[i13b4]));
              A1rhobar[i34] = zscale(1 - f4[i4], zscale(1 - f3[i3], A[i13b4]));
            }
          }
          for (int i2 = 0; i2 < nb; i2++) {
            const int n12 = (i1 * nb + i2) * nb2;
            for (int ia = 0; ia < nb; ia++) {
              const int i12ab = n12 + ia * nb + ib;
              for (int i3 = 0; i3 < nb; i3++) {
                const int n23 = (i2 * nb + i3) * nb2;
                for (int i4 = 0; i4 < nb; i4++) {
                  const int i34 = i3 * nb + i4, i23a4 = n23 + ia * nb + i4;
                  P5[i12ab] = zadd(P5[i12ab], zmul(A1rho[i34], zconj(A[i23a4])));
                  P6[i12ab] = zadd(P6[i12ab], zmul(A1rhobar[i34], zconj(A[i23a4])));
                }
              }
            }
          }
        }
    }
    for (int i = 0; i < nb4; i++) {
      P5[i] = zmul(prefac, P5[i]);
      P6[i] = zmul(prefac, P6[i]);
    }
  }
  free(e); free(table); free(Uih); free(o12); free(o34); free(o14); free(o32); free(mee); free(mex); free(A);
  free(A1rho); free(A1rhobar); free(delta);
}

/* electronphonon::add_Lscij_from_P3_P4 (ElectronPhonon_linear.cpp:199-221) for every pair */
void orc_lsc_add_p3p4(int nb, int64_t npair, const uint64_t* k1, const uint64_t* k2, const zc* P3, const zc* P4,
                      const double* f, zc* Lij, zc* Lji) {
  const int nb2 = nb * nb, nb4 = nb2 * nb2;
  for (int64_t p = 0; p < npair; p++) {
    const int ik = (int)k1[p], jk = (int)k2[p];
    const zc *a3 = P3 + (size_t)p * nb4, *a4 = P4 + (size_t)p * nb4;
    zc *x = Lij + (size_t)p * nb4, *y = Lji + (size_t)p * nb4;
    for (int i1 = 0; i1 < nb; i1++)
      for (int i2 = 0; i2 < nb; i2++) {
        const int i12 = i1 * nb + i2, n12 = i12 * nb2;
        for (int iab = 0; iab < nb2; iab++) {
          const int i12ab = n12 + iab, iab12 = iab * nb2 + i12;
          x[i12ab] = zsub(x[i12ab], zadd(zscale(1 - f[(size_t)ik * nb + i1], a3[i12ab]), zscale(f[(size_t)ik * nb + i2], a4[i12ab])));
          y[i12ab] = zsub(y[i12ab], zadd(zscale(1 - f[(size_t)jk * nb + i1], zconj(a4[iab12])),
                                         zscale(f[(size_t)jk * nb + i2], zconj(a3[iab12]))));
        }
      }
  }
}

/* electronphonon::add_Lscij_from_P5_P6 (ElectronPhonon_linear.cpp:223-245) for every pair */
void orc_lsc_add_p5p6(int nb, int64_t npair, const uint64_t* k1, const uint64_t* k2, const zc* P5, const zc* P6,
                      const double* f, zc* Lij, zc* Lji) {
  const int nb2 = nb * nb, nb4 = nb2 * nb2;
  for (int64_t p = 0; p < npair; p++) {
    const int ik = (int)k1[p], jk = (int)k2[p];
    const zc *a5 = P5 + (size_t)p * nb4, *a6 = P6 + (size_t)p * nb4;
    zc *x = Lij + (size_t)p * nb4, *y = Lji + (size_t)p * nb4;
    for (int i1 = 0; i1 < nb; i1++)
      for (int i2 = 0; i2 < nb; i2++) {
        const int n12 = (i1 * nb + i2) * nb2, i21 = i2 * nb + i1;
        for (int ia = 0; ia < nb; ia++)
          for (int ib = 0; ib < nb; ib++) {
            const int i12ab = n12 + ia * nb + ib, iba21 = (ib * nb + ia) * nb2 + i21;
            x[i12ab] = zsub(x[i12ab], zadd(zscale(1 - f[(size_t)ik * nb + i1], a5[i12ab]), zscale(f[(size_t)ik * nb + i2], a6[i12ab])));
            y[i12ab] = zsub(y[i12ab], zadd(zscale(1 - f[(size_t)jk * nb + i1], a5[iba21]), zscale(f[(size_t)jk * nb + i2], a6[iba21])));
          }
      }
  }
}

/* electronphonon::reset_scatt (ElectronPhonon.cpp:15-42) for the e-e update on state y (the
 * density matrix of all nb_dm bands, in the system's picture) at time t: the window copy, the
 * screening density from its diagonal (coulomb_model::init, Coulomb_Model.h:533-553), the
 * Schrodinger-picture conversion of add_scatt_contrib (ElectronPhonon.cpp:56-66), P_ee, and
 * P = P_base + scale_ee P_ee (ElectronPhonon.cpp:87-100). */
void orc_ee_rebuild(orc_ee* ee, const orc_sys* s, double t, const double* y) {
  const int nk = s->nk, nb = ee->nb, nb2 = nb * nb, nb4 = nb2 * nb2, nd = s->nb_dm, bs = s->bstart;
  const zc* dmx = (const zc*)y;
  zc* dm = (zc*)xmalloc(sizeof(zc) * nk * nb2);
  zc* dm1 = (zc*)xmalloc(sizeof(zc) * nk * nb2);
  for (int ik = 0; ik < nk; ik++)
    for (int i = 0; i < nb; i++)
      for (int j = 0; j < nb; j++) {
        const zc v = dmx[(size_t)ik * nd * nd + (bs + i) * nd + bs + j];
        dm[(size_t)ik * nb2 + i * nb + j] = v;
        dm1[(size_t)ik * nb2 + i * nb + j] = (i == j) ? zsub(zmk(1, 0), v) : zmk(-v.x, -v.y);
      }
  if (ee->update_screening) {
    double n = 0;
    for (int ik = 0; ik < nk; ik++)
      for (int b = 0; b < nb; b++) {
        const double ft = dm[(size_t)ik * nb2 + b * nb + b].x;
        if (b < ee->nv) n += (1 - ft);
        else n += ft;
      }
    ee->nfree = n / (ee->nk_full * ee->cell_size);
  }
  if (!s->picture_schrodinger)
    for (int ik = 0; ik < nk; ik++) {
      const double* e = s->e_dm + (size_t)ik * nd + bs;
      zc* d = dm + (size_t)ik * nb2;
      zc* d1 = dm1 + (size_t)ik * nb2;
      for (int i = 0; i < nb; i++)
        for (int j = i + 1; j < nb; j++) {
          d[i * nb + j] = zmul(d[i * nb + j], zcis((e[j] - e[i]) * t));
          d1[i * nb + j] = zmk(-d[i * nb + j].x, -d[i * nb + j].y);
          d[j * nb + i] = zconj(d[i * nb + j]);
          d1[j * nb + i] = zconj(d1[i * nb + j]);
        }
    }
  orc_ee_P(ee, s, dm, dm1, NULL, ee->nfree, ee->P1ee, ee->P2ee);
  const zc sc = zmk(ee->scale, 0);
  for (size_t i = 0; i < (size_t)s->npair * nb4; i++) {
    const zc a1 = ee->scale != 1. ? zmul(ee->P1ee[i], sc) : ee->P1ee[i];
    const zc a2 = ee->scale != 1. ? zmul(ee->P2ee[i], sc) : ee->P2ee[i];
    ee->P1eff[i] = zadd(a1, ee->P1base[i]);
    ee->P2eff[i] = zadd(a2, ee->P2base[i]);
  }
  free(dm);
  free(dm1);
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
    if (s->ee && s->ee->inside) orc_ee_rebuild(s->ee, s, t, (const double*)dm);  /* update_scatt_inside */
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
