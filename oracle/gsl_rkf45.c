/* CPU restatement of the GSL 2.6 ODE driver that DMD's stepper calls (test infrastructure only).
 *
 * Third-party dependency: GNU Scientific Library 2.6 (make.inc:1, GSL_DIR=.../gsl-2.6), which is
 * not vendored in the reference. Call sites: DensityMatrix_Dynamics.h:197-224
 *   gsl_odeiv2_driver_alloc_y_new(&sys, gsl_odeiv2_step_rkf45, hstart, epsabs, 0.0)
 *   gsl_odeiv2_driver_set_hmin / set_hmax / apply / free.
 * This file restates GSL's published algorithm for exactly those calls:
 *  - step: Runge-Kutta-Fehlberg 4(5) with the Fehlberg tableau; the 5th-order solution is
 *    propagated and the error estimate is the 5th-minus-4th-order difference. The method accepts
 *    dydt_in, so the evolve loop evaluates f(t0, y) once per call and reuses it on retries;
 *    no derivative is evaluated at the step end (6 evaluations per accepted step, as the
 *    reference's own log shows: "ncalls= 6" per output interval).
 *  - control "y_new": D_i = eps_abs + eps_rel*|y_i|; r = max_i |yerr_i| / D_i; if r > 1.1 the
 *    step shrinks by max(0.2, 0.9 r^(-1/5)) and is retried (when that changes t); if r < 0.5 it
 *    grows by min(5, max(1, 0.9 r^(-1/6))).
 *  - driver: loop evolve steps until t reaches t1, clamp |h| to hmax after each step, fail with
 *    GSL_ENOPROG when |h| < hmin.
 * The same arithmetic is implemented on the GPU by the package's adaptive stepper.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include "gsl/gsl_errno.h"
#include "gsl/gsl_odeiv2.h"

static const gsl_odeiv2_step_type rkf45_type = {"rkf45", 1, 0, 5};
const gsl_odeiv2_step_type* gsl_odeiv2_step_rkf45 = &rkf45_type;

/* Fehlberg 4(5) tableau */
static const double ah[] = {1.0 / 4.0, 3.0 / 8.0, 12.0 / 13.0, 1.0, 1.0 / 2.0};
static const double b3[] = {3.0 / 32.0, 9.0 / 32.0};
static const double b4[] = {1932.0 / 2197.0, -7200.0 / 2197.0, 7296.0 / 2197.0};
static const double b5[] = {8341.0 / 4104.0, -32832.0 / 4104.0, 29440.0 / 4104.0, -845.0 / 4104.0};
static const double b6[] = {-6080.0 / 20520.0, 41040.0 / 20520.0, -28352.0 / 20520.0, 9295.0 / 20520.0, -5643.0 / 20520.0};
static const double c1 = 902880.0 / 7618050.0;
static const double c3 = 3953664.0 / 7618050.0;
static const double c4 = 3855735.0 / 7618050.0;
static const double c5 = -1371249.0 / 7618050.0;
static const double c6 = 277020.0 / 7618050.0;
static const double ec[] = {0.0, 1.0 / 360.0, 0.0, -128.0 / 4275.0, -2197.0 / 75240.0, 1.0 / 50.0, 2.0 / 55.0};

static int feval(gsl_odeiv2_driver* d, double t, const double* y, double* f) {
  d->nfev++;
  return d->sys.function(t, y, f, d->sys.params);
}

static int rkf45_apply(gsl_odeiv2_driver* d, double t, double h, double* y, double* yerr, const double* dydt_in) {
  const size_t n = d->dim;
  size_t i;
  int s;
  memcpy(d->ys0, y, n * sizeof(double));
  if (dydt_in) memcpy(d->k1, dydt_in, n * sizeof(double));
  else if ((s = feval(d, t, y, d->k1)) != GSL_SUCCESS) return s;
  for (i = 0; i < n; i++) d->ytmp[i] = y[i] + ah[0] * h * d->k1[i];
  if ((s = feval(d, t + ah[0] * h, d->ytmp, d->k2)) != GSL_SUCCESS) return s;
  for (i = 0; i < n; i++) d->ytmp[i] = y[i] + h * (b3[0] * d->k1[i] + b3[1] * d->k2[i]);
  if ((s = feval(d, t + ah[1] * h, d->ytmp, d->k3)) != GSL_SUCCESS) return s;
  for (i = 0; i < n; i++) d->ytmp[i] = y[i] + h * (b4[0] * d->k1[i] + b4[1] * d->k2[i] + b4[2] * d->k3[i]);
  if ((s = feval(d, t + ah[2] * h, d->ytmp, d->k4)) != GSL_SUCCESS) return s;
  for (i = 0; i < n; i++)
    d->ytmp[i] = y[i] + h * (b5[0] * d->k1[i] + b5[1] * d->k2[i] + b5[2] * d->k3[i] + b5[3] * d->k4[i]);
  if ((s = feval(d, t + ah[3] * h, d->ytmp, d->k5)) != GSL_SUCCESS) return s;
  for (i = 0; i < n; i++)
    d->ytmp[i] = y[i] + h * (b6[0] * d->k1[i] + b6[1] * d->k2[i] + b6[2] * d->k3[i] + b6[3] * d->k4[i] + b6[4] * d->k5[i]);
  if ((s = feval(d, t + ah[4] * h, d->ytmp, d->k6)) != GSL_SUCCESS) return s;
  for (i = 0; i < n; i++) {
    const double di = c1 * d->k1[i] + c3 * d->k3[i] + c4 * d->k4[i] + c5 * d->k5[i] + c6 * d->k6[i];
    y[i] += h * di;
  }
  for (i = 0; i < n; i++)
    yerr[i] = h * (ec[1] * d->k1[i] + ec[3] * d->k3[i] + ec[4] * d->k4[i] + ec[5] * d->k5[i] + ec[6] * d->k6[i]);
  return GSL_SUCCESS;
}

/* 1: decrease, 0: unchanged, 2: increase (the standard control's three outcomes) */
static int std_hadjust(const gsl_odeiv2_driver* d, const double* y, const double* yerr, const double* yp, double* h) {
  const double S = 0.9;
  const double h_old = *h;
  const unsigned int ord = rkf45_type.order;
  double rmax = 2.2250738585072014e-308; /* DBL_MIN */
  for (size_t i = 0; i < d->dim; i++) {
    const double D0 = d->eps_rel * (d->a_y * fabs(y[i]) + d->a_dydt * fabs(h_old * yp[i])) + d->eps_abs;
    const double r = fabs(yerr[i]) / fabs(D0);
    rmax = r > rmax ? r : rmax;
  }
  if (rmax > 1.1) {
    double r = S / pow(rmax, 1.0 / ord);
    if (r < 0.2) r = 0.2;
    *h = r * h_old;
    return 1;
  } else if (rmax < 0.5) {
    double r = S / pow(rmax, 1.0 / (ord + 1.0));
    if (r > 5.0) r = 5.0;
    if (r < 1.0) r = 1.0;
    *h = r * h_old;
    return 2;
  }
  return 0;
}

static int evolve_apply(gsl_odeiv2_driver* d, double* t, double t1, double* h, double* y) {
  const double t0 = *t;
  double h0 = *h;
  const double dt = t1 - t0;
  int final_step, step_status;
  if ((dt < 0.0 && h0 > 0.0) || (dt > 0.0 && h0 < 0.0)) return GSL_EINVAL;
  memcpy(d->y0, y, d->dim * sizeof(double));
  if ((step_status = feval(d, t0, y, d->dydt_in)) != GSL_SUCCESS) return step_status;
try_step:
  if ((dt >= 0.0 && h0 > dt) || (dt < 0.0 && h0 < dt)) {
    h0 = dt;
    final_step = 1;
  } else {
    final_step = 0;
  }
  step_status = rkf45_apply(d, t0, h0, y, d->yerr, d->dydt_in);
  if (step_status != GSL_SUCCESS) {
    const double h_old = h0;
    h0 *= 0.5;
    {
      volatile double t_curr = *t, t_next = (*t) + h0;
      if (fabs(h0) < fabs(h_old) && t_next != t_curr) {
        memcpy(y, d->y0, d->dim * sizeof(double));
        d->failed_steps++;
        goto try_step;
      }
    }
    *h = h0;
    *t = t0;
    return step_status;
  }
  d->count++;
  d->last_step = h0;
  if (final_step) *t = t1;
  else *t = t0 + h0;
  {
    const double h_old = h0;
    const int adj = std_hadjust(d, y, d->yerr, d->dydt_out, &h0);
    if (adj == 1) {
      volatile double t_curr = *t, t_next = (*t) + h0;
      if (fabs(h0) < fabs(h_old) && t_next != t_curr) {
        memcpy(y, d->y0, d->dim * sizeof(double));
        d->failed_steps++;
        goto try_step;
      } else {
        h0 = h_old;
      }
    }
  }
  *h = h0;
  return step_status;
}

gsl_odeiv2_driver* gsl_odeiv2_driver_alloc_y_new(const gsl_odeiv2_system* sys, const gsl_odeiv2_step_type* T,
                                                 double hstart, double epsabs, double epsrel) {
  (void)T;
  gsl_odeiv2_driver* d = (gsl_odeiv2_driver*)calloc(1, sizeof(gsl_odeiv2_driver));
  if (!d) return 0;
  d->sys = *sys;
  d->dim = sys->dimension;
  d->h = hstart;
  d->hmin = 0.0;
  d->hmax = 1.7976931348623157e+308;
  d->nmax = 0;
  d->eps_abs = epsabs;
  d->eps_rel = epsrel;
  d->a_y = 1.0;
  d->a_dydt = 0.0;
  double** bufs[] = {&d->y0, &d->yerr, &d->dydt_in, &d->dydt_out, &d->k1, &d->k2, &d->k3,
                     &d->k4, &d->k5, &d->k6, &d->ytmp, &d->ys0};
  for (size_t i = 0; i < sizeof(bufs) / sizeof(bufs[0]); i++) {
    *bufs[i] = (double*)calloc(d->dim ? d->dim : 1, sizeof(double));
    if (!*bufs[i]) { gsl_odeiv2_driver_free(d); return 0; }
  }
  return d;
}

int gsl_odeiv2_driver_set_hmin(gsl_odeiv2_driver* d, double hmin) {
  if (fabs(hmin) > fabs(d->h) || hmin > d->hmax) return GSL_EINVAL;
  d->hmin = fabs(hmin);
  return GSL_SUCCESS;
}

int gsl_odeiv2_driver_set_hmax(gsl_odeiv2_driver* d, double hmax) {
  if (fabs(hmax) < fabs(d->h) || fabs(hmax) < d->hmin) return GSL_EINVAL;
  if (!(hmax > 0.0 || hmax < 0.0)) return GSL_EINVAL;
  d->hmax = fabs(hmax);
  return GSL_SUCCESS;
}

int gsl_odeiv2_driver_apply(gsl_odeiv2_driver* d, double* t, double t1, double y[]) {
  const int sign = d->h > 0.0 ? 1 : -1;
  d->n = 0;
  if (sign * (t1 - *t) < 0.0) return GSL_EINVAL;
  while (sign * (t1 - *t) > 0.0) {
    int s = evolve_apply(d, t, t1, &d->h, y);
    if (s != GSL_SUCCESS) return s;
    if (d->nmax > 0 && d->n >= d->nmax) return GSL_EMAXITER;
    if (fabs(d->h) > d->hmax) d->h = sign * d->hmax;
    if (fabs(d->h) < d->hmin) return GSL_ENOPROG;
    d->n++;
  }
  return GSL_SUCCESS;
}

void gsl_odeiv2_driver_free(gsl_odeiv2_driver* d) {
  if (!d) return;
  double* bufs[] = {d->y0, d->yerr, d->dydt_in, d->dydt_out, d->k1, d->k2, d->k3,
                    d->k4, d->k5, d->k6, d->ytmp, d->ys0};
  for (size_t i = 0; i < sizeof(bufs) / sizeof(bufs[0]); i++) free(bufs[i]);
  free(d);
}
