/* gsl_odeiv2 subset used by DMD's stepper (DensityMatrix_Dynamics.h:197-224):
 * system struct, the rkf45 step type, and the driver (alloc_y_new / set_hmin / set_hmax / apply /
 * free). The definitions in oracle/gsl_rkf45.c restate GSL 2.6's published algorithm: the
 * Runge-Kutta-Fehlberg 4(5) step, the "standard" step-size control with a_y = 1, a_dydt = 0, the
 * evolve step with one retry per decrease, and the driver loop. Oracle infrastructure only. */
#ifndef ORACLE_SHIM_GSL_ODEIV2_H
#define ORACLE_SHIM_GSL_ODEIV2_H
#include <stddef.h>
#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
  int (*function)(double t, const double y[], double dydt[], void* params);
  int (*jacobian)(double t, const double y[], double* dfdy, double dfdt[], void* params);
  size_t dimension;
  void* params;
} gsl_odeiv2_system;

typedef struct {
  const char* name;
  int can_use_dydt_in;
  int gives_exact_dydt_out;
  unsigned int order;
} gsl_odeiv2_step_type;

extern const gsl_odeiv2_step_type* gsl_odeiv2_step_rkf45;

typedef struct gsl_odeiv2_driver_struct {
  gsl_odeiv2_system sys;
  size_t dim;
  double h, hmin, hmax;
  unsigned long n, nmax;
  double eps_abs, eps_rel, a_y, a_dydt;
  /* evolve state */
  double *y0, *yerr, *dydt_in, *dydt_out;
  unsigned long count, failed_steps;
  double last_step;
  /* step state */
  double *k1, *k2, *k3, *k4, *k5, *k6, *ytmp, *ys0;
  unsigned long nfev; /* right-hand-side evaluations (diagnostic, not part of GSL's API) */
} gsl_odeiv2_driver;

gsl_odeiv2_driver* gsl_odeiv2_driver_alloc_y_new(const gsl_odeiv2_system* sys, const gsl_odeiv2_step_type* T,
                                                 double hstart, double epsabs, double epsrel);
int gsl_odeiv2_driver_set_hmin(gsl_odeiv2_driver* d, double hmin);
int gsl_odeiv2_driver_set_hmax(gsl_odeiv2_driver* d, double hmax);
int gsl_odeiv2_driver_apply(gsl_odeiv2_driver* d, double* t, double t1, double y[]);
void gsl_odeiv2_driver_free(gsl_odeiv2_driver* d);

#ifdef __cplusplus
}
#endif
#endif
