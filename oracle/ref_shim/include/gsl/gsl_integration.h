/* Declarations for the GSL quadrature calls in Coulomb_Model.h:200-348 (model screening and
 * model e-imp/e-e, which the oracle never enables). The oracle build's definitions abort. */
#ifndef ORACLE_SHIM_GSL_INTEGRATION_H
#define ORACLE_SHIM_GSL_INTEGRATION_H
#include <stddef.h>
#ifdef __cplusplus
extern "C" {
#endif
typedef struct { double (*function)(double x, void* params); void* params; } gsl_function;
typedef struct { size_t limit; } gsl_integration_workspace;
gsl_integration_workspace* gsl_integration_workspace_alloc(size_t n);
void gsl_integration_workspace_free(gsl_integration_workspace* w);
int gsl_integration_qagiu(const gsl_function* f, double a, double epsabs, double epsrel, size_t limit,
                          gsl_integration_workspace* w, double* result, double* abserr);
int gsl_integration_qagp(const gsl_function* f, double* pts, size_t npts, double epsabs, double epsrel,
                         size_t limit, gsl_integration_workspace* w, double* result, double* abserr);
int gsl_integration_qag(const gsl_function* f, double a, double b, double epsabs, double epsrel, size_t limit,
                        int key, gsl_integration_workspace* w, double* result, double* abserr);
#ifdef __cplusplus
}
#endif
#endif
