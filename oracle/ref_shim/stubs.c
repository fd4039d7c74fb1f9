/* Link stubs for reference code paths the oracle never enables (test infrastructure only).
 *
 * - GSL quadrature and root finding: only the model screening / model e-imp / e-e code in
 *   scattering_model/Coulomb_Model.h:200-348 calls them (scrMode != none). They abort loudly.
 * - LAPACK names declared in comm/mymatrix.h:11-31 other than zheevr_ (which oracle/ref_shim/
 *   zheevr_shim.c provides) belong to analysis routines the oracle does not call. They abort.
 */
#include <stdio.h>
#include <stdlib.h>
#include "gsl/gsl_errno.h"
#include "gsl/gsl_integration.h"
#include "gsl/gsl_roots.h"

static void die(const char* what) {
  fprintf(stderr, "oracle reference build: %s is not available (model screening / LAPACK analysis path)\n", what);
  abort();
}

static gsl_error_handler_t* g_handler = 0;
gsl_error_handler_t* gsl_set_error_handler_off(void) { gsl_error_handler_t* p = g_handler; g_handler = 0; return p; }

gsl_integration_workspace* gsl_integration_workspace_alloc(size_t n) { (void)n; die("gsl_integration_workspace_alloc"); return 0; }
void gsl_integration_workspace_free(gsl_integration_workspace* w) { (void)w; }
int gsl_integration_qagiu(const gsl_function* f, double a, double ea, double er, size_t l, gsl_integration_workspace* w, double* r, double* e) {
  (void)f; (void)a; (void)ea; (void)er; (void)l; (void)w; (void)r; (void)e; die("gsl_integration_qagiu"); return 0;
}
int gsl_integration_qagp(const gsl_function* f, double* p, size_t np, double ea, double er, size_t l, gsl_integration_workspace* w, double* r, double* e) {
  (void)f; (void)p; (void)np; (void)ea; (void)er; (void)l; (void)w; (void)r; (void)e; die("gsl_integration_qagp"); return 0;
}
int gsl_integration_qag(const gsl_function* f, double a, double b, double ea, double er, size_t l, int key, gsl_integration_workspace* w, double* r, double* e) {
  (void)f; (void)a; (void)b; (void)ea; (void)er; (void)l; (void)key; (void)w; (void)r; (void)e; die("gsl_integration_qag"); return 0;
}

static const gsl_root_fsolver_type brent_type = {"brent"};
const gsl_root_fsolver_type* gsl_root_fsolver_brent = &brent_type;
gsl_root_fsolver* gsl_root_fsolver_alloc(const gsl_root_fsolver_type* T) { (void)T; die("gsl_root_fsolver_alloc"); return 0; }
int gsl_root_fsolver_set(gsl_root_fsolver* s, gsl_function* f, double lo, double hi) { (void)s; (void)f; (void)lo; (void)hi; die("gsl_root_fsolver_set"); return 0; }
int gsl_root_fsolver_iterate(gsl_root_fsolver* s) { (void)s; die("gsl_root_fsolver_iterate"); return 0; }
double gsl_root_fsolver_root(const gsl_root_fsolver* s) { (void)s; die("gsl_root_fsolver_root"); return 0; }
double gsl_root_fsolver_x_lower(const gsl_root_fsolver* s) { (void)s; die("gsl_root_fsolver_x_lower"); return 0; }
double gsl_root_fsolver_x_upper(const gsl_root_fsolver* s) { (void)s; die("gsl_root_fsolver_x_upper"); return 0; }
const char* gsl_root_fsolver_name(const gsl_root_fsolver* s) { (void)s; return "brent"; }
void gsl_root_fsolver_free(gsl_root_fsolver* s) { (void)s; }
int gsl_root_test_interval(double lo, double hi, double ea, double er) { (void)lo; (void)hi; (void)ea; (void)er; die("gsl_root_test_interval"); return 0; }

void zgeev_(void) { die("zgeev_"); }
void zgesdd_(void) { die("zgesdd_"); }
void zgesvd_(void) { die("zgesvd_"); }
void zgetrf_(void) { die("zgetrf_"); }
void zgetri_(void) { die("zgetri_"); }
void zposv_(void) { die("zposv_"); }
