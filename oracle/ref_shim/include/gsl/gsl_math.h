/* gsl_math.h subset for the oracle build: the reference only needs M_PI (from <math.h>). */
#ifndef ORACLE_SHIM_GSL_MATH_H
#define ORACLE_SHIM_GSL_MATH_H
#include <math.h>
#define GSL_MAX(a, b) ((a) > (b) ? (a) : (b))
#define GSL_MIN(a, b) ((a) < (b) ? (a) : (b))
#define GSL_DBL_MAX 1.7976931348623157e+308
#endif
