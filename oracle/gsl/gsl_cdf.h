/* GSL-API adapter onto oracle/specfun.c. TEST INFRASTRUCTURE ONLY. */
#ifndef PF_ORACLE_GSL_CDF_H
#define PF_ORACLE_GSL_CDF_H
#include "../specfun.h"
static inline double gsl_cdf_gamma_Pinv(double P, double a, double b) { return b * orc_qgamma(P, a); }
static inline double gsl_cdf_gamma_P(double x, double a, double b) { return orc_pgamma(x / b, a); }
#endif
