/* GSL-API adapter onto oracle/specfun.c. TEST INFRASTRUCTURE ONLY. */
#ifndef PF_ORACLE_GSL_SF_GAMMA_H
#define PF_ORACLE_GSL_SF_GAMMA_H
#include <math.h>
#include "gsl_errno.h"
#include "../specfun.h"
typedef struct { double val; double err; } gsl_sf_result;
static inline int gsl_sf_gamma_e(double x, gsl_sf_result *r)
{
	double v = orc_gammafn(x);
	r->val = v;
	r->err = 0;
	if (isnan(v)) return GSL_EDOM;
	if (isinf(v)) return GSL_EOVRFLW;
	if (v == 0) return GSL_EUNDRFLW;
	return GSL_SUCCESS;
}
static inline int gsl_sf_beta_e(double a, double b, gsl_sf_result *r)
{
	double v = orc_beta(a, b);
	r->val = v;
	r->err = 0;
	if (isnan(v)) return GSL_EDOM;
	if (v == 0) return GSL_EUNDRFLW;
	return GSL_SUCCESS;
}
#endif
