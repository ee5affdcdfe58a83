/* GSL-API adapter onto oracle/specfun.c (QUADPACK restatement).
 * TEST INFRASTRUCTURE ONLY. */
#ifndef PF_ORACLE_GSL_INTEGRATION_H
#define PF_ORACLE_GSL_INTEGRATION_H
#include <stdlib.h>
#include "../specfun.h"
typedef struct { double (*function)(double x, void *params); void *params; } gsl_function;
typedef struct { size_t limit; } gsl_integration_workspace;
static inline gsl_integration_workspace *gsl_integration_workspace_alloc(size_t n)
{
	gsl_integration_workspace *w = (gsl_integration_workspace *)malloc(sizeof(*w));
	w->limit = n;
	return w;
}
static inline void gsl_integration_workspace_free(gsl_integration_workspace *w) { free(w); }
static inline int gsl_integration_qags(const gsl_function *f, double a, double b, double epsabs,
                                       double epsrel, size_t limit, gsl_integration_workspace *w,
                                       double *result, double *abserr)
{
	int ier = 0;
	(void)w;
	*result = orc_qags(f->function, f->params, a, b, epsabs, epsrel, (int)limit, &ier, abserr);
	return ier;
}
static inline int gsl_integration_qagiu(gsl_function *f, double a, double epsabs, double epsrel,
                                        size_t limit, gsl_integration_workspace *w,
                                        double *result, double *abserr)
{
	int ier = 0;
	(void)w;
	*result = orc_qagiu(f->function, f->params, a, epsabs, epsrel, (int)limit, &ier, abserr);
	return ier;
}
#endif
