/*
 * Oracle special functions: TEST INFRASTRUCTURE ONLY.
 *
 * libprofit takes its special functions from GSL (src/utils.cpp:109-186):
 *   qgamma  -> gsl_cdf_gamma_Pinv(p, shape, 1)      (src/utils.cpp:109-111)
 *   pgamma  -> gsl_cdf_gamma_P(q, shape, 1)         (src/utils.cpp:113-115)
 *   gammafn -> gsl_sf_gamma_e                       (src/utils.cpp:117-132)
 *   beta    -> gsl_sf_beta_e                        (src/utils.cpp:134-153)
 *   integrate_qagi / integrate_qags -> gsl_integration_qagiu / qags with
 *     epsabs = epsrel = 1e-4 and a 100-interval workspace (src/utils.cpp:155-186)
 * GSL (no version pinned by the reference's CMakeLists.txt:81-98) is not
 * vendored and is absent from this machine, so this file restates the
 * published algorithms GSL implements:
 *   - Gamma / log-Gamma: the C99 libm tgamma / lgamma.
 *   - Regularised incomplete gamma P(a,x), Q(a,x): the power series for
 *     x < a+1 and the Legendre continued fraction (modified Lentz) otherwise
 *     (DLMF 8.7.1, 8.9.2).
 *   - Inverse P: Wilson-Hilferty start (DLMF 8.10.11 style normal
 *     approximation), refined with Halley steps on P (or on Q for p > 0.5).
 *   - QAGS / QAGIU: QUADPACK dqagse / dqagie (Piessens, de Doncker-Kapenga,
 *     Ueberhuber, Kahaner 1983): 21-point (15-point for the transformed
 *     semi-infinite range) Gauss-Kronrod, adaptive bisection and Wynn's
 *     epsilon extrapolation (dqelg), error list kept by dqpsrt.
 * Parity of these values with real GSL is unpinned by the reference's own
 * tests; they are cross-checked against scipy in tests/.
 */
#ifndef PF_ORACLE_SPECFUN_H
#define PF_ORACLE_SPECFUN_H

#ifdef __cplusplus
extern "C" {
#endif

typedef double (*orc_integrand)(double x, void *ctx);

double orc_gammafn(double x);
double orc_lgammafn(double x);
double orc_beta(double a, double b);
double orc_pgamma(double x, double a);            /* P(a, x), scale 1 */
double orc_qgamma_upper(double x, double a);      /* Q(a, x) = 1 - P  */
double orc_qgamma(double p, double a);            /* inverse of P      */
/* status: 0 ok, >0 QUADPACK ier code (result still returned) */
double orc_qags(orc_integrand f, void *ctx, double a, double b,
                double epsabs, double epsrel, int limit, int *ier, double *abserr);
double orc_qagiu(orc_integrand f, void *ctx, double a,
                 double epsabs, double epsrel, int limit, int *ier, double *abserr);

#ifdef __cplusplus
}
#endif

#endif
