// Device FP64 special functions for the per-profile setup kernel.
//
// libprofit obtains these from GSL on the host (src/utils.cpp:109-186):
//   qgamma(p, a)   = gsl_cdf_gamma_Pinv(p, a, 1)   bn, flux fractions
//   pgamma(x, a)   = gsl_cdf_gamma_P(x, a, 1)      sersic rescale_flux
//   gammafn(x)     = gsl_sf_gamma_e                sersic luminosity
//   beta(a, b)     = gsl_sf_beta_e                 boxiness r_box, ferrer luminosity
//   integrate_qagi / integrate_qags (epsabs = epsrel = 1e-4, 100 intervals)
//                                                  coresersic, brokenexp, king luminosity
// Here they run on the GPU, one thread per profile, from the published methods:
//   * Gamma / log-Gamma: CUDA's tgamma / lgamma.
//   * P(a,x), Q(a,x): power series (DLMF 8.7.1) for x < a+1, else the Legendre
//     continued fraction (DLMF 8.9.2) evaluated with the modified Lentz method.
//   * P^-1: bracketing by doubling, then safeguarded Halley steps on P (on Q
//     above the median for conditioning).
//   * QAGS / QAGIU: QUADPACK dqagse / dqagie (Piessens et al. 1983): 21-point
//     Gauss-Kronrod (15-point on the transformed half-line), adaptive
//     bisection, Wynn epsilon extrapolation (dqelg), ordered error list (dqpsrt).
// Arrays in the QUADPACK part are 1-based like the published algorithm.
#pragma once

#include <cfloat>
#include <math_constants.h>
#include <cmath>

namespace pf {
namespace sf {

__device__ __forceinline__ double dmax(double a, double b) { return a > b ? a : b; }
__device__ __forceinline__ double dmin(double a, double b) { return a < b ? a : b; }

__device__ inline double gammafn(double x)
{
	if (x == 0.0 || (x < 0.0 && x == floor(x))) {
		return CUDART_NAN;
	}
	return tgamma(x);
}

__device__ inline double beta(double a, double b)
{
	if (a < 0. || b < 0.) {
		return CUDART_NAN;
	}
	if (a == 0. || b == 0.) {
		return CUDART_INF;
	}
	if (a + b < 170.) {
		return tgamma(a) * tgamma(b) / tgamma(a + b);
	}
	return exp(lgamma(a) + lgamma(b) - lgamma(a + b));
}

// Digamma psi(x) for x > 0: upward recurrence psi(x) = psi(x+1) - 1/x to
// x >= 10, then the asymptotic series ln x - 1/(2x) - sum B_2k / (2k x^2k)
// (DLMF 5.15.8, 5.11.2) through the x^-12 term.
__device__ inline double digamma(double x)
{
	double acc = 0.;
	while (x < 10.) {
		acc -= 1. / x;
		x += 1.;
	}
	const double r = 1. / x, r2 = r * r;
	const double series = r2 * (1. / 12 - r2 * (1. / 120 - r2 * (1. / 252 - r2 * (1. / 240 - r2 * (1. / 132)))));
	return acc + log(x) - 0.5 * r - series;
}

// P(a, x) = x^a e^-x / Gamma(a + 1) sum_n x^n / ((a + 1) ... (a + n)): the
// terms' ratios x / (a + n) taken four at a time, so that their divisions
// (hundreds of cycles each in FP64 on this GPU) run side by side instead of
// on the running product's dependency chain; the terms, the sum and the stop
// are the one-at-a-time loop's, in its order.
__device__ inline double pgamma_series(double a, double x, double lga1)
{
	double ap = a, term = 1., sum = 1.;
	int n = 1;
	while (n < 2000) {
		double ratio[4];
#pragma unroll
		for (int q = 0; q < 4; q++) {
			ap += 1.;
			ratio[q] = x / ap;
		}
		bool done = false;
#pragma unroll
		for (int q = 0; q < 4; q++) {
			term *= ratio[q];
			sum += term;
			n++;
			if (fabs(term) < fabs(sum) * DBL_EPSILON || n >= 2000) {
				done = true;
				break;
			}
		}
		if (done) break;
	}
	return exp(a * log(x) - x - lga1) * sum;
}

__device__ inline double pgamma_series(double a, double x) { return pgamma_series(a, x, lgamma(a + 1.)); }

// Q(a, x) = x^a e^-x / Gamma(a) / (b_0 + a_1 / (b_1 + a_2 / (b_2 + ...))),
// b_i = x + 2i + 1 - a, a_i = -i (i - a), for x >= a + 1. The continued
// fraction by the three-term recurrence of its convergents A_i / B_i
// (A_i = b_i A_{i-1} + a_i A_{i-2}, the same for B; the Wallis form),
// rescaled by exact powers of two against overflow: two multiply-adds per
// term on the dependency chain instead of two divisions; converged when four
// more terms move B / A by less than 2 eps relative.
__device__ inline double qgamma_cf(double a, double x, double lga)
{
	double b = x + 1. - a;
	double A2 = 1., A1 = b, B2 = 0., B1 = 1.;  // A_{i-2}, A_{i-1}, B_{i-2}, B_{i-1}
	double f = B1 / A1;
	for (int i = 1; i < 2000; i += 4) {
#pragma unroll
		for (int q = 0; q < 4; q++) {
			const double an = -(double)(i + q) * ((double)(i + q) - a);
			b += 2.;
			const double A = b * A1 + an * A2, B = b * B1 + an * B2;
			A2 = A1;
			A1 = A;
			B2 = B1;
			B1 = B;
		}
		// both convergents' pairs scaled by the same power of two: exact
		int e;
		frexp(A1, &e);
		if (e > 600 || e < -600) {
			A1 = ldexp(A1, -e);
			A2 = ldexp(A2, -e);
			B1 = ldexp(B1, -e);
			B2 = ldexp(B2, -e);
		}
		const double fn = B1 / A1;
		if (fabs(fn - f) <= 2. * DBL_EPSILON * fabs(fn)) {
			f = fn;
			break;
		}
		f = fn;
	}
	return exp(a * log(x) - x - lga) * f;
}

__device__ inline double qgamma_cf(double a, double x) { return qgamma_cf(a, x, lgamma(a)); }

__device__ inline double pgamma(double x, double a)
{
	if (x <= 0.) return 0.;
	if (isinf(x)) return 1.;
	if (x < a + 1.) return pgamma_series(a, x);
	return 1. - qgamma_cf(a, x);
}

__device__ inline double qgamma_upper(double x, double a)
{
	if (x <= 0.) return 1.;
	if (isinf(x)) return 0.;
	if (x < a + 1.) return 1. - pgamma_series(a, x);
	return qgamma_cf(a, x);
}

// Starting point for bn = P^-1(1/2, 2n): the asymptotic series of Ciotti &
// Bertin (1999, A&A 352, 447), eq. 18; refined to full precision by qgamma.
__device__ inline double bn_guess(double n)
{
	if (n < 0.36) return -1.;
	const double r = 1. / n;
	return 2 * n - 1. / 3 + r * (4. / 405 + r * (46. / 25515 + r * (131. / 1148175 - r * (2194697. / 30690717750.))));
}

// Starting point for P^-1(p, a), a >= 1: the Wilson-Hilferty cube-root normal
// approximation x = a (1 - 1/(9a) + z / (3 sqrt(a)))^3, z the standard normal
// quantile of p (= sqrt(2) erfcinv(2 (1 - p))); relative error ~1e-3 for the
// shapes used here, refined to full precision by qgamma.
__device__ inline double wilson_hilferty_guess(double p, double a)
{
	if (a < 1. || !(p > 0.) || !(p < 1.)) return -1.;
	const double z = 1.4142135623730951 * erfcinv(2. * (1. - p));
	const double t = 1. - 1. / (9. * a) + z / (3. * sqrt(a));
	if (!(t > 0.)) return -1.;
	return a * t * t * t;
}

// Inverse of P(a, .) by safeguarded Halley iterations on f(x) = P(a, x) - p
// (Q(a, x) - q for p > 1/2), one evaluation of f per iteration. With a usable
// starting point (guess > 0) the iteration starts there, the bracket [lo, hi]
// of the root growing from (0, +inf) as the signs of f are seen; without one,
// the root is first bracketed by doubling from max(a, 1). A step that leaves
// the bracket is replaced by bisection (or by doubling while hi is unknown).
// The iteration stops when a Halley step moves x by less than 1e-7 relative
// (cubic convergence: the next step would be below 1e-20) or by less than
// 4 eps, or when f is exactly 0.
__device__ inline double qgamma(double p, double a, double guess = -1.)
{
	if (!(p > 0.)) return 0.;
	if (p >= 1.) return CUDART_INF;
	const bool use_q = p > 0.5;
	const double q = 1. - p;
	double lo = 0., hi = CUDART_INF;
	double x;
	if (guess > 0.) {
		x = guess;
	}
	else {
		hi = a > 1. ? a : 1.;
		for (int it = 0; it < 2000; it++) {
			bool below = use_q ? (qgamma_upper(hi, a) > q) : (pgamma(hi, a) < p);
			if (!below) break;
			lo = hi;
			hi *= 2.;
		}
		x = a;
		if (!(x > lo && x < hi)) x = 0.5 * (lo + hi);
	}
	// log Gamma(a) and log Gamma(a + 1) once for all the iterations' P and Q
	// (each from lgamma itself: the solves feed ceilings, src/sersic.cpp:
	// 262-276, so they stay as close to the reference's values as lgamma is)
	const double lga = lgamma(a), lga1 = lgamma(a + 1.);
	for (int it = 0; it < 200; it++) {
		double f;
		if (!(x > 0.)) f = use_q ? q - 1. : -p;
		else if (isinf(x)) f = use_q ? q : 1. - p;
		else if (x < a + 1.) f = use_q ? (q - (1. - pgamma_series(a, x, lga1))) : (pgamma_series(a, x, lga1) - p);
		else f = use_q ? (q - qgamma_cf(a, x, lga)) : ((1. - qgamma_cf(a, x, lga)) - p);
		if (f == 0.) break;
		if (f < 0.) lo = x; else hi = x;
		const double pdf = exp((a - 1.) * log(x) - x - lga);
		double dx = f / pdf;
		const double t = 0.5 * dx * ((a - 1.) / x - 1.);
		const bool halley = fabs(t) < 0.5;
		if (halley) dx = dx / (1. - t);
		double xn = x - dx;
		if (!(xn > lo && xn < hi)) {
			xn = isinf(hi) ? 2. * x : 0.5 * (lo + hi);
		}
		const double step = fabs(xn - x);
		x = xn;
		if (step <= 4. * DBL_EPSILON * xn || (halley && step <= 1e-7 * xn)) break;
	}
	return x;
}

// ------------------------------------------------------------- QUADPACK

struct GK {
	static __device__ __forceinline__ double xgk21(int i)
	{
		switch (i) {
		case 1: return 0.995657163025808080735527280689003;
		case 2: return 0.973906528517171720077964012084452;
		case 3: return 0.930157491355708226001207180059508;
		case 4: return 0.865063366688984510732096688423493;
		case 5: return 0.780817726586416897063717578345042;
		case 6: return 0.679409568299024406234327365114874;
		case 7: return 0.562757134668604683339000099272694;
		case 8: return 0.433395394129247190799265943165784;
		case 9: return 0.294392862701460198131126603103866;
		case 10: return 0.148874338981631210884826001129720;
		default: return 0.0;
		}
	}
	static __device__ __forceinline__ double wgk21(int i)
	{
		switch (i) {
		case 1: return 0.011694638867371874278064396062192;
		case 2: return 0.032558162307964727478818972459390;
		case 3: return 0.054755896574351996031381300244580;
		case 4: return 0.075039674810919952767043140916190;
		case 5: return 0.093125454583697605535065465083366;
		case 6: return 0.109387158802297641899210590325805;
		case 7: return 0.123491976262065851077208608978567;
		case 8: return 0.134709217311473325928054001771707;
		case 9: return 0.142775938577060080797094273138717;
		case 10: return 0.147739104901338491374841515972068;
		default: return 0.149445554002916905664936468389821;
		}
	}
	static __device__ __forceinline__ double wg10(int i)
	{
		switch (i) {
		case 1: return 0.066671344308688137593568809893332;
		case 2: return 0.149451349150580593145776339657697;
		case 3: return 0.219086362515982043995534934228163;
		case 4: return 0.269266719309996355091226921569469;
		default: return 0.295524224714752870173892994651338;
		}
	}
	static __device__ __forceinline__ double xgk15(int i)
	{
		switch (i) {
		case 1: return 0.991455371120812639206854697526329;
		case 2: return 0.949107912342758524526189684047851;
		case 3: return 0.864864423359769072789712788640926;
		case 4: return 0.741531185599394439863864773280788;
		case 5: return 0.586087235467691130294144845693013;
		case 6: return 0.405845151377397166906606412076961;
		case 7: return 0.207784955007898467600689403773245;
		default: return 0.0;
		}
	}
	static __device__ __forceinline__ double wgk15(int i)
	{
		switch (i) {
		case 1: return 0.022935322010529224963732008058970;
		case 2: return 0.063092092629978553290700663189204;
		case 3: return 0.104790010322250183839876322541518;
		case 4: return 0.140653259715525918745189590510238;
		case 5: return 0.169004726639267902826583426598550;
		case 6: return 0.190350578064785409913256402421014;
		case 7: return 0.204432940075298892414161999234649;
		default: return 0.209482141084727828012999174891714;
		}
	}
	static __device__ __forceinline__ double wg7(int i)
	{
		switch (i) {
		case 2: return 0.129484966168869693270611432679082;
		case 4: return 0.279705391489276667901467771423780;
		case 6: return 0.381830050505118944950369775488975;
		case 8: return 0.417959183673469387755102040816327;
		default: return 0.0;
		}
	}
};

__device__ inline double qk_error(double resk, double resg, double hlgth, double resabs, double resasc)
{
	double abserr = fabs((resk - resg) * hlgth);
	if (resasc != 0. && abserr != 0.) {
		abserr = resasc * dmin(1., pow(200. * abserr / resasc, 1.5));
	}
	if (resabs > DBL_MIN / (50. * DBL_EPSILON)) {
		abserr = dmax(DBL_EPSILON * 50. * resabs, abserr);
	}
	return abserr;
}

template <typename F>
__device__ void qk21(const F &f, double a, double b, double *result, double *abserr,
                     double *resabs, double *resasc)
{
	double fv1[11], fv2[11];
	double centr = 0.5 * (a + b), hlgth = 0.5 * (b - a), dhlgth = fabs(hlgth);
	double resg = 0., fc = f(centr), resk = GK::wgk21(11) * fc;
	*resabs = fabs(resk);
	for (int j = 1; j <= 5; j++) {
		int jtw = 2 * j;
		double absc = hlgth * GK::xgk21(jtw);
		double fval1 = f(centr - absc), fval2 = f(centr + absc);
		double fsum = fval1 + fval2;
		fv1[jtw] = fval1;
		fv2[jtw] = fval2;
		resg += GK::wg10(j) * fsum;
		resk += GK::wgk21(jtw) * fsum;
		*resabs += GK::wgk21(jtw) * (fabs(fval1) + fabs(fval2));
	}
	for (int j = 1; j <= 5; j++) {
		int jtwm1 = 2 * j - 1;
		double absc = hlgth * GK::xgk21(jtwm1);
		double fval1 = f(centr - absc), fval2 = f(centr + absc);
		double fsum = fval1 + fval2;
		fv1[jtwm1] = fval1;
		fv2[jtwm1] = fval2;
		resk += GK::wgk21(jtwm1) * fsum;
		*resabs += GK::wgk21(jtwm1) * (fabs(fval1) + fabs(fval2));
	}
	double reskh = resk * 0.5;
	*resasc = GK::wgk21(11) * fabs(fc - reskh);
	for (int j = 1; j <= 10; j++) {
		*resasc += GK::wgk21(j) * (fabs(fv1[j] - reskh) + fabs(fv2[j] - reskh));
	}
	*result = resk * hlgth;
	*resabs *= dhlgth;
	*resasc *= dhlgth;
	*abserr = qk_error(resk, resg, hlgth, *resabs, *resasc);
}

template <typename F>
__device__ void qk15i(const F &f, double boun, double a, double b, double *result, double *abserr,
                      double *resabs, double *resasc)
{
	double fv1[8], fv2[8];
	double centr = 0.5 * (a + b), hlgth = 0.5 * (b - a);
	double tabsc1 = boun + (1. - centr) / centr;
	double fval1 = f(tabsc1);
	double fc = (fval1 / centr) / centr;
	double resg = GK::wg7(8) * fc, resk = GK::wgk15(8) * fc;
	*resabs = fabs(resk);
	for (int j = 1; j <= 7; j++) {
		double absc = hlgth * GK::xgk15(j);
		double absc1 = centr - absc, absc2 = centr + absc;
		double t1 = boun + (1. - absc1) / absc1, t2 = boun + (1. - absc2) / absc2;
		double f1 = f(t1), f2 = f(t2);
		f1 = (f1 / absc1) / absc1;
		f2 = (f2 / absc2) / absc2;
		fv1[j] = f1;
		fv2[j] = f2;
		double fsum = f1 + f2;
		resg += GK::wg7(j) * fsum;
		resk += GK::wgk15(j) * fsum;
		*resabs += GK::wgk15(j) * (fabs(f1) + fabs(f2));
	}
	double reskh = resk * 0.5;
	*resasc = GK::wgk15(8) * fabs(fc - reskh);
	for (int j = 1; j <= 7; j++) {
		*resasc += GK::wgk15(j) * (fabs(fv1[j] - reskh) + fabs(fv2[j] - reskh));
	}
	*result = resk * hlgth;
	*resasc *= hlgth;
	*resabs *= hlgth;
	*abserr = qk_error(resk, resg, hlgth, *resabs, *resasc);
}

constexpr int kQuadLimit = 100;

__device__ inline void qpsrt(int limit, int last, int *maxerr, double *ermax, const double *elist,
                             int *iord, int *nrmax)
{
	if (last <= 2) {
		iord[1] = 1;
		iord[2] = 2;
	}
	else {
		double errmax = elist[*maxerr];
		if (*nrmax != 1) {
			int ido = *nrmax - 1;
			for (int i = 1; i <= ido; i++) {
				int isucc = iord[*nrmax - 1];
				if (errmax <= elist[isucc]) break;
				iord[*nrmax] = isucc;
				(*nrmax)--;
			}
		}
		int jupbn = last;
		if (last > (limit / 2 + 2)) jupbn = limit + 3 - last;
		double errmin = elist[last];
		int jbnd = jupbn - 1;
		int ibeg = *nrmax + 1;
		bool inserted = false;
		for (int i = ibeg; i <= jbnd; i++) {
			int isucc = iord[i];
			if (errmax >= elist[isucc]) {
				iord[i - 1] = *maxerr;
				int k = jbnd;
				bool placed = false;
				for (int j = i; j <= jbnd; j++) {
					int is2 = iord[k];
					if (errmin < elist[is2]) {
						iord[k + 1] = last;
						placed = true;
						break;
					}
					iord[k + 1] = is2;
					k--;
				}
				if (!placed) iord[i] = last;
				inserted = true;
				break;
			}
			iord[i - 1] = isucc;
		}
		if (!inserted) {
			iord[jbnd] = *maxerr;
			iord[jupbn] = last;
		}
	}
	*maxerr = iord[*nrmax];
	*ermax = elist[*maxerr];
}

__device__ inline void qelg(int *n, double *epstab, double *result, double *abserr, double *res3la, int *nres)
{
	const int limexp = 50;
	(*nres)++;
	*abserr = DBL_MAX;
	*result = epstab[*n];
	if (*n < 3) {
		*abserr = dmax(*abserr, 5. * DBL_EPSILON * fabs(*result));
		return;
	}
	epstab[*n + 2] = epstab[*n];
	int newelm = (*n - 1) / 2;
	epstab[*n] = DBL_MAX;
	int num = *n;
	int k1 = *n;
	for (int i = 1; i <= newelm; i++) {
		int k2 = k1 - 1, k3 = k1 - 2;
		double res = epstab[k1 + 2];
		double e0 = epstab[k3], e1 = epstab[k2], e2 = res;
		double e1abs = fabs(e1);
		double delta2 = e2 - e1, err2 = fabs(delta2);
		double tol2 = dmax(fabs(e2), e1abs) * DBL_EPSILON;
		double delta3 = e1 - e0, err3 = fabs(delta3);
		double tol3 = dmax(e1abs, fabs(e0)) * DBL_EPSILON;
		if (err2 <= tol2 && err3 <= tol3) {
			*result = res;
			*abserr = err2 + err3;
			*abserr = dmax(*abserr, 5. * DBL_EPSILON * fabs(*result));
			return;
		}
		double e3 = epstab[k1];
		epstab[k1] = e1;
		double delta1 = e1 - e3, err1 = fabs(delta1);
		double tol1 = dmax(e1abs, fabs(e3)) * DBL_EPSILON;
		if (err1 <= tol1 || err2 <= tol2 || err3 <= tol3) {
			*n = i + i - 1;
			break;
		}
		double ss = 1. / delta1 + 1. / delta2 - 1. / delta3;
		double epsinf = fabs(ss * e1);
		if (!(epsinf > 1e-4)) {
			*n = i + i - 1;
			break;
		}
		res = e1 + 1. / ss;
		epstab[k1] = res;
		k1 -= 2;
		double error = err2 + fabs(res - e2) + err3;
		if (error > *abserr) continue;
		*abserr = error;
		*result = res;
	}
	if (*n == limexp) *n = 2 * (limexp / 2) - 1;
	int ib = (num % 2 == 0) ? 2 : 1;
	int ie = newelm + 1;
	for (int i = 1; i <= ie; i++) {
		int ib2 = ib + 2;
		epstab[ib] = epstab[ib2];
		ib = ib2;
	}
	if (num != *n) {
		int indx = num - *n + 1;
		for (int i = 1; i <= *n; i++) {
			epstab[i] = epstab[indx];
			indx++;
		}
	}
	if (*nres < 4) {
		res3la[*nres] = *result;
		*abserr = DBL_MAX;
	}
	else {
		*abserr = fabs(*result - res3la[3]) + fabs(*result - res3la[2]) + fabs(*result - res3la[1]);
		res3la[1] = res3la[2];
		res3la[2] = res3la[3];
		res3la[3] = *result;
	}
	*abserr = dmax(*abserr, 5. * DBL_EPSILON * fabs(*result));
}

// dqagse (infinite == false, rule qk21 on [a,b]) or dqagie with inf = 1
// (infinite == true, rule qk15i on t in (0,1], x = a + (1-t)/t).
template <typename F>
__device__ double qag(const F &f, double a, double b, bool infinite, double epsabs, double epsrel,
                      int *ier_out)
{
	const int limit = kQuadLimit;
	double alist[kQuadLimit + 2], blist[kQuadLimit + 2], rlist[kQuadLimit + 2], elist[kQuadLimit + 2];
	int iord[kQuadLimit + 2];
	double rlist2[55], res3la[4];
	for (int i = 0; i < 55; i++) rlist2[i] = 0.;
	for (int i = 0; i < 4; i++) res3la[i] = 0.;
	for (int i = 0; i < kQuadLimit + 2; i++) {
		alist[i] = blist[i] = rlist[i] = elist[i] = 0.;
		iord[i] = 0;
	}
	const double epmach = DBL_EPSILON;
	double boun = a, lo = a, hi = b;
	if (infinite) {
		lo = 0.;
		hi = 1.;
	}
	double area = 0., area1, area12, area2, a1, a2, b1, b2, correc = 0., defabs, defab1, defab2;
	double dres, erlarg = 0., erlast, errbnd, errmax = 0., error1, error2, erro12;
	double errsum = 0., ertest = 0., resabs, reseps, result = 0., abserr = 0., small = 0., abseps;
	int ier = 0, ierro = 0, iroff1 = 0, iroff2 = 0, iroff3 = 0, ksgn = -1, ktmin = 0, last = 1, maxerr = 1;
	int nres = 0, nrmax = 1, numrl2 = 2;
	bool extrap = false, noext = false;
	enum { kSum, kFinal, kDec, kFinish } exit_mode = kFinish;

	alist[1] = lo;
	blist[1] = hi;
	if (epsabs <= 0. && epsrel < dmax(50. * epmach, 0.5e-28)) {
		ier = 6;
		goto finish;
	}
	if (infinite) qk15i(f, boun, lo, hi, &result, &abserr, &defabs, &resabs);
	else qk21(f, lo, hi, &result, &abserr, &defabs, &resabs);
	dres = fabs(result);
	errbnd = dmax(epsabs, epsrel * dres);
	last = 1;
	rlist[1] = result;
	elist[1] = abserr;
	iord[1] = 1;
	if (abserr <= 100. * epmach * defabs && abserr > errbnd) ier = 2;
	if (limit == 1) ier = 1;
	if (ier != 0 || (abserr <= errbnd && abserr != resabs) || abserr == 0.) goto finish;

	rlist2[1] = result;
	errmax = abserr;
	maxerr = 1;
	area = result;
	errsum = abserr;
	abserr = DBL_MAX;
	if (dres >= (1. - 50. * epmach) * defabs) ksgn = 1;

	exit_mode = kFinal;
	for (last = 2; last <= limit; last++) {
		a1 = alist[maxerr];
		b1 = 0.5 * (alist[maxerr] + blist[maxerr]);
		a2 = b1;
		b2 = blist[maxerr];
		erlast = errmax;
		if (infinite) {
			qk15i(f, boun, a1, b1, &area1, &error1, &resabs, &defab1);
			qk15i(f, boun, a2, b2, &area2, &error2, &resabs, &defab2);
		}
		else {
			qk21(f, a1, b1, &area1, &error1, &resabs, &defab1);
			qk21(f, a2, b2, &area2, &error2, &resabs, &defab2);
		}
		area12 = area1 + area2;
		erro12 = error1 + error2;
		errsum = errsum + erro12 - errmax;
		area = area + area12 - rlist[maxerr];
		if (defab1 != error1 && defab2 != error2) {
			if (fabs(rlist[maxerr] - area12) <= 1e-5 * fabs(area12) && erro12 >= 0.99 * errmax) {
				if (extrap) iroff2++;
				else iroff1++;
			}
			if (last > 10 && erro12 > errmax) iroff3++;
		}
		rlist[maxerr] = area1;
		rlist[last] = area2;
		errbnd = dmax(epsabs, epsrel * fabs(area));
		if (iroff1 + iroff2 >= 10 || iroff3 >= 20) ier = 2;
		if (iroff2 >= 5) ierro = 3;
		if (last == limit) ier = 1;
		if (dmax(fabs(a1), fabs(b2)) <= (1. + 100. * epmach) * (fabs(a2) + 1000. * DBL_MIN)) ier = 4;
		if (error2 > error1) {
			alist[maxerr] = a2;
			alist[last] = a1;
			blist[last] = b1;
			rlist[maxerr] = area2;
			rlist[last] = area1;
			elist[maxerr] = error2;
			elist[last] = error1;
		}
		else {
			alist[last] = a2;
			blist[maxerr] = b1;
			blist[last] = b2;
			elist[maxerr] = error1;
			elist[last] = error2;
		}
		qpsrt(limit, last, &maxerr, &errmax, elist, iord, &nrmax);
		if (errsum <= errbnd) {
			exit_mode = kSum;
			break;
		}
		if (ier != 0) {
			exit_mode = kFinal;
			break;
		}
		if (last == 2) {
			small = fabs(hi - lo) * 0.375;
			erlarg = errsum;
			ertest = errbnd;
			rlist2[2] = area;
			continue;
		}
		if (noext) continue;
		erlarg -= erlast;
		if (fabs(b1 - a1) > small) erlarg += erro12;
		if (!extrap) {
			if (fabs(blist[maxerr] - alist[maxerr]) > small) continue;
			extrap = true;
			nrmax = 2;
		}
		if (ierro != 3 && erlarg > ertest) {
			bool next = false;
			int id = nrmax;
			int jupbnd = last;
			if (last > (2 + limit / 2)) jupbnd = limit + 3 - last;
			for (int k = id; k <= jupbnd; k++) {
				maxerr = iord[nrmax];
				errmax = elist[maxerr];
				if (fabs(blist[maxerr] - alist[maxerr]) > small) {
					next = true;
					break;
				}
				nrmax++;
			}
			if (next) continue;
		}
		numrl2++;
		rlist2[numrl2] = area;
		qelg(&numrl2, rlist2, &reseps, &abseps, res3la, &nres);
		ktmin++;
		if (ktmin > 5 && abserr < 1e-3 * errsum) ier = 5;
		if (abseps < abserr) {
			ktmin = 0;
			abserr = abseps;
			result = reseps;
			correc = erlarg;
			ertest = dmax(epsabs, epsrel * fabs(reseps));
			if (abserr <= ertest) {
				exit_mode = kFinal;
				break;
			}
		}
		if (numrl2 == 1) noext = true;
		if (ier == 5) {
			exit_mode = kFinal;
			break;
		}
		maxerr = iord[1];
		errmax = elist[maxerr];
		nrmax = 1;
		extrap = false;
		small *= 0.5;
		erlarg = errsum;
	}
	if (last > limit) last = limit;

	if (exit_mode == kFinal) {
		if (abserr == DBL_MAX) {
			exit_mode = kSum;
		}
		else {
			exit_mode = kDec;
			bool to_divergence = true;
			if (ier + ierro != 0) {
				if (ierro == 3) abserr += correc;
				if (ier == 0) ier = 3;
				if (result != 0. && area != 0.) {
					if (abserr / fabs(result) > errsum / fabs(area)) {
						exit_mode = kSum;
						to_divergence = false;
					}
				}
				else if (abserr > errsum) {
					exit_mode = kSum;
					to_divergence = false;
				}
				else if (area == 0.) {
					to_divergence = false;
				}
			}
			if (to_divergence) {
				if (!(ksgn == -1 && dmax(fabs(result), fabs(area)) <= defabs * 0.01)) {
					if (0.01 > (result / area) || (result / area) > 100. || errsum > fabs(area)) ier = 6;
				}
			}
		}
	}
	if (exit_mode == kSum) {
		result = 0.;
		for (int k = 1; k <= last; k++) result += rlist[k];
		abserr = errsum;
		exit_mode = kDec;
	}
	if (exit_mode == kDec) {
		if (ier > 2) ier--;
	}
finish:
	if (ier_out) *ier_out = ier;
	return result;
}

}  // namespace sf
}  // namespace pf
