/*
 * Oracle special functions: TEST INFRASTRUCTURE ONLY (never linked into the
 * product library). Restates the published algorithms behind the GSL calls
 * libprofit makes in src/utils.cpp:109-186; the header lists each one.
 *
 * Arrays in the QUADPACK part are 1-based (element 0 unused) so that the
 * control flow reads like the published dqagse / dqagie / dqelg / dqpsrt.
 */
#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "specfun.h"

/* ------------------------------------------------------------------ gamma */

double orc_gammafn(double x)
{
	/* src/utils.cpp:117-132: underflow -> 0, overflow(x>0) -> +inf, else NaN */
	if (x == 0 || (x < 0 && x == floor(x))) {
		return NAN;
	}
	return tgamma(x);
}

double orc_lgammafn(double x)
{
	return lgamma(x);
}

double orc_beta(double a, double b)
{
	/* src/utils.cpp:134-153 edge behaviour */
	if (a < 0. || b < 0.) {
		return NAN;
	}
	if (a == 0. || b == 0.) {
		return INFINITY;
	}
	if (a + b < 170.) {
		return tgamma(a) * tgamma(b) / tgamma(a + b);
	}
	return exp(lgamma(a) + lgamma(b) - lgamma(a + b));
}

/* ----------------------------------------------------- incomplete gamma */

#define ORC_FPMIN 1e-300

/* P(a,x) by its power series (DLMF 8.7.1), valid and used for x < a+1 */
static double pgamma_series(double a, double x)
{
	double ap = a, term = 1., sum = 1.;
	int n;
	for (n = 1; n < 2000; n++) {
		ap += 1.;
		term *= x / ap;
		sum += term;
		if (fabs(term) < fabs(sum) * DBL_EPSILON) {
			break;
		}
	}
	return exp(a * log(x) - x - lgamma(a + 1.)) * sum;
}

/* Q(a,x) by the Legendre continued fraction (DLMF 8.9.2), modified Lentz */
static double qgamma_cf(double a, double x)
{
	double b = x + 1. - a, c = 1. / ORC_FPMIN, d = 1. / b, h = d;
	int i;
	for (i = 1; i < 2000; i++) {
		double an = -i * (i - a);
		double del;
		b += 2.;
		d = an * d + b;
		if (fabs(d) < ORC_FPMIN) d = ORC_FPMIN;
		c = b + an / c;
		if (fabs(c) < ORC_FPMIN) c = ORC_FPMIN;
		d = 1. / d;
		del = d * c;
		h *= del;
		if (fabs(del - 1.) < DBL_EPSILON) {
			break;
		}
	}
	return exp(a * log(x) - x - lgamma(a)) * h;
}

double orc_pgamma(double x, double a)
{
	if (x <= 0.) {
		return 0.;
	}
	if (isinf(x)) {
		return 1.;
	}
	if (x < a + 1.) {
		return pgamma_series(a, x);
	}
	return 1. - qgamma_cf(a, x);
}

double orc_qgamma_upper(double x, double a)
{
	if (x <= 0.) {
		return 1.;
	}
	if (isinf(x)) {
		return 0.;
	}
	if (x < a + 1.) {
		return 1. - pgamma_series(a, x);
	}
	return qgamma_cf(a, x);
}

/*
 * Inverse of P(a, .): bracket the root by doubling, then safeguarded Halley
 * iterations on f(x) = P(a,x) - p (or q - Q(a,x) when p > 0.5, which keeps
 * the upper tail well conditioned). f' is the gamma density and
 * f''/f' = (a-1)/x - 1.
 */
double orc_qgamma(double p, double a)
{
	int use_q, it;
	double q, lo, hi, x;
	if (!(p > 0.)) {
		return 0.;
	}
	if (p >= 1.) {
		return INFINITY;
	}
	use_q = p > 0.5;
	q = 1. - p;
	lo = 0.;
	hi = a > 1. ? a : 1.;
	for (it = 0; it < 2000; it++) {
		double below = use_q ? (orc_qgamma_upper(hi, a) > q) : (orc_pgamma(hi, a) < p);
		if (!below) {
			break;
		}
		lo = hi;
		hi *= 2.;
	}
	x = a;
	if (!(x > lo && x < hi)) {
		x = 0.5 * (lo + hi);
	}
	for (it = 0; it < 200; it++) {
		double f = use_q ? (q - orc_qgamma_upper(x, a)) : (orc_pgamma(x, a) - p);
		double pdf, dx, t, xn;
		if (f == 0.) {
			break;
		}
		if (f < 0.) lo = x; else hi = x;
		pdf = exp((a - 1.) * log(x) - x - lgamma(a));
		dx = f / pdf;
		t = 0.5 * dx * ((a - 1.) / x - 1.);
		if (fabs(t) < 0.5) {
			dx = dx / (1. - t);
		}
		xn = x - dx;
		if (!(xn > lo && xn < hi)) {
			xn = 0.5 * (lo + hi);
		}
		if (fabs(xn - x) <= 4. * DBL_EPSILON * xn) {
			x = xn;
			break;
		}
		x = xn;
	}
	return x;
}

/* ------------------------------------------------------------ QUADPACK */

static const double xgk21[12] = {0,
	0.995657163025808080735527280689003, 0.973906528517171720077964012084452,
	0.930157491355708226001207180059508, 0.865063366688984510732096688423493,
	0.780817726586416897063717578345042, 0.679409568299024406234327365114874,
	0.562757134668604683339000099272694, 0.433395394129247190799265943165784,
	0.294392862701460198131126603103866, 0.148874338981631210884826001129720,
	0.000000000000000000000000000000000};
static const double wgk21[12] = {0,
	0.011694638867371874278064396062192, 0.032558162307964727478818972459390,
	0.054755896574351996031381300244580, 0.075039674810919952767043140916190,
	0.093125454583697605535065465083366, 0.109387158802297641899210590325805,
	0.123491976262065851077208608978567, 0.134709217311473325928054001771707,
	0.142775938577060080797094273138717, 0.147739104901338491374841515972068,
	0.149445554002916905664936468389821};
static const double wg10[6] = {0,
	0.066671344308688137593568809893332, 0.149451349150580593145776339657697,
	0.219086362515982043995534934228163, 0.269266719309996355091226921569469,
	0.295524224714752870173892994651338};

static const double xgk15[9] = {0,
	0.991455371120812639206854697526329, 0.949107912342758524526189684047851,
	0.864864423359769072789712788640926, 0.741531185599394439863864773280788,
	0.586087235467691130294144845693013, 0.405845151377397166906606412076961,
	0.207784955007898467600689403773245, 0.000000000000000000000000000000000};
static const double wgk15[9] = {0,
	0.022935322010529224963732008058970, 0.063092092629978553290700663189204,
	0.104790010322250183839876322541518, 0.140653259715525918745189590510238,
	0.169004726639267902826583426598550, 0.190350578064785409913256402421014,
	0.204432940075298892414161999234649, 0.209482141084727828012999174891714};
static const double wg7[9] = {0,
	0.0, 0.129484966168869693270611432679082, 0.0, 0.279705391489276667901467771423780,
	0.0, 0.381830050505118944950369775488975, 0.0, 0.417959183673469387755102040816327};

#define EPMACH DBL_EPSILON
#define UFLOW DBL_MIN
#define OFLOW DBL_MAX

static double fmax2(double a, double b) { return a > b ? a : b; }
static double fmin2(double a, double b) { return a < b ? a : b; }

/* The error estimate shared by both rules (dqk21 / dqk15i epilogue). */
static double qk_error(double resk, double resg, double hlgth, double resabs, double resasc)
{
	double abserr = fabs((resk - resg) * hlgth);
	if (resasc != 0. && abserr != 0.) {
		abserr = resasc * fmin2(1., pow(200. * abserr / resasc, 1.5));
	}
	if (resabs > UFLOW / (50. * EPMACH)) {
		abserr = fmax2(EPMACH * 50. * resabs, abserr);
	}
	return abserr;
}

/* 21-point Gauss-Kronrod rule on [a,b] (dqk21) */
static void qk21(orc_integrand f, void *ctx, double a, double b,
                 double *result, double *abserr, double *resabs, double *resasc)
{
	double fv1[11], fv2[11];
	double centr = 0.5 * (a + b), hlgth = 0.5 * (b - a), dhlgth = fabs(hlgth);
	double resg = 0., fc = f(centr, ctx), resk = wgk21[11] * fc, reskh;
	int j;
	*resabs = fabs(resk);
	for (j = 1; j <= 5; j++) {
		int jtw = 2 * j;
		double absc = hlgth * xgk21[jtw];
		double fval1 = f(centr - absc, ctx), fval2 = f(centr + absc, ctx);
		double fsum = fval1 + fval2;
		fv1[jtw] = fval1;
		fv2[jtw] = fval2;
		resg += wg10[j] * fsum;
		resk += wgk21[jtw] * fsum;
		*resabs += wgk21[jtw] * (fabs(fval1) + fabs(fval2));
	}
	for (j = 1; j <= 5; j++) {
		int jtwm1 = 2 * j - 1;
		double absc = hlgth * xgk21[jtwm1];
		double fval1 = f(centr - absc, ctx), fval2 = f(centr + absc, ctx);
		double fsum = fval1 + fval2;
		fv1[jtwm1] = fval1;
		fv2[jtwm1] = fval2;
		resk += wgk21[jtwm1] * fsum;
		*resabs += wgk21[jtwm1] * (fabs(fval1) + fabs(fval2));
	}
	reskh = resk * 0.5;
	*resasc = wgk21[11] * fabs(fc - reskh);
	for (j = 1; j <= 10; j++) {
		*resasc += wgk21[j] * (fabs(fv1[j] - reskh) + fabs(fv2[j] - reskh));
	}
	*result = resk * hlgth;
	*resabs *= dhlgth;
	*resasc *= dhlgth;
	*abserr = qk_error(resk, resg, hlgth, *resabs, *resasc);
}

/* 15-point Gauss-Kronrod rule on the transformed range (dqk15i, inf = 1):
 * integrates f(boun + (1-t)/t) / t^2 over t in [a,b] within (0,1]. */
static void qk15i(orc_integrand f, void *ctx, double boun, double a, double b,
                  double *result, double *abserr, double *resabs, double *resasc)
{
	double fv1[8], fv2[8];
	double centr = 0.5 * (a + b), hlgth = 0.5 * (b - a);
	double tabsc1 = boun + (1. - centr) / centr;
	double fval1 = f(tabsc1, ctx);
	double fc = (fval1 / centr) / centr;
	double resg = wg7[8] * fc, resk = wgk15[8] * fc, reskh;
	int j;
	*resabs = fabs(resk);
	for (j = 1; j <= 7; j++) {
		double absc = hlgth * xgk15[j];
		double absc1 = centr - absc, absc2 = centr + absc;
		double t1 = boun + (1. - absc1) / absc1, t2 = boun + (1. - absc2) / absc2;
		double f1 = f(t1, ctx), f2 = f(t2, ctx), fsum;
		f1 = (f1 / absc1) / absc1;
		f2 = (f2 / absc2) / absc2;
		fv1[j] = f1;
		fv2[j] = f2;
		fsum = f1 + f2;
		resg += wg7[j] * fsum;
		resk += wgk15[j] * fsum;
		*resabs += wgk15[j] * (fabs(f1) + fabs(f2));
	}
	reskh = resk * 0.5;
	*resasc = wgk15[8] * fabs(fc - reskh);
	for (j = 1; j <= 7; j++) {
		*resasc += wgk15[j] * (fabs(fv1[j] - reskh) + fabs(fv2[j] - reskh));
	}
	*result = resk * hlgth;
	*resasc *= hlgth;
	*resabs *= hlgth;
	*abserr = qk_error(resk, resg, hlgth, *resabs, *resasc);
}

/* dqpsrt: keep iord[1..] ordered by decreasing elist, pick the next maxerr */
static void qpsrt(int limit, int last, int *maxerr, double *ermax,
                  const double *elist, int *iord, int *nrmax)
{
	double errmax, errmin;
	int i, ibeg, ido, isucc, j, jbnd, jupbn, k;
	if (last <= 2) {
		iord[1] = 1;
		iord[2] = 2;
		goto done;
	}
	errmax = elist[*maxerr];
	if (*nrmax != 1) {
		ido = *nrmax - 1;
		for (i = 1; i <= ido; i++) {
			isucc = iord[*nrmax - 1];
			if (errmax <= elist[isucc]) {
				break;
			}
			iord[*nrmax] = isucc;
			(*nrmax)--;
		}
	}
	jupbn = last;
	if (last > (limit / 2 + 2)) {
		jupbn = limit + 3 - last;
	}
	errmin = elist[last];
	jbnd = jupbn - 1;
	ibeg = *nrmax + 1;
	if (ibeg <= jbnd) {
		for (i = ibeg; i <= jbnd; i++) {
			isucc = iord[i];
			if (errmax >= elist[isucc]) {
				/* insert errmin by traversing the list bottom-up */
				iord[i - 1] = *maxerr;
				k = jbnd;
				for (j = i; j <= jbnd; j++) {
					isucc = iord[k];
					if (errmin < elist[isucc]) {
						iord[k + 1] = last;
						goto done;
					}
					iord[k + 1] = isucc;
					k--;
				}
				iord[i] = last;
				goto done;
			}
			iord[i - 1] = isucc;
		}
	}
	iord[jbnd] = *maxerr;
	iord[jupbn] = last;
done:
	*maxerr = iord[*nrmax];
	*ermax = elist[*maxerr];
}

/* dqelg: Wynn's epsilon algorithm on epstab[1..n] (n updated in place) */
static void qelg(int *n, double *epstab, double *result, double *abserr,
                 double *res3la, int *nres)
{
	const int limexp = 50;
	double delta1, delta2, delta3, e0, e1, e1abs, e2, e3, epsinf, err1, err2, err3;
	double error, res, ss, tol1, tol2, tol3;
	int i, ib, ib2, ie, indx, k1, k2, k3, newelm, num;

	(*nres)++;
	*abserr = OFLOW;
	*result = epstab[*n];
	if (*n < 3) {
		goto out;
	}
	epstab[*n + 2] = epstab[*n];
	newelm = (*n - 1) / 2;
	epstab[*n] = OFLOW;
	num = *n;
	k1 = *n;
	for (i = 1; i <= newelm; i++) {
		k2 = k1 - 1;
		k3 = k1 - 2;
		res = epstab[k1 + 2];
		e0 = epstab[k3];
		e1 = epstab[k2];
		e2 = res;
		e1abs = fabs(e1);
		delta2 = e2 - e1;
		err2 = fabs(delta2);
		tol2 = fmax2(fabs(e2), e1abs) * EPMACH;
		delta3 = e1 - e0;
		err3 = fabs(delta3);
		tol3 = fmax2(e1abs, fabs(e0)) * EPMACH;
		if (err2 <= tol2 && err3 <= tol3) {
			/* e0, e1, e2 agree to machine accuracy: convergence assumed */
			*result = res;
			*abserr = err2 + err3;
			goto out;
		}
		e3 = epstab[k1];
		epstab[k1] = e1;
		delta1 = e1 - e3;
		err1 = fabs(delta1);
		tol1 = fmax2(e1abs, fabs(e3)) * EPMACH;
		if (err1 <= tol1 || err2 <= tol2 || err3 <= tol3) {
			*n = i + i - 1;
			break;
		}
		ss = 1. / delta1 + 1. / delta2 - 1. / delta3;
		epsinf = fabs(ss * e1);
		if (!(epsinf > 1e-4)) {
			*n = i + i - 1;
			break;
		}
		res = e1 + 1. / ss;
		epstab[k1] = res;
		k1 -= 2;
		error = err2 + fabs(res - e2) + err3;
		if (error > *abserr) {
			continue;
		}
		*abserr = error;
		*result = res;
	}
	/* shift the table */
	if (*n == limexp) {
		*n = 2 * (limexp / 2) - 1;
	}
	ib = (num % 2 == 0) ? 2 : 1;
	ie = newelm + 1;
	for (i = 1; i <= ie; i++) {
		ib2 = ib + 2;
		epstab[ib] = epstab[ib2];
		ib = ib2;
	}
	if (num != *n) {
		indx = num - *n + 1;
		for (i = 1; i <= *n; i++) {
			epstab[i] = epstab[indx];
			indx++;
		}
	}
	if (*nres < 4) {
		res3la[*nres] = *result;
		*abserr = OFLOW;
	}
	else {
		*abserr = fabs(*result - res3la[3]) + fabs(*result - res3la[2]) + fabs(*result - res3la[1]);
		res3la[1] = res3la[2];
		res3la[2] = res3la[3];
		res3la[3] = *result;
	}
out:
	*abserr = fmax2(*abserr, 5. * EPMACH * fabs(*result));
}

/*
 * Shared adaptive driver: dqagse when infinite == 0 (rule qk21 on [a,b]),
 * dqagie with inf = 1 when infinite != 0 (rule qk15i on t in (0,1], x = a + (1-t)/t).
 */
static double qag_driver(orc_integrand f, void *ctx, double a, double b, int infinite,
                         double epsabs, double epsrel, int limit, int *ier_out, double *abserr_out)
{
	double *alist, *blist, *rlist, *elist;
	int *iord;
	double rlist2[53], res3la[4];
	double area, area1, area12, area2, a1, a2, b1, b2, correc = 0., defabs, defab1, defab2;
	double dres, epmach = EPMACH, erlarg = 0., erlast, errbnd, errmax, error1, error2, erro12;
	double errsum, ertest = 0., resabs, reseps, result, abserr, small = 0., abseps;
	double boun = a, lo = a, hi = b;
	int id, ier = 0, ierro, iroff1, iroff2, iroff3, jupbnd, k, ksgn, ktmin, last, maxerr;
	int nres, nrmax, numrl2, extrap, noext;

	if (limit < 1) {
		limit = 1;
	}
	alist = (double *)calloc((size_t)limit + 2, sizeof(double));
	blist = (double *)calloc((size_t)limit + 2, sizeof(double));
	rlist = (double *)calloc((size_t)limit + 2, sizeof(double));
	elist = (double *)calloc((size_t)limit + 2, sizeof(double));
	iord = (int *)calloc((size_t)limit + 2, sizeof(int));
	memset(rlist2, 0, sizeof(rlist2));
	memset(res3la, 0, sizeof(res3la));

	if (infinite) {
		lo = 0.;
		hi = 1.;
	}
	alist[1] = lo;
	blist[1] = hi;
	rlist[1] = 0.;
	elist[1] = 0.;
	result = 0.;
	abserr = 0.;
	if (epsabs <= 0. && epsrel < fmax2(50. * epmach, 0.5e-28)) {
		ier = 6;
		goto finish;
	}

	/* first approximation to the integral */
	ierro = 0;
	if (infinite) {
		qk15i(f, ctx, boun, lo, hi, &result, &abserr, &defabs, &resabs);
	}
	else {
		qk21(f, ctx, lo, hi, &result, &abserr, &defabs, &resabs);
	}
	dres = fabs(result);
	errbnd = fmax2(epsabs, epsrel * dres);
	last = 1;
	rlist[1] = result;
	elist[1] = abserr;
	iord[1] = 1;
	if (abserr <= 100. * epmach * defabs && abserr > errbnd) ier = 2;
	if (limit == 1) ier = 1;
	if (ier != 0 || (abserr <= errbnd && abserr != resabs) || abserr == 0.) {
		goto finish;
	}

	/* initialisation */
	rlist2[1] = result;
	errmax = abserr;
	maxerr = 1;
	area = result;
	errsum = abserr;
	abserr = OFLOW;
	nrmax = 1;
	nres = 0;
	numrl2 = 2;
	ktmin = 0;
	extrap = 0;
	noext = 0;
	iroff1 = iroff2 = iroff3 = 0;
	ksgn = -1;
	if (dres >= (1. - 50. * epmach) * defabs) ksgn = 1;

	for (last = 2; last <= limit; last++) {
		/* bisect the subinterval with the nrmax-th largest error estimate */
		a1 = alist[maxerr];
		b1 = 0.5 * (alist[maxerr] + blist[maxerr]);
		a2 = b1;
		b2 = blist[maxerr];
		erlast = errmax;
		if (infinite) {
			qk15i(f, ctx, boun, a1, b1, &area1, &error1, &resabs, &defab1);
			qk15i(f, ctx, boun, a2, b2, &area2, &error2, &resabs, &defab2);
		}
		else {
			qk21(f, ctx, a1, b1, &area1, &error1, &resabs, &defab1);
			qk21(f, ctx, a2, b2, &area2, &error2, &resabs, &defab2);
		}

		/* improve previous approximations to integral and error; test accuracy */
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
		errbnd = fmax2(epsabs, epsrel * fabs(area));

		/* roundoff, interval-limit and bad-integrand flags */
		if (iroff1 + iroff2 >= 10 || iroff3 >= 20) ier = 2;
		if (iroff2 >= 5) ierro = 3;
		if (last == limit) ier = 1;
		if (fmax2(fabs(a1), fabs(b2)) <= (1. + 100. * epmach) * (fabs(a2) + 1000. * UFLOW)) ier = 4;

		/* append the newly-created intervals to the list */
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

		if (errsum <= errbnd) goto sum_up;
		if (ier != 0) goto final_result;
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
			/* is the interval to be bisected next the smallest one? */
			if (fabs(blist[maxerr] - alist[maxerr]) > small) continue;
			extrap = 1;
			nrmax = 2;
		}
		if (ierro != 3 && erlarg > ertest) {
			/* the smallest interval has the largest error: before bisecting,
			 * decrease the sum of the errors over the larger intervals (erlarg)
			 * and perform extrapolation */
			int goto_next = 0;
			id = nrmax;
			jupbnd = last;
			if (last > (2 + limit / 2)) jupbnd = limit + 3 - last;
			for (k = id; k <= jupbnd; k++) {
				maxerr = iord[nrmax];
				errmax = elist[maxerr];
				if (fabs(blist[maxerr] - alist[maxerr]) > small) {
					goto_next = 1;
					break;
				}
				nrmax++;
			}
			if (goto_next) continue;
		}

		/* perform extrapolation */
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
			ertest = fmax2(epsabs, epsrel * fabs(reseps));
			if (abserr <= ertest) goto final_result;
		}

		/* prepare bisection of the smallest interval */
		if (numrl2 == 1) noext = 1;
		if (ier == 5) goto final_result;
		maxerr = iord[1];
		errmax = elist[maxerr];
		nrmax = 1;
		extrap = 0;
		small *= 0.5;
		erlarg = errsum;
	}
	if (last > limit) {
		last = limit;
	}

final_result:
	/* set final result and error estimate */
	if (abserr == OFLOW) goto sum_up;
	if (ier + ierro != 0) {
		if (ierro == 3) abserr += correc;
		if (ier == 0) ier = 3;
		if (result != 0. && area != 0.) {
			if (abserr / fabs(result) > errsum / fabs(area)) goto sum_up;
		}
		else if (abserr > errsum) {
			goto sum_up;
		}
		else if (area == 0.) {
			goto dec_ier;
		}
	}
	/* test on divergence */
	if (ksgn == -1 && fmax2(fabs(result), fabs(area)) <= defabs * 0.01) goto dec_ier;
	if (0.01 > (result / area) || (result / area) > 100. || errsum > fabs(area)) ier = 6;
	goto dec_ier;

sum_up:
	/* compute global integral sum */
	result = 0.;
	for (k = 1; k <= last; k++) {
		result += rlist[k];
	}
	abserr = errsum;

dec_ier:
	if (ier > 2) ier--;

finish:
	free(alist);
	free(blist);
	free(rlist);
	free(elist);
	free(iord);
	if (ier_out) *ier_out = ier;
	if (abserr_out) *abserr_out = abserr;
	return result;
}

double orc_qags(orc_integrand f, void *ctx, double a, double b,
                double epsabs, double epsrel, int limit, int *ier, double *abserr)
{
	return qag_driver(f, ctx, a, b, 0, epsabs, epsrel, limit, ier, abserr);
}

double orc_qagiu(orc_integrand f, void *ctx, double a,
                 double epsabs, double epsrel, int limit, int *ier, double *abserr)
{
	return qag_driver(f, ctx, a, 0., 1, epsabs, epsrel, limit, ier, abserr);
}
