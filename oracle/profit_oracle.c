/*
 * CPU oracle for libprofit's image-generation path: TEST INFRASTRUCTURE ONLY.
 * See profit_oracle.h for the list of reference functions restated here; each
 * function below cites the reference lines it follows. Compiled with
 * -ffp-contract=off so that no multiply-add is fused, as in the reference's
 * x86-64 build.
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "profit_oracle.h"
#include "specfun.h"

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

static char g_err[512];

const char *orc_last_error(void) { return g_err; }

static int fail(const char *msg)
{
	snprintf(g_err, sizeof(g_err), "%s", msg);
	return -1;
}

double orc_api_qgamma(double p, double a) { return orc_qgamma(p, a); }
double orc_api_pgamma(double x, double a) { return orc_pgamma(x, a); }
double orc_api_gammafn(double x) { return orc_gammafn(x); }
double orc_api_beta(double a, double b) { return orc_beta(a, b); }

/* ------------------------------------------------------------- profiles */

enum { RF_GENERAL, RF_POINTFIVE, RF_ONE, RF_TWO, RF_THREE, RF_FOUR, RF_EIGHT, RF_SIXTEEN };

typedef struct {
	int kind;
	/* parameters (src/radial.cpp:724-752 defaults are applied by the caller) */
	double xcen, ycen, mag, ang, axrat, box;
	int rough, adjust, rescale_flux;
	unsigned int resolution, max_recursions;
	double acc, rscale_switch, rscale_max;
	double re, nser, rb, a, b, fwhm, con, rout, rc, rt, h1, h2;
	/* internally calculated (src/radial.cpp:271-279) */
	double rscale, ie, bn, lumtot, rescale_factor;
	double cos_ang, sin_ang, xc, yc, magzero;
	int rf_boxy, rf_t;
	double image_scale_x, image_scale_y;
	long long counts[32];
	signed char *depth;
	unsigned int depth_w;
} radial_t;

/* boxy radius, include/profit/radial.h:93-102 */
static double boxy_r(const radial_t *p, double x, double y)
{
	double box_plus_2;
	if (p->box == 0) {
		return sqrt(x * x + y * y);
	}
	box_plus_2 = p->box + 2.;
	return pow(pow(fabs(x), box_plus_2) + pow(fabs(y), box_plus_2), 1. / box_plus_2);
}

/* src/sersic.cpp:79-198: base^(1/invexp) with the reference's specialisations */
static double sersic_eval(const radial_t *p, double x, double y)
{
	double B = p->box + 2;
	double base, invexp, rf;
	if (p->rf_boxy) {
		base = pow(fabs(x / p->re), B) + pow(fabs(y / p->re), B);
		invexp = p->nser * B;
		switch (p->rf_t) {
		case RF_POINTFIVE: rf = base * base; break;
		case RF_ONE: rf = base; break;
		case RF_TWO: rf = sqrt(base); break;
		case RF_THREE: rf = cbrt(base); break;
		case RF_FOUR: rf = sqrt(sqrt(base)); break;
		case RF_EIGHT: rf = sqrt(sqrt(sqrt(base))); break;
		case RF_SIXTEEN: rf = sqrt(sqrt(sqrt(sqrt(base)))); break;
		default: rf = pow(base, 1 / invexp); break;
		}
	}
	else {
		base = (x * x + y * y) / (p->re * p->re);
		invexp = p->nser;
		switch (p->rf_t) {
		case RF_POINTFIVE: rf = base; break;
		case RF_ONE: rf = sqrt(base); break;
		case RF_TWO: rf = sqrt(sqrt(base)); break;
		case RF_THREE: rf = cbrt(sqrt(base)); break;
		case RF_FOUR: rf = sqrt(sqrt(sqrt(base))); break;
		case RF_EIGHT: rf = sqrt(sqrt(sqrt(sqrt(base)))); break;
		case RF_SIXTEEN: rf = sqrt(sqrt(sqrt(sqrt(sqrt(base))))); break;
		default: rf = pow(sqrt(base), 1 / invexp); break;
		}
	}
	return exp(-p->bn * (rf - 1));
}

/* src/brokenexponential.cpp:38-77 */
static double broken_exponential(double r, double h1, double h2, double rb, double a)
{
	double base = r - rb;
	double expo = 1 / h1 - 1 / h2;
	if (a * base < 40) {
		base = log(1 + exp(a * base)) / a;
	}
	return exp(-r / h1 + expo * base);
}

static double evaluate_at(const radial_t *p, double x, double y)
{
	double r, rf;
	switch (p->kind) {
	case ORC_SERSIC:
		return sersic_eval(p, x, y);
	case ORC_CORESERSIC: /* src/coresersic.cpp:51-59 */
		r = boxy_r(p, x, y);
		return pow(1 + pow(r / p->rb, -p->a), p->b / p->a) *
		       exp(-p->bn * pow((pow(r, p->a) + pow(p->rb, p->a)) / pow(p->re, p->a), 1 / (p->nser * p->a)));
	case ORC_MOFFAT: /* src/moffat.cpp:52-58 */
		r = boxy_r(p, x, y);
		rf = r / p->rscale;
		return pow(1 + rf * rf, -p->con);
	case ORC_FERRER: /* src/ferrer.cpp:50-60 */
		r = boxy_r(p, x, y);
		rf = r / p->rscale;
		if (rf < 1) {
			return pow(1 - pow(rf, 2 - p->b), p->a);
		}
		return 0;
	case ORC_KING: /* src/king.cpp:51-59 */
		r = boxy_r(p, x, y);
		if (r < p->rt) {
			return pow(1 / pow(1 + pow(r / p->rc, 2), 1 / p->a) - 1 / pow(1 + pow(p->rt / p->rc, 2), 1 / p->a), p->a);
		}
		return 0;
	case ORC_BROKENEXP: /* src/brokenexponential.cpp:91-94 */
		return broken_exponential(boxy_r(p, x, y), p->h1, p->h2, p->rb, p->a);
	}
	return 0;
}

/* integrands for the numerical luminosities */
static double coresersic_integrand(double r, void *ctx) /* src/coresersic.cpp:80-87 */
{
	const radial_t *p = (const radial_t *)ctx;
	return r * pow(1 + pow(r / p->rb, -p->a), p->b / p->a) *
	       exp(-p->bn * pow((pow(r, p->a) + pow(p->rb, p->a)) / pow(p->re, p->a), 1 / (p->nser * p->a)));
}

static double king_integrand(double r, void *ctx) /* src/king.cpp:76-84 */
{
	const radial_t *p = (const radial_t *)ctx;
	if (r < p->rt) {
		return r * pow(1 / pow(1 + pow(r / p->rc, 2), 1 / p->a) - 1 / pow(1 + pow(p->rt / p->rc, 2), 1 / p->a), p->a);
	}
	return 0;
}

static double brokenexp_integrand(double r, void *ctx) /* src/brokenexponential.cpp:111-113 */
{
	const radial_t *p = (const radial_t *)ctx;
	return r * broken_exponential(r, p->h1, p->h2, p->rb, p->a);
}

static double integrate_qagi(orc_integrand f, void *ctx)
{
	return orc_qagiu(f, ctx, 0., 1e-4, 1e-4, 100, NULL, NULL);
}

static double get_rscale(const radial_t *p)
{
	switch (p->kind) {
	case ORC_SERSIC: case ORC_CORESERSIC: return p->re;
	case ORC_MOFFAT: return p->fwhm / (2 * sqrt(pow(2, (1 / p->con)) - 1)); /* src/moffat.cpp:81-83 */
	case ORC_FERRER: return p->rout;
	case ORC_KING: return p->rt;
	case ORC_BROKENEXP: return p->h1 * 4;
	}
	return 0;
}

static double get_lumtot(radial_t *p)
{
	switch (p->kind) {
	case ORC_SERSIC: { /* src/sersic.cpp:283-289 */
		double g_factor = orc_gammafn(2 * p->nser);
		return pow(p->re, 2) * 2 * M_PI * p->nser * g_factor * exp(p->bn) / pow(p->bn, 2 * p->nser);
	}
	case ORC_CORESERSIC: /* src/coresersic.cpp:92-104 */
		return 2 * M_PI * integrate_qagi(coresersic_integrand, p);
	case ORC_MOFFAT: /* src/moffat.cpp:77-79 */
		return pow(p->rscale, 2) * M_PI / (p->con - 1);
	case ORC_FERRER: { /* src/ferrer.cpp:78-101 */
		double g_factor = p->a * orc_beta(p->a, 1 + 2 / (2 - p->b));
		return pow(p->rout, 2) * M_PI * g_factor;
	}
	case ORC_KING: /* src/king.cpp:87-96 */
		return 2 * M_PI * orc_qags(king_integrand, p, 0, p->rt, 1e-4, 1e-4, 100, NULL, NULL);
	case ORC_BROKENEXP: /* src/brokenexponential.cpp:115-126 */
		return 2 * M_PI * integrate_qagi(brokenexp_integrand, p);
	}
	return 0;
}

static double sersic_fluxfrac(const radial_t *p, double fraction) /* src/sersic.cpp:257-260 */
{
	double ratio = orc_qgamma(fraction, 2 * p->nser) / p->bn;
	return p->re * pow(ratio, p->nser);
}

static double moffat_fluxfrac(const radial_t *p, double fraction) /* src/moffat.cpp:73-75 */
{
	return p->rscale * sqrt(pow(1 - fraction, 1 / (1 - p->con)) - 1);
}

static double fmax2(double a, double b) { return a > b ? a : b; }
static double fmin2(double a, double b) { return a < b ? a : b; }

static double adjust_rscale_switch(const radial_t *p)
{
	double rs;
	switch (p->kind) {
	case ORC_SERSIC: /* src/sersic.cpp:262-272 */
		rs = ceil(sersic_fluxfrac(p, 1. - p->nser * p->nser / 2e3));
		rs = fmax2(fmin2(rs, 20.), 2.);
		return rs / p->re;
	case ORC_MOFFAT: /* src/moffat.cpp:88-91 */
		rs = fmax2(moffat_fluxfrac(p, 0.9999), 1.823 * p->fwhm);
		return fmax2(fmin2(rs, 20.), 2.) / p->rscale;
	case ORC_CORESERSIC: return 1;
	case ORC_FERRER: return 0.5;
	case ORC_KING: return 0.5;
	case ORC_BROKENEXP: return 1;
	}
	return 1;
}

static double adjust_rscale_max(const radial_t *p)
{
	switch (p->kind) {
	case ORC_SERSIC: return ceil(fmax2(sersic_fluxfrac(p, 0.9999), 2.) / p->re); /* src/sersic.cpp:274-276 */
	case ORC_MOFFAT: return ceil(fmax2(moffat_fluxfrac(p, 0.9999), 2.) / p->rscale); /* src/moffat.cpp:93-95 */
	case ORC_CORESERSIC: return 100;
	case ORC_FERRER: return 1;
	case ORC_KING: return 1.5;
	case ORC_BROKENEXP: return 100;
	}
	return 0;
}

static double adjust_acc(const radial_t *p, double acc)
{
	switch (p->kind) {
	case ORC_SERSIC: /* src/sersic.cpp:278-281 */
		acc /= sqrt(p->nser);
		return fmax2(0.1, acc) / p->axrat;
	case ORC_MOFFAT: /* src/moffat.cpp:97-99 */
		return 0.1 / p->axrat;
	}
	return acc;
}

static int almost_equals(double x, double y) /* src/utils.cpp:101-103, e = 1e-10 */
{
	return fabs(x - y) < fabs(1e-10);
}

/* src/sersic.cpp:225-255 */
static void sersic_choose_rfactor(radial_t *p)
{
	double inv_exponent = p->nser;
	p->rf_boxy = p->box != 0;
	if (p->box != 0) {
		inv_exponent *= (p->box + 2);
	}
	if (almost_equals(inv_exponent, 0.5)) p->rf_t = RF_POINTFIVE;
	else if (almost_equals(inv_exponent, 1)) p->rf_t = RF_ONE;
	else if (almost_equals(inv_exponent, 2)) p->rf_t = RF_TWO;
	else if (almost_equals(inv_exponent, 3)) p->rf_t = RF_THREE;
	else if (almost_equals(inv_exponent, 4)) p->rf_t = RF_FOUR;
	else if (almost_equals(inv_exponent, 8)) p->rf_t = RF_EIGHT;
	else if (almost_equals(inv_exponent, 16)) p->rf_t = RF_SIXTEEN;
	else p->rf_t = RF_GENERAL;
}

/* RadialProfile::initial_calculations, src/radial.cpp:137-199, with the
 * sersic / coresersic overrides (src/sersic.cpp:291-313, src/coresersic.cpp:106-117) */
static void initial_calculations(radial_t *p)
{
	double b2, r_box, lumtot, angrad;
	if (p->kind == ORC_SERSIC || p->kind == ORC_CORESERSIC) {
		p->bn = orc_qgamma(0.5, 2 * p->nser);
	}
	p->rscale = get_rscale(p);
	b2 = p->box + 2;
	r_box = M_PI * b2 / (2 * orc_beta(1 / b2, 1 / b2));
	lumtot = get_lumtot(p) * p->axrat / r_box;
	p->lumtot = lumtot;
	p->ie = pow(10, -0.4 * (p->mag - p->magzero)) / lumtot;
	if (p->adjust) {
		unsigned int res;
		p->rscale_switch = adjust_rscale_switch(p);
		res = (unsigned int)ceil(160 / (p->rscale_switch * p->rscale));
		res += res % 2;
		res = res < 16U ? res : 16U;
		res = res > 4U ? res : 4U;
		p->resolution = res;
		if (p->rscale_max == 0) {
			p->rscale_max = adjust_rscale_max(p);
		}
		p->acc = adjust_acc(p, p->acc);
	}
	angrad = fmod(p->ang + 90, 360.) * M_PI / 180.;
	p->cos_ang = cos(angrad);
	p->sin_ang = sin(angrad);
	if (p->kind == ORC_SERSIC && p->adjust) {
		p->rescale_factor = 1;
		if (p->rescale_flux) {
			double flux_r = p->bn * pow(p->rscale_max / p->re, 1 / p->nser);
			flux_r = orc_pgamma(flux_r, 2 * p->nser);
			p->rescale_factor = 1 / flux_r;
		}
	}
}

/* src/radial.cpp:46-53 */
static void to_profile(const radial_t *p, double x, double y, double *xp, double *yp)
{
	x -= p->xc;
	y -= p->yc;
	*xp = x * p->cos_ang + y * p->sin_ang;
	*yp = -x * p->sin_ang + y * p->cos_ang;
	*yp /= p->axrat;
}

/* src/radial.cpp:55-135. `deepest` tracks the deepest level visited. */
static double subsample_pixel(radial_t *p, double x0, double x1, double y0, double y1,
                              unsigned int recur_level, unsigned int max_recursions,
                              unsigned int resolution, int *deepest)
{
	double xbin = (x1 - x0) / resolution;
	double ybin = (y1 - y0) / resolution;
	double half_xbin = xbin / 2.;
	double half_ybin = ybin / 2.;
	double total = 0, x_prof, y_prof, x = x0;
	int recurse = resolution > 1 && recur_level < max_recursions;
	unsigned int i, j, n_sub = 0;
	double *sub_x = NULL, *sub_y = NULL;

	if ((int)recur_level + 1 > *deepest) {
		*deepest = (int)recur_level + 1;
	}
	if (recur_level < 32) {
#pragma omp atomic
		p->counts[recur_level]++;
	}

	if (recurse) {
		sub_x = (double *)malloc(sizeof(double) * resolution * resolution);
		sub_y = (double *)malloc(sizeof(double) * resolution * resolution);
		for (i = 0; i < resolution; i++) {
			double y = y0;
			x += half_xbin;
			for (j = 0; j < resolution; j++) {
				double subval, delta_y_prof, testval;
				y += half_ybin;
				to_profile(p, x, y, &x_prof, &y_prof);
				subval = evaluate_at(p, x_prof, y_prof);
				delta_y_prof = (-xbin * p->sin_ang + ybin * p->cos_ang) / p->axrat;
				testval = evaluate_at(p, fabs(x_prof), fabs(y_prof) + fabs(delta_y_prof));
				if (fabs(testval / subval - 1.0) > p->acc) {
					sub_x[n_sub] = x;
					sub_y[n_sub] = y;
					n_sub++;
				}
				else {
					total += subval;
				}
				y += half_ybin;
			}
			x += half_xbin;
		}
	}
	else {
		for (i = 0; i < resolution; i++) {
			double y = y0;
			x += half_xbin;
			for (j = 0; j < resolution; j++) {
				y += half_ybin;
				to_profile(p, x, y, &x_prof, &y_prof);
				total += evaluate_at(p, x_prof, y_prof);
				y += half_ybin;
			}
			x += half_xbin;
		}
	}

	for (i = 0; i < n_sub; i++) {
		double sx = sub_x[i], sy = sub_y[i];
		total += subsample_pixel(p, sx - half_xbin, sx + half_xbin, sy - half_ybin, sy + half_ybin,
		                         recur_level + 1, max_recursions, resolution, deepest);
	}
	free(sub_x);
	free(sub_y);
	return total / (resolution * resolution);
}

/* RadialProfile::subsampling_params + SersicProfile override (src/sersic.cpp:331-347) */
static void subsampling_params(const radial_t *p, double x, double y, unsigned int *res, unsigned int *max_rec)
{
	*res = p->resolution;
	*max_rec = p->max_recursions;
	if (p->kind == ORC_SERSIC) {
		int center_pixel = fabs(x - p->xc) < p->image_scale_x && fabs(y - p->yc) < p->image_scale_y;
		if (p->adjust && center_pixel && p->nser > 1) {
			*res = 8;
			*max_rec = 10;
		}
	}
}

static double get_pixel_scale(const radial_t *p, double sx, double sy) /* src/radial.cpp:219-222 */
{
	double flux_scale = sx * sy * p->ie;
	if (p->kind == ORC_SERSIC && p->rescale_flux) { /* src/sersic.cpp:319-325 */
		flux_scale *= p->rescale_factor;
	}
	return flux_scale;
}

/* RadialProfile::evaluate_cpu, src/radial.cpp:291-344 */
static void evaluate_radial(radial_t *p, double *image, unsigned int width, unsigned int height,
                            const unsigned char *mask, double sx, double sy, int threads)
{
	double half_xbin = sx / 2.;
	double half_ybin = sy / 2.;
	double flux_scale = get_pixel_scale(p, sx, sy);
	long long n = (long long)width * height, k;
	(void)threads;
#pragma omp parallel for schedule(dynamic, 10) if (threads > 1) num_threads(threads > 1 ? threads : 1)
	for (k = 0; k < n; k++) {
		unsigned int i = (unsigned int)(k % width), j = (unsigned int)(k / width);
		double x_prof, y_prof, r_prof, pixel_val, x, y;
		int deepest = 0;
		if (mask && !mask[i + j * width]) {
			if (p->depth) p->depth[k] = -1;
			continue;
		}
		y = half_ybin + j * sy;
		x = half_xbin + i * sx;
		to_profile(p, x, y, &x_prof, &y_prof);
		r_prof = sqrt(x_prof * x_prof + y_prof * y_prof);
		if (p->rscale_max > 0 && r_prof / p->rscale > p->rscale_max) {
			pixel_val = 0.;
			deepest = -1;
		}
		else if (p->rough || r_prof / p->rscale > p->rscale_switch) {
			pixel_val = evaluate_at(p, x_prof, y_prof);
		}
		else {
			unsigned int ss_res, ss_max;
			subsampling_params(p, x, y, &ss_res, &ss_max);
			pixel_val = subsample_pixel(p, x - half_xbin, x + half_xbin, y - half_ybin, y + half_ybin,
			                            0, ss_max, ss_res, &deepest);
		}
		if (p->depth) p->depth[k] = (signed char)deepest;
		image[k] += flux_scale * pixel_val;
	}
}

static unsigned int bind(double value, unsigned int max) /* src/psf.cpp:47-55 */
{
	int intval = (int)floor(value);
	unsigned int u;
	if (intval < 0) {
		return 0;
	}
	u = (unsigned int)intval;
	return u < max ? u : max;
}

/* PsfProfile::evaluate, src/psf.cpp:58-145 (including the offset.x/offset.y mix-up) */
static void evaluate_psf_profile(const orc_profile *pp, const orc_model *m, const double *psf,
                                 double *image, unsigned int width, unsigned int height,
                                 double scale_x, double scale_y, double off_x, double off_y)
{
	double xcen = pp->par[ORC_P_XCEN], ycen = pp->par[ORC_P_YCEN], mag = pp->par[ORC_P_MAG];
	double scale = pow(10, -0.4 * (mag - m->magzero));
	double psf_scale_x = m->psf_scale_x, psf_scale_y = m->psf_scale_y;
	unsigned int psf_width = m->psf_w, psf_height = m->psf_h;
	double origin_x = xcen + off_x * scale_x - psf_width * psf_scale_x / 2;
	double end_x = xcen + off_y * scale_y + psf_width * psf_scale_x / 2;
	double origin_y = ycen + off_x * scale_x - psf_height * psf_scale_y / 2;
	double end_y = ycen + off_y * scale_y + psf_height * psf_scale_y / 2;
	unsigned int x0 = bind(origin_x / scale_x, width - 1);
	unsigned int y0 = bind(origin_y / scale_y, height - 1);
	unsigned int x1 = bind(end_x / scale_x, width - 1);
	unsigned int y1 = bind(end_y / scale_y, height - 1);
	unsigned int pix_x, pix_y;
	for (pix_y = y0; pix_y <= y1; pix_y++) {
		double y = pix_y * scale_y;
		for (pix_x = x0; pix_x <= x1; pix_x++) {
			double x = pix_x * scale_x;
			int psf_pix_x0 = (int)bind(floor((x - origin_x) / psf_scale_x), psf_width - 1);
			int psf_pix_x1 = (int)bind(floor((x - origin_x + scale_x) / psf_scale_x), psf_height - 1);
			int psf_pix_y0 = (int)bind(floor((y - origin_y) / psf_scale_y), psf_width - 1);
			int psf_pix_y1 = (int)bind(floor((y - origin_y + scale_y) / psf_scale_y), psf_height - 1);
			double val = 0;
			int py, px;
			for (py = psf_pix_y0; py <= psf_pix_y1; py++) {
				double psf_y = py * psf_scale_y + origin_y;
				for (px = psf_pix_x0; px <= psf_pix_x1; px++) {
					double psf_x = px * psf_scale_x + origin_x;
					double ix = fmin2(x + scale_x, psf_x + psf_scale_x) - fmax2(x, psf_x);
					double iy = fmin2(y + scale_y, psf_y + psf_scale_y) - fmax2(y, psf_y);
					val += psf[px + py * psf_width] * (ix * iy) / (psf_scale_x * psf_scale_y);
				}
			}
			image[pix_x + pix_y * width] += val * scale;
		}
	}
}

/* ---------------------------------------------------------- convolution */

/* BruteForceConvolver (old_variant) or AssociativeBruteForceConvolver
 * (src/convolve.cpp:101-231): out(i,j) = sum src * reversed kernel, zero
 * outside, masked output pixels set to 0. */
void orc_convolve_brute(const double *src, unsigned int src_width, unsigned int src_height,
                        const double *krn, unsigned int krn_width, unsigned int krn_height,
                        const unsigned char *mask, double *out, int old_variant, int threads)
{
	unsigned int krn_half_width = krn_width / 2, krn_half_height = krn_height / 2;
	long long n = (long long)src_width * src_height, k;
	size_t krn_size = (size_t)krn_width * krn_height;
	double *ikrn = (double *)malloc(sizeof(double) * (krn_size ? krn_size : 1));
	size_t q;
	(void)threads;
	for (q = 0; q < krn_size; q++) {
		ikrn[q] = krn[krn_size - 1 - q];
	}
#pragma omp parallel for schedule(dynamic, 10) if (threads > 1) num_threads(threads > 1 ? threads : 1)
	for (k = 0; k < n; k++) {
		unsigned int i = (unsigned int)(k % src_width), j = (unsigned int)(k / src_width);
		double pixel = 0;
		if (mask && !mask[k]) {
			out[k] = 0;
			continue;
		}
		if (old_variant) {
			unsigned int l, kk;
			for (l = 0; l < krn_height; l++) {
				int src_j = (int)j + (int)l - (int)krn_half_height;
				for (kk = 0; kk < krn_width; kk++) {
					int src_i = (int)i + (int)kk - (int)krn_half_width;
					if (src_i >= 0 && (unsigned int)src_i < src_width && src_j >= 0 && (unsigned int)src_j < src_height) {
						pixel += src[src_i + (size_t)src_j * src_width] * ikrn[kk + (size_t)l * krn_width];
					}
				}
			}
		}
		else {
			unsigned int l_min = 0, l_max = krn_height, k_min = 0, k_max = krn_width, l, kk;
			if (j < krn_half_height) l_min = krn_half_height - j;
			else if ((j + krn_half_height) >= src_height) l_max = src_height + krn_half_height - j;
			if (i < krn_half_width) k_min = krn_half_width - i;
			else if ((i + krn_half_width) >= src_width) k_max = src_width + krn_half_width - i;
			for (l = l_min; l < l_max; l++) {
				double dot = 0;
				long long srow = (long long)j + l - krn_half_height;
				for (kk = k_min; kk < k_max; kk++) {
					long long scol = (long long)i + kk - krn_half_width;
					dot += src[scol + srow * src_width] * ikrn[kk + (size_t)l * krn_width];
				}
				pixel += dot;
			}
		}
		out[k] = pixel;
	}
	free(ikrn);
}

/* ---------------------------------------------------------------- model */

static int is_radial(int kind) { return kind >= ORC_SERSIC && kind <= ORC_BROKENEXP; }

static int validate_profile(const orc_profile *pp, const orc_model *m)
{
	const double *v = pp->par;
	if (is_radial(pp->kind)) { /* src/radial.cpp:204-214 */
		if (v[ORC_P_AXRAT] <= 0) return fail("axrat <= 0, must have axrat > 0");
		if (v[ORC_P_AXRAT] > 1) return fail("axrat > 1, must have axrat <= 1");
		if (v[ORC_P_BOX] <= -2) return fail("box <= -2, must have box > -2");
	}
	switch (pp->kind) {
	case ORC_SERSIC:
		if (v[6] <= 0) return fail("re <= 0, must have re > 0");
		if (v[7] <= 0) return fail("nser <= 0, must have nser > 0");
		break;
	case ORC_CORESERSIC:
		if (v[6] <= 0) return fail("re <= 0, must have re > 0");
		if (v[8] <= 0) return fail("rb <= 0, must have rb > 0");
		if (v[7] <= 0) return fail("nser <= 0, must have nser > 0");
		if (v[9] <= 0) return fail("a <= 0, must have a > 0");
		if (v[10] > 1.999) return fail("b > 1.999, must have b < 1.999");
		break;
	case ORC_MOFFAT:
		if (v[6] <= 0) return fail("fwhm <= 0, must have fwhm > 0");
		if (v[7] < 0) return fail("con < 0, must have con >= 0");
		break;
	case ORC_FERRER:
		if (v[6] <= 0) return fail("rout <= 0, must have rout >= 0");
		if (v[7] < 0) return fail("a < 0, must have a >= 0");
		if (v[8] > 2) return fail("b > 2, must have b <= 2");
		break;
	case ORC_KING:
		if (v[6] <= 0) return fail("rc <= 0, must have rc > 0");
		if (v[7] <= 0) return fail("rt <= 0, must have rt > 0");
		if (v[8] < 0) return fail("a < 0, must have a >=0");
		break;
	case ORC_BROKENEXP:
		if (v[6] <= 0) return fail("h1 <= 0, must have h1 > 0");
		if (v[7] <= 0) return fail("h2 <= 0, must have h2 > 0");
		if (v[8] <= 0) return fail("rb <= 0, must have rb > 0");
		break;
	case ORC_PSF:
		if (!m->psf || m->psf_w == 0 || m->psf_h == 0) {
			return fail("No psf present in the model, cannot produce a psf profile");
		}
		break;
	case ORC_SKY: case ORC_NULL:
		break;
	default:
		return fail("Unknown profile kind");
	}
	return 0;
}

static void fill_radial(radial_t *r, const orc_profile *pp, const orc_model *m)
{
	const double *v = pp->par;
	memset(r, 0, sizeof(*r));
	r->kind = pp->kind;
	r->xcen = v[ORC_P_XCEN];
	r->ycen = v[ORC_P_YCEN];
	r->mag = v[ORC_P_MAG];
	r->ang = v[ORC_P_ANG];
	r->axrat = v[ORC_P_AXRAT];
	r->box = v[ORC_P_BOX];
	r->rough = pp->rough;
	r->adjust = pp->adjust;
	r->rescale_flux = pp->rescale_flux;
	r->resolution = pp->resolution;
	r->max_recursions = pp->max_recursions;
	r->acc = pp->acc;
	r->rscale_switch = pp->rscale_switch;
	r->rscale_max = pp->rscale_max;
	r->rescale_factor = 1;
	switch (pp->kind) {
	case ORC_SERSIC: r->re = v[6]; r->nser = v[7]; break;
	case ORC_CORESERSIC: r->re = v[6]; r->nser = v[7]; r->rb = v[8]; r->a = v[9]; r->b = v[10]; break;
	case ORC_MOFFAT: r->fwhm = v[6]; r->con = v[7]; break;
	case ORC_FERRER: r->rout = v[6]; r->a = v[7]; r->b = v[8]; break;
	case ORC_KING: r->rc = v[6]; r->rt = v[7]; r->a = v[8]; break;
	case ORC_BROKENEXP: r->h1 = v[6]; r->h2 = v[7]; r->rb = v[8]; r->a = v[9]; break;
	}
	r->magzero = m->magzero;
	r->image_scale_x = m->scale_x;
	r->image_scale_y = m->scale_y;
	if (r->kind == ORC_SERSIC) {
		sersic_choose_rfactor(r);
	}
}

int orc_profile_constants(const orc_model *m, const orc_profile *pp, orc_constants *c)
{
	radial_t r;
	unsigned int fs = m->finesampling ? m->finesampling : 1;
	if (!is_radial(pp->kind)) {
		return fail("not a radial profile");
	}
	if (validate_profile(pp, m)) {
		return -1;
	}
	fill_radial(&r, pp, m);
	initial_calculations(&r);
	c->rscale = r.rscale;
	c->ie = r.ie;
	c->bn = r.bn;
	c->lumtot = r.lumtot;
	c->rescale_factor = r.rescale_factor;
	c->rscale_switch = r.rscale_switch;
	c->rscale_max = r.rscale_max;
	c->acc = r.acc;
	c->resolution = r.resolution;
	c->cos_ang = r.cos_ang;
	c->sin_ang = r.sin_ang;
	c->flux_scale = get_pixel_scale(&r, m->scale_x / fs, m->scale_y / fs);
	return 0;
}

/* Model::analyze_expansion_requirements (src/model.cpp:152-184): the PSF
 * padding, and what the mask needs. With an adjustable mask and convolution,
 * the padding is needed only if the mask's bounding box (times the
 * finesampling) lies closer than half the PSF to an edge. */
typedef struct {
	unsigned int pad_x, pad_y;
	int mask_needs_convolution, mask_needs_psf_padding, mask_needs_adjustment;
} expansion_t;

static expansion_t analyze_expansion(const orc_model *m, int conv, unsigned int fs)
{
	expansion_t e = {0, 0, 0, 0, 0};
	int needs_padding = conv;
	if (m->mask && !m->adjust_mask) {
		/* a mask used as given: padding if it is larger than the model (times
		 * the finesampling) in both directions, whether or not anything is
		 * convolved (src/model.cpp:165-167) */
		needs_padding = m->mask_w > m->width * fs && m->mask_h > m->height * fs;
	}
	else if (m->mask && conv) {
		/* Surface::bounding_box (include/profit/image.h:472-501): [lb, ub) of
		 * the non-zero pixels, empty (all zero) for an all-zero mask */
		unsigned int lbx = m->width, lby = m->height, ubx = 0, uby = 0, i, j;
		int any = 0;
		for (j = 0; j < m->height; j++) {
			for (i = 0; i < m->width; i++) {
				if (!m->mask[i + (size_t)j * m->width]) continue;
				if (i < lbx) lbx = i;
				if (j < lby) lby = j;
				if (i + 1 > ubx) ubx = i + 1;
				if (j + 1 > uby) uby = j + 1;
				any = 1;
			}
		}
		if (!any) lbx = lby = ubx = uby = 0;
		{
			const unsigned int lowx = lbx * fs, lowy = lby * fs;
			const unsigned int upx = m->width * fs - ubx * fs, upy = m->height * fs - uby * fs;
			const unsigned int nx = m->psf_w / 2, ny = m->psf_h / 2;
			needs_padding = !(lowx >= nx && lowy >= ny) || !(upx >= nx && upy >= ny);
		}
		e.mask_needs_convolution = 1;
		e.mask_needs_psf_padding = needs_padding;
	}
	if (needs_padding) {
		e.pad_x = m->psf_w / 2;
		e.pad_y = m->psf_h / 2;
	}
	/* Model::needs_adjustment (src/model.cpp:221-228) */
	e.mask_needs_adjustment = m->mask && m->adjust_mask &&
	                          (e.mask_needs_convolution || e.mask_needs_psf_padding || fs > 1);
	return e;
}

/* Model::adjust (src/model.cpp:230-246): the mask upsampled by the
 * finesampling (Mask::upsample, src/image.cpp:51-65), extended by the PSF
 * padding (Surface::extend) and expanded by half the PSF (Mask::expand_by,
 * src/image.cpp:112-160: a drawing pixel is set if any mask pixel within
 * half the PSF is). Returns a new dw x dh mask. */
static unsigned char *adjusted_mask(const orc_model *m, const expansion_t *e, unsigned int fs, unsigned int dw,
                                    unsigned int dh)
{
	const unsigned int uw = m->width * fs, uh = m->height * fs;
	unsigned char *a = (unsigned char *)calloc((size_t)dw * dh, 1), *b;
	unsigned int i, j;
	for (j = 0; j < uh; j++) {
		for (i = 0; i < uw; i++) {
			a[(i + e->pad_x) + (size_t)(j + e->pad_y) * dw] = m->mask[i / fs + (size_t)(j / fs) * m->width] != 0;
		}
	}
	if (!e->mask_needs_convolution) return a;
	b = (unsigned char *)calloc((size_t)dw * dh, 1);
	{
		const unsigned int px = m->psf_w / 2, py = m->psf_h / 2;
		for (j = 0; j < dh; j++) {
			for (i = 0; i < dw; i++) {
				const unsigned int y0 = j >= py ? j - py : 0, y1 = j + py < dh ? j + py : dh - 1;
				const unsigned int x0 = i >= px ? i - px : 0, x1 = i + px < dw ? i + px : dw - 1;
				unsigned int x, y;
				int set = a[i + (size_t)j * dw];
				for (y = y0; y <= y1 && !set; y++) {
					for (x = x0; x <= x1; x++) {
						if (a[x + (size_t)y * dw]) {
							set = 1;
							break;
						}
					}
				}
				b[i + (size_t)j * dw] = (unsigned char)set;
			}
		}
	}
	free(a);
	return b;
}

/* Model::analyze_inputs (src/model.cpp:186-219) */
int orc_output_dims(const orc_model *m, const orc_profile *profiles, int n_profiles,
                    unsigned int *out_w, unsigned int *out_h, unsigned int *draw_w, unsigned int *draw_h)
{
	int i, conv = 0;
	unsigned int fs = m->finesampling ? m->finesampling : 1;
	unsigned int pad_x = 0, pad_y = 0;
	if (m->width == 0 || m->height == 0) return fail("Model's requested dimensions are 0");
	if (m->scale_x <= 0) return fail("Model's scale_x cannot be negative or zero");
	if (m->scale_y <= 0) return fail("Model's scale_y cannot be negative or zero");
	for (i = 0; i < n_profiles; i++) {
		conv |= profiles[i].convolve != 0;
	}
	/* src/model.cpp:198-201 */
	if (m->mask && m->adjust_mask && (m->mask_w != m->width || m->mask_h != m->height)) {
		return fail("Mask dimensions != model dimensions");
	}
	if (conv && (!m->psf || m->psf_w == 0 || m->psf_h == 0)) {
		return fail("No psf provided but profile(s) requested convolution");
	}
	for (i = 0; i < n_profiles; i++) {
		if (validate_profile(&profiles[i], m)) return -1;
	}
	{
		const expansion_t e = analyze_expansion(m, conv, fs);
		pad_x = e.pad_x;
		pad_y = e.pad_y;
	}
	*draw_w = m->width * fs + 2 * pad_x;
	*draw_h = m->height * fs + 2 * pad_y;
	/* src/model.cpp:277-283 */
	if (m->mask && !m->adjust_mask && (m->mask_w != *draw_w || m->mask_h != *draw_h)) {
		snprintf(g_err, sizeof g_err, "Mask dimensions != drawing dimensions: [%u, %u] != [%u, %u]", m->mask_w,
		         m->mask_h, *draw_w, *draw_h);
		return -1;
	}
	*out_w = m->width * fs;
	*out_h = m->height * fs;
	if (fs > 1 && !m->return_finesampled) {
		*out_w = (*out_w + fs - 1) / fs;
		*out_h = (*out_h + fs - 1) / fs;
	}
	return 0;
}

/* Model::evaluate + produce_image, src/model.cpp:259-360 */
int orc_evaluate(const orc_model *m, const orc_profile *profiles, int n_profiles,
                 double *out, unsigned int *out_w, unsigned int *out_h,
                 signed char *depth, long long *level_counts)
{
	unsigned int ow, oh, dw, dh, pad_x = 0, pad_y = 0, fs = m->finesampling ? m->finesampling : 1;
	int i, conv = 0;
	size_t npix;
	const unsigned char *mask = NULL;
	unsigned char *adj = NULL;
	double *model_image, *to_convolve = NULL, *psf = NULL;
	double sx, sy;
	int threads = m->omp_threads;

	if (orc_output_dims(m, profiles, n_profiles, &ow, &oh, &dw, &dh)) {
		return -1;
	}
	for (i = 0; i < n_profiles; i++) {
		conv |= profiles[i].convolve != 0;
	}
	{
		const expansion_t e = analyze_expansion(m, conv, fs);
		pad_x = e.pad_x;
		pad_y = e.pad_y;
		/* the mask the profiles and the convolution see: adjusted (Model::evaluate,
		 * src/model.cpp:269-286), as given, or none */
		if (m->mask && m->adjust_mask && e.mask_needs_adjustment) mask = adj = adjusted_mask(m, &e, fs, dw, dh);
		else if (m->mask && m->adjust_mask) mask = m->mask;  /* no adjustment: model = drawing dims */
		else mask = m->mask;
	}
	npix = (size_t)dw * dh;
	model_image = (double *)calloc(npix, sizeof(double));
	if (conv) {
		to_convolve = (double *)calloc(npix, sizeof(double));
	}
	if (m->psf && m->psf_w && m->psf_h) {
		/* Model::set_psf normalises (include/profit/model.h:148-158, src/image.cpp:208-215) */
		size_t np = (size_t)m->psf_w * m->psf_h, q;
		double sum = 0;
		psf = (double *)malloc(sizeof(double) * np);
		for (q = 0; q < np; q++) sum += m->psf[q];
		for (q = 0; q < np; q++) psf[q] = sum > 0 ? m->psf[q] / sum : m->psf[q];
	}
	sx = m->scale_x / fs;
	sy = m->scale_y / fs;

	for (i = 0; i < n_profiles; i++) {
		const orc_profile *pp = &profiles[i];
		double *target = pp->convolve ? to_convolve : model_image;
		if (depth) {
			memset(depth + (size_t)i * npix, -1, npix);
		}
		if (is_radial(pp->kind)) {
			radial_t r;
			fill_radial(&r, pp, m);
			initial_calculations(&r);
			r.xc = r.xcen + pad_x * sx; /* src/radial.cpp:254-255 */
			r.yc = r.ycen + pad_y * sy;
			r.depth = depth ? depth + (size_t)i * npix : NULL;
			r.depth_w = dw;
			evaluate_radial(&r, target, dw, dh, mask, sx, sy, threads);
			if (level_counts) {
				memcpy(level_counts + (size_t)i * 32, r.counts, sizeof(r.counts));
			}
		}
		else if (pp->kind == ORC_SKY) { /* src/sky.cpp:42-63 */
			double bg = pp->par[6] / (fs * fs);
			size_t q;
			for (q = 0; q < npix; q++) {
				if (mask && !mask[q]) continue;
				target[q] += bg;
			}
		}
		else if (pp->kind == ORC_PSF) {
			evaluate_psf_profile(pp, m, psf, target, dw, dh, sx, sy, pad_x, pad_y);
		}
	}

	if (conv) {
		/* Convolver::convolve (src/convolve.cpp:55-79): images smaller than
		 * the kernel are extended first (with the max() quirk of
		 * include/profit/image.h:204-207) */
		double *conv_out;
		if (!(dw >= m->psf_w && dh >= m->psf_h)) {
			unsigned int nx = dw > m->psf_w ? dw : m->psf_w;
			unsigned int ny = nx;
			double *ext = (double *)calloc((size_t)nx * ny, sizeof(double));
			double *res = (double *)calloc((size_t)nx * ny, sizeof(double));
			unsigned char *emask = NULL;
			unsigned int a, b;
			for (b = 0; b < dh; b++) for (a = 0; a < dw; a++) ext[a + (size_t)b * nx] = to_convolve[a + (size_t)b * dw];
			if (mask) {
				emask = (unsigned char *)calloc((size_t)nx * ny, 1);
				for (b = 0; b < dh; b++) for (a = 0; a < dw; a++) emask[a + (size_t)b * nx] = mask[a + (size_t)b * dw];
			}
			orc_convolve_brute(ext, nx, ny, psf, m->psf_w, m->psf_h, emask, res, m->convolver == 1, threads);
			for (b = 0; b < dh; b++) for (a = 0; a < dw; a++) to_convolve[a + (size_t)b * dw] = res[a + (size_t)b * nx];
			free(ext);
			free(res);
			free(emask);
			conv_out = to_convolve;
		}
		else {
			conv_out = (double *)malloc(sizeof(double) * npix);
			orc_convolve_brute(to_convolve, dw, dh, psf, m->psf_w, m->psf_h, mask, conv_out, m->convolver == 1, threads);
			free(to_convolve);
			to_convolve = conv_out;
		}
		{
			size_t q;
			for (q = 0; q < npix; q++) model_image[q] += to_convolve[q];
		}
	}

	/* crop the psf padding (src/model.cpp:289-306) then optionally downsample */
	{
		unsigned int cw = dw - 2 * pad_x, ch = dh - 2 * pad_y, a, b;
		if (fs > 1 && !m->return_finesampled) {
			/* Image::downsample(SUM), src/image.cpp:250-262 */
			unsigned int ddw = (cw + fs - 1) / fs;
			memset(out, 0, sizeof(double) * (size_t)ow * oh);
			for (b = 0; b < ch; b++) {
				for (a = 0; a < cw; a++) {
					out[(a / fs) + (size_t)(b / fs) * ddw] += model_image[(a + pad_x) + (size_t)(b + pad_y) * dw];
				}
			}
		}
		else {
			for (b = 0; b < ch; b++) {
				for (a = 0; a < cw; a++) {
					out[a + (size_t)b * cw] = model_image[(a + pad_x) + (size_t)(b + pad_y) * dw];
				}
			}
		}
	}
	/* image &= mask after an adjustment (src/model.cpp:313-317): the model's
	 * own mask over the output. (For finesampled output the reference's
	 * element-wise product runs past the smaller mask, undefined; here output
	 * pixel (x, y) takes mask pixel (x / fs, y / fs).) */
	if (adj) {
		unsigned int a, b;
		const unsigned int f = (fs > 1 && m->return_finesampled) ? fs : 1;
		for (b = 0; b < oh; b++) {
			for (a = 0; a < ow; a++) {
				if (!m->mask[a / f + (size_t)(b / f) * m->width]) out[a + (size_t)b * ow] = 0;
			}
		}
	}
	*out_w = ow;
	*out_h = oh;
	free(model_image);
	free(to_convolve);
	free(psf);
	free(adj);
	return 0;
}
