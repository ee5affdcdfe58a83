// Per-profile setup on the device, in FP64, one thread per profile:
// RadialProfile::initial_calculations (src/radial.cpp:137-199) with each
// profile's get_rscale / get_lumtot / adjust_* overrides, the centre shift of
// RadialProfile::evaluate (src/radial.cpp:253-255), the flux scale
// (src/radial.cpp:219-222, src/sersic.cpp:319-325), the sky level
// (src/sky.cpp:42-45) and the psf profile's magnitude scale (src/psf.cpp:66).
// Also the per-model PSF normalisation of Model::set_psf
// (include/profit/model.h:148-158, src/image.cpp:204-215).
// Compiled with -fmad=false: the reference's arithmetic is not contracted.
#include <cmath>

#include "pf_device.cuh"
#include "profiles_f64.cuh"
#include "profiles_grad.cuh"
#include "specfun.cuh"

namespace pf {

namespace {

struct CoreSersicIntegrand {  // src/coresersic.cpp:80-87
	const ProfileDev *p;
	__device__ double operator()(double r) const
	{
		const double re = p->par[6], nser = p->par[7], rb = p->par[8], a = p->par[9], b = p->par[10];
		return r * pow(1 + pow(r / rb, -a), b / a) *
		       exp(-p->bn * pow((pow(r, a) + pow(rb, a)) / pow(re, a), 1 / (nser * a)));
	}
};

struct KingIntegrand {  // src/king.cpp:76-84
	const ProfileDev *p;
	__device__ double operator()(double r) const
	{
		const double rc = p->par[6], rt = p->par[7], a = p->par[8];
		if (r < rt) {
			return r * pow(1 / pow(1 + pow(r / rc, 2), 1 / a) - 1 / pow(1 + pow(rt / rc, 2), 1 / a), a);
		}
		return 0;
	}
};

struct BrokenExpIntegrand {  // src/brokenexponential.cpp:111-113
	const ProfileDev *p;
	__device__ double operator()(double r) const
	{
		return r * f64::broken_exponential(r, p->par[6], p->par[7], p->par[8], p->par[9]);
	}
};

__device__ double get_rscale(const ProfileDev &p)
{
	switch (p.kind) {
	case PF_SERSIC: case PF_CORESERSIC: return p.par[6];
	case PF_MOFFAT: return p.par[6] / (2 * sqrt(pow(2, (1 / p.par[7])) - 1));  // src/moffat.cpp:81-83
	case PF_FERRER: return p.par[6];
	case PF_KING: return p.par[7];
	case PF_BROKENEXP: return p.par[6] * 4;
	case PF_USER: return user::get_rscale(p.par);
	}
	return 0;
}

__device__ double get_lumtot(ProfileDev &p)
{
	switch (p.kind) {
	case PF_SERSIC: {  // src/sersic.cpp:283-289
		const double re = p.par[6], nser = p.par[7];
		double g_factor = sf::gammafn(2 * nser);
		return pow(re, 2) * 2 * M_PI * nser * g_factor * exp(p.bn) / pow(p.bn, 2 * nser);
	}
	case PF_CORESERSIC:  // src/coresersic.cpp:92-104
		return 2 * M_PI * sf::qag(CoreSersicIntegrand{&p}, 0., 0., true, 1e-4, 1e-4, nullptr);
	case PF_MOFFAT:  // src/moffat.cpp:77-79
		return pow(p.rscale, 2) * M_PI / (p.par[7] - 1);
	case PF_FERRER: {  // src/ferrer.cpp:78-101
		const double a = p.par[7], b = p.par[8];
		double g_factor = a * sf::beta(a, 1 + 2 / (2 - b));
		return pow(p.par[6], 2) * M_PI * g_factor;
	}
	case PF_KING:  // src/king.cpp:87-96
		return 2 * M_PI * sf::qag(KingIntegrand{&p}, 0., p.par[7], false, 1e-4, 1e-4, nullptr);
	case PF_BROKENEXP:  // src/brokenexponential.cpp:115-126
		return 2 * M_PI * sf::qag(BrokenExpIntegrand{&p}, 0., 0., true, 1e-4, 1e-4, nullptr);
	case PF_USER:
		return user::get_lumtot(p.par, p.rscale);
	}
	return 0;
}

// Inverse-gamma values a sersic profile's setup needs, solved by separate
// lanes of the profile's warp: P^-1(1 - n^2/2000, 2n) for the switch radius
// and P^-1(0.9999, 2n) for rscale_max (SersicProfile::fluxfrac), and
// d bn / d n for the adjoint.
struct SersicSolves {
	double q_switch, q_max, dbn;
};

// SersicProfile::fluxfrac (src/sersic.cpp:257-260) given qgamma(fraction, 2n)
__device__ double sersic_fluxfrac(const ProfileDev &p, double qgamma_value)
{
	double ratio = qgamma_value / p.bn;
	return p.par[6] * pow(ratio, p.par[7]);
}

__device__ double moffat_fluxfrac(const ProfileDev &p, double fraction)  // src/moffat.cpp:73-75
{
	return p.rscale * sqrt(pow(1 - fraction, 1 / (1 - p.par[7])) - 1);
}

__device__ double adjust_rscale_switch(const ProfileDev &p, const SersicSolves &sv)
{
	switch (p.kind) {
	case PF_SERSIC: {  // src/sersic.cpp:262-272 (fraction 1 - nser^2 / 2e3)
		double rs = ceil(sersic_fluxfrac(p, sv.q_switch));
		rs = sf::dmax(sf::dmin(rs, 20.), 2.);
		return rs / p.par[6];
	}
	case PF_MOFFAT: {  // src/moffat.cpp:88-91
		double rs = sf::dmax(moffat_fluxfrac(p, 0.9999), 1.823 * p.par[6]);
		return sf::dmax(sf::dmin(rs, 20.), 2.) / p.rscale;
	}
	case PF_CORESERSIC: return 1;     // src/coresersic.cpp:119-121
	case PF_FERRER: return 0.5;       // src/ferrer.cpp:103-105
	case PF_KING: return 0.5;         // src/king.cpp:98-100
	case PF_BROKENEXP: return 1;      // src/brokenexponential.cpp:128-130
	case PF_USER: return user::adjust_rscale_switch(p.par, p.rscale);
	}
	return 1;
}

__device__ double adjust_rscale_max(const ProfileDev &p, const SersicSolves &sv)
{
	switch (p.kind) {
	case PF_SERSIC: return ceil(sf::dmax(sersic_fluxfrac(p, sv.q_max), 2.) / p.par[6]);  // src/sersic.cpp:274-276
	case PF_MOFFAT: return ceil(sf::dmax(moffat_fluxfrac(p, 0.9999), 2.) / p.rscale);  // src/moffat.cpp:93-95
	case PF_CORESERSIC: return 100;
	case PF_FERRER: return 1;
	case PF_KING: return 1.5;
	case PF_BROKENEXP: return 100;
	case PF_USER: return user::adjust_rscale_max(p.par, p.rscale);
	}
	return 0;
}

__device__ double adjust_acc(const ProfileDev &p, double acc)
{
	switch (p.kind) {
	case PF_SERSIC:  // src/sersic.cpp:278-281
		acc /= sqrt(p.par[7]);
		return sf::dmax(0.1, acc) / p.par[PF_P_AXRAT];
	case PF_MOFFAT:  // src/moffat.cpp:97-99
		return 0.1 / p.par[PF_P_AXRAT];
	case PF_USER:
		return user::adjust_acc(p.par, acc);
	}
	return acc;
}

__device__ bool almost_equals(double x, double y)  // src/utils.cpp:101-103 with e = 1e-10
{
	return fabs(x - y) < fabs(1e-10);
}

__device__ void choose_rfactor(ProfileDev &p)  // src/sersic.cpp:225-255
{
	const double box = p.par[PF_P_BOX];
	double inv_exponent = p.par[7];
	p.rf_boxy = box != 0;
	if (box != 0) {
		inv_exponent *= (box + 2);
	}
	if (almost_equals(inv_exponent, 0.5)) p.rf_t = RF_POINTFIVE;
	else if (almost_equals(inv_exponent, 1)) p.rf_t = RF_ONE;
	else if (almost_equals(inv_exponent, 2)) p.rf_t = RF_TWO;
	else if (almost_equals(inv_exponent, 3)) p.rf_t = RF_THREE;
	else if (almost_equals(inv_exponent, 4)) p.rf_t = RF_FOUR;
	else if (almost_equals(inv_exponent, 8)) p.rf_t = RF_EIGHT;
	else if (almost_equals(inv_exponent, 16)) p.rf_t = RF_SIXTEEN;
	else p.rf_t = RF_GENERAL;
}

__device__ int clamp_index(double v, int lo, int hi)
{
	if (!(v > lo)) return lo;   // also catches NaN
	if (v > hi) return hi;
	return (int)v;
}

// Constants of the FP32 path (profiles_f32.cuh), folded once per profile.
__device__ void fold_single_precision(ProfileDev &p)
{
	const double box = p.par[PF_P_BOX];
	const double B = box + 2;
	p.fxc_hi = (float)p.xc;
	p.fxc_lo = (float)(p.xc - (double)p.fxc_hi);
	p.fyc_hi = (float)p.yc;
	p.fyc_lo = (float)(p.yc - (double)p.fyc_hi);
	p.fcos = (float)p.cos_ang;
	p.fsin = (float)p.sin_ang;
	p.finv_axrat = (float)(1 / p.par[PF_P_AXRAT]);
	p.finv_rscale = (float)(1 / p.rscale);
	p.fswitch = (float)p.rscale_switch;
	p.frmax = (float)p.rscale_max;
	p.facc = (float)p.acc;
	p.fflux_scale = (float)p.flux_scale;
	p.fboxy = box != 0;
	float *c = p.fpar;
	for (int i = 0; i < 12; i++) c[i] = 0.f;
	c[FP_B] = (float)B;
	c[FP_INVB] = (float)(1 / B);
	const double log2e = 1.4426950408889634;
	switch (p.kind) {
	case PF_SERSIC: {
		const double re = p.par[6], n = p.par[7];
		c[FP_S_INV_RE2] = (float)(1 / (re * re));
		c[FP_S_HALF_INV_N] = (float)(0.5 / n);
		c[FP_S_INV_RE] = (float)(1 / re);
		c[FP_S_INV_NB] = (float)(1 / (n * B));
		c[FP_S_K] = (float)(p.bn * log2e);
		break;
	}
	case PF_CORESERSIC: {
		const double re = p.par[6], n = p.par[7], rb = p.par[8], a = p.par[9], b = p.par[10];
		c[FP_C_A] = (float)a;
		c[FP_C_B_OVER_A] = (float)(b / a);
		c[FP_C_INV_RB] = (float)(1 / rb);
		c[FP_C_RB_A] = (float)pow(rb, a);
		c[FP_C_INV_RE_A] = (float)(1 / pow(re, a));
		c[FP_C_K] = (float)(p.bn * log2e);
		c[FP_C_INV_NA] = (float)(1 / (n * a));
		break;
	}
	case PF_MOFFAT:
		c[FP_M_INV_RS2] = (float)(1 / (p.rscale * p.rscale));
		c[FP_M_INV_RS] = (float)(1 / p.rscale);
		c[FP_M_CON] = (float)p.par[7];
		break;
	case PF_FERRER:
		c[FP_F_INV_ROUT] = (float)(1 / p.rscale);
		c[FP_F_A] = (float)p.par[7];
		c[FP_F_2MB] = (float)(2 - p.par[8]);
		break;
	case PF_KING: {
		const double rc = p.par[6], rt = p.par[7], a = p.par[8];
		c[FP_K_RT] = (float)rt;
		c[FP_K_INV_RC] = (float)(1 / rc);
		c[FP_K_A] = (float)a;
		c[FP_K_INV_A] = (float)(1 / a);
		c[FP_K_TEMP] = (float)(1 / pow(1 + pow(rt / rc, 2), 1 / a));
		break;
	}
	case PF_BROKENEXP: {
		const double h1 = p.par[6], h2 = p.par[7], rb = p.par[8], a = p.par[9];
		c[FP_E_RB] = (float)rb;
		c[FP_E_A] = (float)a;
		c[FP_E_INV_A] = (float)(1 / a);
		c[FP_E_INV_H1] = (float)(1 / h1);
		c[FP_E_EXPO] = (float)(1 / h1 - 1 / h2);
		break;
	}
	}
}

// Constants of the adjoint. For a sersic profile
//   ln flux_scale = const - 0.4 ln(10) mag - ln lumtot(re, n) - ln axrat + ln r_box(box)
// with ln lumtot = 2 ln re + ln(2 pi) + ln n + lnGamma(2n) + bn - 2n ln bn
// (src/sersic.cpp:283-289) and r_box = pi B / (2 beta(1/B, 1/B)), B = box + 2
// (src/radial.cpp:150-152). bn(n) solves P(2n, bn) = 1/2, so by implicit
// differentiation d bn / d n = -2 (dP/da)(2n, bn) / p(bn; 2n), p the gamma
// density; dP/da is a central difference of P in its shape.
__device__ double dbn_dn(double n, double bn)
{
	const double a = 2 * n, d = 1e-4 * a;
	const double dpda = (sf::pgamma(bn, a + d) - sf::pgamma(bn, a - d)) / (2 * d);
	const double pdf = exp((a - 1.) * log(bn) - bn - lgamma(a));
	return -2 * dpda / pdf;
}

// r f(r) d ln f / d par[6 + k]: the integrand of d lumtot / d par[6 + k]
// (divided by 2 pi) for the profiles whose lumtot is an integral
struct LumtotDerivIntegrand {
	const grad::GShape<double> *s;
	int k;
	__device__ double operator()(double r) const
	{
		double lnf, G, d[5] = {0., 0., 0., 0., 0.};
		if (!grad::radial_terms<double>(*s, r, lnf, G, d)) return 0.;
		const double f = exp(lnf);
		return f > 0. ? r * f * d[k] : 0.;
	}
};

// d ln flux_scale / d par[k] of the other radial profiles:
//   ln flux_scale = const - 0.4 ln(10) mag - ln get_lumtot(shape) - ln axrat + ln r_box(box)
// (src/radial.cpp:147-153). get_lumtot is closed-form for moffat
// (pi rs^2 / (con - 1), src/moffat.cpp:77-79) and ferrer (pi rout^2 a B(a, 1 +
// 2/(2-b)), src/ferrer.cpp:78-101), and 2 pi int_0^R r f(r) dr otherwise
// (src/coresersic.cpp:92-104, src/king.cpp:87-96, src/brokenexponential.cpp:
// 115-126), whose derivatives are the integrals of r df/dpar over the same
// range (f vanishes at the king's R = rt), taken with the same QUADPACK
// routines at a tighter tolerance. `lum_int` = that integral.
__device__ void other_lumtot_derivatives(ProfileDev &p, double lum_int)
{
	const grad::GShape<double> s = grad::make_gshape<double>(p);
	switch (p.kind) {
	case PF_MOFFAT: {
		const double fwhm = p.par[6], con = p.par[7];
		p.dlnfs[6] = -2 / fwhm;
		p.dlnfs[7] = 1 / (con - 1) - 2 * (double)s.k[1];
		break;
	}
	case PF_FERRER: {
		const double rout = p.par[6], a = p.par[7], b = p.par[8];
		const double c = 1 + 2 / (2 - b);
		p.dlnfs[6] = -2 / rout;
		p.dlnfs[7] = -(1 / a + sf::digamma(a) - sf::digamma(a + c));
		p.dlnfs[8] = -(sf::digamma(c) - sf::digamma(a + c)) * 2 / ((2 - b) * (2 - b));
		break;
	}
	case PF_CORESERSIC:
	case PF_KING:
	case PF_BROKENEXP: {
		const int n_shape = p.kind == PF_CORESERSIC ? 5 : (p.kind == PF_KING ? 3 : 4);
		const bool infinite = p.kind != PF_KING;
		const double upper = p.kind == PF_KING ? p.par[7] : 0.;
		for (int k = 0; k < n_shape; k++) {
			const double dint = sf::qag(LumtotDerivIntegrand{&s, k}, 0., upper, infinite,
			                            1e-12 * fabs(lum_int), 1e-9, nullptr);
			p.dlnfs[6 + k] = -dint / lum_int;
		}
		break;
	}
	default:
		break;
	}
}

// `lum_int` = get_lumtot / (2 pi) for the integral profiles; `want` = the
// batch runs the adjoint (the integrals are skipped otherwise)
__device__ void adjoint_constants(ProfileDev &p, double dbn, double lum_int, int want)
{
	for (int k = 0; k < PF_NPAR; k++) p.dlnfs[k] = 0.;
	p.dbn = 0.;
	p.grad_ok = 0;
	if (p.kind < PF_SERSIC || p.kind > PF_BROKENEXP) {
		return;
	}
	const double q = p.par[PF_P_AXRAT], B = p.par[PF_P_BOX] + 2;
	p.dlnfs[PF_P_MAG] = -0.4 * log(10.);
	p.dlnfs[PF_P_AXRAT] = -1 / q;
	p.dlnfs[PF_P_BOX] = 1 / B + (2 / (B * B)) * (sf::digamma(1 / B) - sf::digamma(2 / B));
	if (p.kind == PF_SERSIC) {
		const double n = p.par[7], re = p.par[6];
		p.dbn = dbn;
		p.dlnfs[6] = -2 / re;
		p.dlnfs[7] = -(1 / n + 2 * sf::digamma(2 * n) + dbn - 2 * log(p.bn) - 2 * n * dbn / p.bn);
		if (p.adjust && p.rescale_flux && want) {
			// flux_scale also divides by P(2n, x), x = bn (rscale_max / re)^(1/n)
			// (src/sersic.cpp:302-311); rscale_max, when derived, moves in steps
			// (a ceiling) and contributes nothing between them
			const double lr = log(p.rscale_max) - log(re);
			const double x = p.bn * exp(lr / n);
			const double a = 2 * n, d = 1e-4 * a;
			const double P = sf::pgamma(x, a);
			const double dPda = (sf::pgamma(x, a + d) - sf::pgamma(x, a - d)) / (2 * d);
			const double px = exp((a - 1.) * log(x) - x - lgamma(a)) * x;  // x p(x; a)
			p.dlnfs[6] -= px * (-1 / (n * re)) / P;
			p.dlnfs[7] -= (2 * dPda + px * (dbn / p.bn - lr / (n * n))) / P;
		}
		p.fbn = (float)p.bn;
		p.fdbn = (float)dbn;
		p.fnser = (float)n;
		p.fre = (float)re;
	}
	else {
		if (p.kind == PF_CORESERSIC) p.dbn = dbn;
		if (want) other_lumtot_derivatives(p, lum_int);
	}
	p.grad_ok = 1;
}

__device__ void radial_setup(ProfileDev &p, const ModelDev &m, double bn, const SersicSolves &sv, int want_grad,
                             unsigned int *err)
{
	if (p.kind == PF_SERSIC) {
		choose_rfactor(p);
	}
	if (p.kind == PF_SERSIC || p.kind == PF_CORESERSIC) {  // src/sersic.cpp:297, src/coresersic.cpp:112
		p.bn = bn;
	}
	p.rscale = get_rscale(p);
	const double box = p.par[PF_P_BOX], axrat = p.par[PF_P_AXRAT];
	double b2 = box + 2;
	double r_box = M_PI * b2 / (2 * sf::beta(1 / b2, 1 / b2));
	const double lum_raw = get_lumtot(p);
	double lumtot = lum_raw * axrat / r_box;
	p.lumtot = lumtot;
	p.ie = pow(10, -0.4 * (p.par[PF_P_MAG] - m.magzero)) / lumtot;
	if (p.adjust) {
		p.rscale_switch = adjust_rscale_switch(p, sv);
		unsigned int res = (unsigned int)ceil(160 / (p.rscale_switch * p.rscale));
		res += res % 2;
		res = res < 16U ? res : 16U;
		res = res > 4U ? res : 4U;
		p.resolution = res;
		if (p.rscale_max == 0) {
			p.rscale_max = adjust_rscale_max(p, sv);
		}
		p.acc = adjust_acc(p, p.acc);
	}
	double angrad = fmod(p.par[PF_P_ANG] + 90, 360.) * M_PI / 180.;
	p.cos_ang = cos(angrad);
	p.sin_ang = sin(angrad);
	p.rescale_factor = 1;
	if (p.kind == PF_SERSIC && p.adjust && p.rescale_flux) {  // src/sersic.cpp:302-311
		double flux_r = p.bn * pow(p.rscale_max / p.par[6], 1 / p.par[7]);
		flux_r = sf::pgamma(flux_r, 2 * p.par[7]);
		p.rescale_factor = 1 / flux_r;
	}
	p.xc = p.par[PF_P_XCEN] + m.pad_x * m.sx;
	p.yc = p.par[PF_P_YCEN] + m.pad_y * m.sy;
	double flux_scale = m.sx * m.sy * p.ie;
	if (p.kind == PF_SERSIC && p.rescale_flux) {
		flux_scale *= p.rescale_factor;
	}
	p.flux_scale = flux_scale;

	// Culling box: a pixel whose centre has r_prof > rscale_max * rscale is
	// exactly 0 (src/radial.cpp:323-325). r_prof^2 = xp^2 + yp^2 with (xp,
	// yp * axrat) the centre offset rotated by the position angle, so the
	// pixels kept lie in an ellipse of semi-axes R (along (cos, sin)) and
	// R axrat, whose half-extents are R sqrt(cos^2 + axrat^2 sin^2) in x and
	// R sqrt(sin^2 + axrat^2 cos^2) in y. One pixel of margin.
	const double q2 = axrat * axrat;
	const double ex = sqrt(p.cos_ang * p.cos_ang + q2 * p.sin_ang * p.sin_ang);
	const double ey = sqrt(p.sin_ang * p.sin_ang + q2 * p.cos_ang * p.cos_ang);
	p.bbx0 = 0;
	p.bby0 = 0;
	p.bbx1 = (int)m.draw_w - 1;
	p.bby1 = (int)m.draw_h - 1;
	if (p.rscale_max > 0) {
		const double R = p.rscale_max * p.rscale;
		if (R == R && R < 1e12 && axrat > 0 && axrat <= 1) {
			const double hx = R * ex, hy = R * ey;
			p.bbx0 = clamp_index(floor((p.xc - hx) / m.sx - 0.5) - 1, 0, (int)m.draw_w);
			p.bbx1 = clamp_index(ceil((p.xc + hx) / m.sx - 0.5) + 1, -1, (int)m.draw_w - 1);
			p.bby0 = clamp_index(floor((p.yc - hy) / m.sy - 0.5) - 1, 0, (int)m.draw_h);
			p.bby1 = clamp_index(ceil((p.yc + hy) / m.sy - 0.5) + 1, -1, (int)m.draw_h - 1);
		}
	}
	// Subsampling box: a pixel is subsampled only if r_prof <= rscale_switch *
	// rscale (src/radial.cpp:327-331), so, as above, only within that ellipse.
	// Used to schedule the costly tiles first.
	p.sbx0 = p.sby0 = 0;
	p.sbx1 = p.sby1 = -1;
	if (is_radial(p.kind) && !p.rough) {
		const double R = p.rscale_switch * p.rscale;
		if (R == R && R < 1e12 && axrat > 0 && axrat <= 1) {
			const double hx = R * ex, hy = R * ey;
			p.sbx0 = clamp_index(floor((p.xc - hx) / m.sx - 0.5) - 1, 0, (int)m.draw_w);
			p.sbx1 = clamp_index(ceil((p.xc + hx) / m.sx - 0.5) + 1, -1, (int)m.draw_w - 1);
			p.sby0 = clamp_index(floor((p.yc - hy) / m.sy - 0.5) - 1, 0, (int)m.draw_h);
			p.sby1 = clamp_index(ceil((p.yc + hy) / m.sy - 0.5) + 1, -1, (int)m.draw_h - 1);
		}
		else {
			p.sbx1 = (int)m.draw_w - 1;
			p.sby1 = (int)m.draw_h - 1;
		}
	}
	fold_single_precision(p);
	adjoint_constants(p, sv.dbn, lum_raw / (2 * M_PI), want_grad);
	p.center_boost = p.kind == PF_SERSIC && p.adjust && p.par[7] > 1;
	unsigned int max_res = p.resolution;
	unsigned int max_rec = p.max_recursions;
	if (p.kind == PF_SERSIC && p.adjust && p.par[7] > 1) {  // central pixel, src/sersic.cpp:339-345
		max_res = max_res > 8U ? max_res : 8U;
		max_rec = max_rec > 10U ? max_rec : 10U;
	}
	if (!p.rough) {
		if (max_rec + 1 > (unsigned int)kMaxLevels) atomicOr(err, (unsigned int)ERR_LEVELS);
		if (max_res > (unsigned int)kMaxRes) atomicOr(err, (unsigned int)ERR_RES);
	}
}

}  // namespace

// The independent inverse-gamma solves of the sersic-like profiles, one per
// thread, the task in blockIdx.y so that each warp runs one kind of solve:
//   task 0  bn = P^-1(1/2, 2n)                 (sersic, coresersic)
//   task 1  P^-1(1 - n^2/2000, 2n)             (sersic switch radius, adjust)
//   task 2  P^-1(0.9999, 2n)                   (sersic rscale_max, adjust, rscale_max = 0)
__global__ void setup_solves_kernel(const ProfileDev *profs, int n_profiles, double *solves, unsigned int *err)
{
	// task blockIdx.y, profile i: each warp runs one kind of solve (a warp
	// mixing them would run their iterations one after another)
	const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
	if (t == 0 && blockIdx.y == 0) err[1] = 0xffffffffu;  // this pass's first invalid profile: none yet
	if (t >= n_profiles) {
		return;
	}
	const int task = (int)blockIdx.y, i = (int)t;
	const int kind = profs[i].kind;
	const double nser = profs[i].par[7];
	// a valid profile's solve depends on nser alone (kind and flags are fixed
	// per batch): kept while nser is (the keys, after the 3 n_profiles
	// values, start NaN; an invalid profile's stays NaN)
	double *key = solves + 3LL * n_profiles + (size_t)i * 3 + task;
	if (*key == nser) return;
	double v = 0.;
	const bool valid = param_rule(kind, profs[i].par) == PR_OK;
	if (!valid) {
		// invalid parameters (written on the device): the profile is not set up
	}
	else if (task == 0 && (kind == PF_SERSIC || kind == PF_CORESERSIC)) {
		v = sf::qgamma(0.5, 2 * nser, sf::bn_guess(nser));
	}
	else if (task == 1 && kind == PF_SERSIC && profs[i].adjust) {
		const double p = 1. - nser * nser / 2e3;
		v = sf::qgamma(p, 2 * nser, sf::wilson_hilferty_guess(p, 2 * nser));
	}
	else if (task == 2 && kind == PF_SERSIC && profs[i].adjust && profs[i].rscale_max_in == 0) {
		v = sf::qgamma(0.9999, 2 * nser, sf::wilson_hilferty_guess(0.9999, 2 * nser));
	}
	solves[(size_t)i * 3 + task] = v;
	*key = valid ? nser : CUDART_NAN;
}

__global__ void setup_profiles_kernel(const ModelDev *models, ProfileDev *profs, int n_profiles,
                                      const double *solves, int want_grad, unsigned int *tile_counter,
                                      unsigned int *err)
{
	if (blockIdx.x == 0 && threadIdx.x == 0) {
		// the eval kernels' work counters (two: the FP32 one's phases), then the
		// FP32 path's split-box pool counters (SplitPool::cnt) or the FP64
		// path's level pool counters (LevelPool64::cnt)
		for (int i = 0; i < 2 + kSplitCounters; i++) tile_counter[i] = 0;
	}
	const int t = blockIdx.x * blockDim.x + threadIdx.x;
	if (t >= n_profiles) {
		return;
	}
	const int kind = profs[t].kind;
	const double nser = profs[t].par[7];
	const double bn = solves[(size_t)t * 3 + 0];
	SersicSolves sv{solves[(size_t)t * 3 + 1], solves[(size_t)t * 3 + 2], 0.};
	if ((kind == PF_SERSIC || kind == PF_CORESERSIC) && want_grad) {
		sv.dbn = dbn_dn(nser, bn);
	}
	ProfileDev p = profs[t];
	const ModelDev &m = models[p.model];
	p.resolution = p.resolution_in;
	p.acc = p.acc_in;
	p.rscale_switch = p.rscale_switch_in;
	p.rscale_max = p.rscale_max_in;
	const int rule = param_rule(p.kind, p.par);
	if (rule != PR_OK) {
		// Parameters the reference's validate() refuses, written on the device
		// (pf_batch_set_params_dev, pf_step_graph): the first such profile is
		// recorded for pf_batch_check, and this one draws nothing and gets no
		// gradient (empty culling and subsampling boxes, zero flux scale).
		atomicMin(&err[1], ((unsigned int)t << 5) | (unsigned int)rule);
		p.bbx0 = p.bby0 = p.sbx0 = p.sby0 = 0;
		p.bbx1 = p.bby1 = p.sbx1 = p.sby1 = -1;
		p.flux_scale = 0.;
		p.fflux_scale = 0.f;
		for (int k = 0; k < PF_NPAR; k++) p.dlnfs[k] = 0.;
		p.grad_ok = 0;
		p.center_boost = 0;
	}
	else if (is_radial(p.kind)) {
		radial_setup(p, m, bn, sv, want_grad, err);
	}
	else if (p.kind == PF_SKY) {
		p.bg = p.par[6] / (m.fs * m.fs);  // src/sky.cpp:42-45
		p.fbg = (float)p.bg;
		p.grad_ok = 1;
	}
	else if (p.kind == PF_PSF) {
		p.psf_mag_scale = pow(10, -0.4 * (p.par[PF_P_MAG] - m.magzero));
	}
	profs[t] = p;
}

// One block per model: sum in element order (std::accumulate), then divide.
__global__ void normalise_psf_kernel(const ModelDev *models, const double *raw, double *norm)
{
	const ModelDev &m = models[blockIdx.x];
	if (m.psf_off < 0) {
		return;
	}
	const size_t n = (size_t)m.psf_w * m.psf_h;
	__shared__ double total;
	if (threadIdx.x == 0) {
		double s = 0.;
		for (size_t i = 0; i < n; i++) s += raw[m.psf_off + i];
		total = s;
	}
	__syncthreads();
	const double s = total;
	for (size_t i = threadIdx.x; i < n; i += blockDim.x) {
		double v = raw[m.psf_off + i];
		norm[m.psf_off + i] = s > 0 ? v / s : v;
	}
}

void launch_setup(const ModelDev *models, ProfileDev *profs, int n_profiles, int n_models,
                  unsigned int *tile_counter, unsigned int *err, const double *psf_raw, double *psf_norm,
                  bool have_psf, double *solves, int want_grad, cudaStream_t stream)
{
	// single-warp blocks: the FP64-heavy work spreads over as many SMs as possible
	if (n_profiles > 0) {
		setup_solves_kernel<<<dim3((unsigned int)((n_profiles + 31) / 32), 3), 32, 0, stream>>>(profs, n_profiles,
		                                                                                        solves, err);
	}
	int blocks = (n_profiles + 31) / 32;
	if (blocks < 1) blocks = 1;
	setup_profiles_kernel<<<blocks, 32, 0, stream>>>(models, profs, n_profiles, solves, want_grad, tile_counter,
	                                                 err);
	if (have_psf && n_models > 0) {
		normalise_psf_kernel<<<n_models, 128, 0, stream>>>(models, psf_raw, psf_norm);
	}
}

}  // namespace pf
