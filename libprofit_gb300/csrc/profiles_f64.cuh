// FP64 profile functions with the reference's operation order. Translation
// units including this file are compiled with -fmad=false so that no multiply
// and add is fused, as in the reference's x86-64 build.
//
//   boxy_r            include/profit/radial.h:93-102
//   sersic            src/sersic.cpp:79-198 (r_factor specialisations kept)
//   coresersic        src/coresersic.cpp:51-59
//   moffat            src/moffat.cpp:52-58
//   ferrer            src/ferrer.cpp:50-60
//   king              src/king.cpp:51-59
//   brokenexp         src/brokenexponential.cpp:38-94
#pragma once

#include <cmath>

#include "pf_device.cuh"

namespace pf {
namespace f64 {

__device__ __forceinline__ double boxy_r(double box, double x, double y)
{
	if (box == 0) {
		return sqrt(x * x + y * y);
	}
	double box_plus_2 = box + 2.;
	return pow(pow(fabs(x), box_plus_2) + pow(fabs(y), box_plus_2), 1. / box_plus_2);
}

__device__ __forceinline__ double sersic(const ProfileDev &p, double x, double y)
{
	const double box = p.par[PF_P_BOX], re = p.par[6], nser = p.par[7];
	double B = box + 2;
	double base, rf;
	if (p.rf_boxy) {
		base = pow(fabs(x / re), B) + pow(fabs(y / re), B);
		double invexp = nser * B;
		switch (p.rf_t) {
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
		base = (x * x + y * y) / (re * re);
		double invexp = nser;
		switch (p.rf_t) {
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
	return exp(-p.bn * (rf - 1));
}

__device__ __forceinline__ double coresersic_r(const ProfileDev &p, double r)
{
	const double re = p.par[6], nser = p.par[7], rb = p.par[8], a = p.par[9], b = p.par[10];
	return pow(1 + pow(r / rb, -a), b / a) * exp(-p.bn * pow((pow(r, a) + pow(rb, a)) / pow(re, a), 1 / (nser * a)));
}

__device__ __forceinline__ double king_r(const ProfileDev &p, double r)
{
	const double rc = p.par[6], rt = p.par[7], a = p.par[8];
	if (r < rt) {
		return pow(1 / pow(1 + pow(r / rc, 2), 1 / a) - 1 / pow(1 + pow(rt / rc, 2), 1 / a), a);
	}
	return 0;
}

__device__ __forceinline__ double broken_exponential(double r, double h1, double h2, double rb, double a)
{
	double base = r - rb;
	double expo = 1 / h1 - 1 / h2;
	if (a * base < 40) {
		base = log(1 + exp(a * base)) / a;
	}
	return exp(-r / h1 + expo * base);
}

// evaluate_at for one radial kind at profile coordinates (x, y)
__device__ __forceinline__ double evaluate_at(const ProfileDev &p, double x, double y)
{
	const double box = p.par[PF_P_BOX];
	switch (p.kind) {
	case PF_SERSIC:
		return sersic(p, x, y);
	case PF_CORESERSIC:
		return coresersic_r(p, boxy_r(box, x, y));
	case PF_MOFFAT: {
		double r = boxy_r(box, x, y);
		double r_factor = r / p.rscale;
		return pow(1 + r_factor * r_factor, -p.par[7]);
	}
	case PF_FERRER: {
		double r = boxy_r(box, x, y);
		double r_factor = r / p.rscale;
		if (r_factor < 1) {
			return pow(1 - pow(r_factor, 2 - p.par[8]), p.par[7]);
		}
		return 0;
	}
	case PF_KING:
		return king_r(p, boxy_r(box, x, y));
	case PF_BROKENEXP:
		return broken_exponential(boxy_r(box, x, y), p.par[6], p.par[7], p.par[8], p.par[9]);
	case PF_USER:
		return user::evaluate_at(p.par, p.rscale, x, y);
	}
	return 0;
}

// RadialProfile::_image_to_profile_coordinates, src/radial.cpp:46-53
__device__ __forceinline__ void to_profile(const ProfileDev &p, double x, double y, double &xp, double &yp)
{
	x -= p.xc;
	y -= p.yc;
	xp = x * p.cos_ang + y * p.sin_ang;
	yp = -x * p.sin_ang + y * p.cos_ang;
	yp /= p.par[PF_P_AXRAT];
}

}  // namespace f64
}  // namespace pf
