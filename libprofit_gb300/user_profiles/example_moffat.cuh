// An example user-defined radial profile: the Moffat profile of libprofit
// (src/moffat.cpp) under the name "usermoffat", with the same arithmetic, so
// that a library built with it renders "usermoffat" exactly as it renders
// the built-in "moffat". Build it in with
//     python libprofit_gb300/build.py --user-profile libprofit_gb300/user_profiles/example_moffat.cuh
//
// A user profile file defines, in namespace pf_user, the RadialProfile
// methods a libprofit profile class implements (include/profit/radial.h:
// 104-174, docs/new_profile.rst). `par` is the profile's 12 parameter slots:
// xcen, ycen, mag, ang, axrat, box (the radial ones, already checked by
// RadialProfile::validate's rules), then the profile's own n_params ones.
// Functions must be inline: every translation unit of the library sees them.
//   name, n_params (at most 6), param_names, param_defaults  the profile's
//       Model::add_profile name and its own parameters, slots 6, 7, ...
//   validate(par) -> 0, or k >= 1 for messages[k - 1] (at most 11 messages),
//       the invalid_parameter its validate() throws
//   get_rscale(par), get_lumtot(par, rscale), adjust_rscale_switch(par,
//       rscale) and adjust_rscale_max(par, rscale) (both in units of rscale),
//       adjust_acc(par, acc): as the RadialProfile virtuals of those names;
//       get_lumtot is the luminosity of the circular profile (the framework
//       applies axrat and boxiness, src/radial.cpp:147-153)
//   evaluate_at(par, rscale, x, y): the profile at profile coordinates (x, y)
// User profiles are evaluated in double precision (PF_ENV_DOUBLE) with the
// library's subsampling; the single-precision path and the adjoint refuse
// them.
#pragma once

#include <math.h>

namespace pf_user {

constexpr const char *name = "usermoffat";
constexpr int n_params = 2;
constexpr const char *param_names[n_params] = {"fwhm", "con"};
constexpr double param_defaults[n_params] = {3.0, 2.0};
constexpr const char *messages[] = {"fwhm <= 0, must have fwhm > 0", "con < 0, must have con >= 0"};

__host__ __device__ inline int validate(const double *par)
{
	if (par[6] <= 0) return 1;
	if (par[7] < 0) return 2;
	return 0;
}

__device__ inline double get_rscale(const double *par) { return par[6] / (2 * sqrt(pow(2, (1 / par[7])) - 1)); }

__device__ inline double get_lumtot(const double *par, double rscale) { return pow(rscale, 2) * M_PI / (par[7] - 1); }

// the radius holding `fraction` of the flux
__device__ inline double fluxfrac(const double *par, double rscale, double fraction)
{
	return rscale * sqrt(pow(1 - fraction, 1 / (1 - par[7])) - 1);
}

__device__ inline double adjust_rscale_switch(const double *par, double rscale)
{
	double rs = fmax(fluxfrac(par, rscale, 0.9999), 1.823 * par[6]);
	return fmax(fmin(rs, 20.), 2.) / rscale;
}

__device__ inline double adjust_rscale_max(const double *par, double rscale)
{
	return ceil(fmax(fluxfrac(par, rscale, 0.9999), 2.) / rscale);
}

__device__ inline double adjust_acc(const double *par, double) { return 0.1 / par[4]; }

__device__ inline double evaluate_at(const double *par, double rscale, double x, double y)
{
	const double box = par[5];
	double r;
	if (box == 0) {
		r = sqrt(x * x + y * y);
	}
	else {
		const double b2 = box + 2;
		r = pow(pow(fabs(x), b2) + pow(fabs(y), b2), 1 / b2);
	}
	const double r_factor = r / rscale;
	return pow(1 + r_factor * r_factor, -par[7]);
}

}  // namespace pf_user
