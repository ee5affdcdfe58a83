// A user-defined radial profile compiled into the library: the CUDA
// counterpart of adding a RadialProfile subclass to libprofit
// (docs/new_profile.rst; include/profit/radial.h:104-174 lists the methods
// such a class implements). Built with
//     python libprofit_gb300/build.py --user-profile <file>
// the file's profile is kind PF_USER under its own name; without one, PF_USER
// is refused. libprofit_gb300/user_profiles/example_moffat.cuh documents what
// the file defines and gives an example.
#pragma once

#ifdef PF_USER_PROFILE_FILE
#include PF_USER_PROFILE_FILE
#endif

namespace pf {
namespace user {

#ifdef PF_USER_PROFILE_FILE
constexpr bool available = true;
constexpr int n_params = pf_user::n_params;
static_assert(n_params >= 0 && n_params <= 6, "a user profile has at most 6 parameters after the radial ones");
inline const char *name() { return pf_user::name; }
inline const char *const *param_names() { return pf_user::param_names; }
inline const double *param_defaults() { return pf_user::param_defaults; }
inline const char *message(int k) { return pf_user::messages[k]; }
__host__ __device__ inline int validate(const double *par) { return pf_user::validate(par); }
__device__ inline double get_rscale(const double *par) { return pf_user::get_rscale(par); }
__device__ inline double get_lumtot(const double *par, double rscale) { return pf_user::get_lumtot(par, rscale); }
__device__ inline double adjust_rscale_switch(const double *par, double rscale)
{
	return pf_user::adjust_rscale_switch(par, rscale);
}
__device__ inline double adjust_rscale_max(const double *par, double rscale)
{
	return pf_user::adjust_rscale_max(par, rscale);
}
__device__ inline double adjust_acc(const double *par, double acc) { return pf_user::adjust_acc(par, acc); }
__device__ inline double evaluate_at(const double *par, double rscale, double x, double y)
{
	return pf_user::evaluate_at(par, rscale, x, y);
}
#else
constexpr bool available = false;
constexpr int n_params = 0;
inline const char *name() { return ""; }
inline const char *const *param_names() { return nullptr; }
inline const double *param_defaults() { return nullptr; }
inline const char *message(int) { return ""; }
__host__ __device__ inline int validate(const double *) { return 0; }
__device__ inline double get_rscale(const double *) { return 0; }
__device__ inline double get_lumtot(const double *, double) { return 0; }
__device__ inline double adjust_rscale_switch(const double *, double) { return 1; }
__device__ inline double adjust_rscale_max(const double *, double) { return 0; }
__device__ inline double adjust_acc(const double *, double acc) { return acc; }
__device__ inline double evaluate_at(const double *, double, double, double) { return 0; }
#endif

}  // namespace user
}  // namespace pf
