// Stream-ordered parameter update for fitting loops: copies n_profiles x
// PF_NPAR doubles from device memory into the profiles' parameter slots. The
// next pf_forward recomputes every per-profile constant from them.
#include "pf_device.cuh"

namespace pf {

namespace {

__global__ void set_params_kernel(ProfileDev *profs, int n_profiles, const double *params)
{
	const int t = blockIdx.x * blockDim.x + threadIdx.x;
	if (t >= n_profiles * PF_NPAR) {
		return;
	}
	const int i = t / PF_NPAR, k = t % PF_NPAR;
	profs[i].par[k] = params[t];
}

}  // namespace

void launch_set_params(ProfileDev *profs, int n_profiles, const double *params, cudaStream_t stream)
{
	const int n = n_profiles * PF_NPAR;
	if (n <= 0) return;
	set_params_kernel<<<(n + 255) / 256, 256, 0, stream>>>(profs, n_profiles, params);
}

}  // namespace pf
