// Per-model total flux of the rendered images (Image::total,
// src/image.cpp:204-206), summed in FP64 with a fixed-shape block reduction
// so that repeated runs give identical bits.
#include <cstdint>

#include "pf_device.cuh"

namespace pf {

namespace {

template <typename T>
__global__ void flux_sum_kernel(const ModelDev *__restrict__ models, const T *__restrict__ images,
                                double *__restrict__ flux)
{
	const ModelDev &m = models[blockIdx.x];
	const long long n = (long long)m.out_w * m.out_h;
	const T *img = images + m.out_off;
	double s = 0;
	for (long long i = threadIdx.x; i < n; i += blockDim.x) {
		s += (double)img[i];
	}
	__shared__ double part[256];
	part[threadIdx.x] = s;
	__syncthreads();
	for (int w = blockDim.x / 2; w > 0; w >>= 1) {
		if ((int)threadIdx.x < w) part[threadIdx.x] += part[threadIdx.x + w];
		__syncthreads();
	}
	if (threadIdx.x == 0) flux[blockIdx.x] = part[0];
}

}  // namespace

void launch_flux_sum(const ModelDev *models, int n_models, const void *images, int is_double, double *flux,
                     cudaStream_t stream)
{
	if (n_models <= 0) return;
	if (is_double) flux_sum_kernel<double><<<n_models, 256, 0, stream>>>(models, (const double *)images, flux);
	else flux_sum_kernel<float><<<n_models, 256, 0, stream>>>(models, (const float *)images, flux);
}

}  // namespace pf
