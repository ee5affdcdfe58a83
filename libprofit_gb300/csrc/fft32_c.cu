// The single-precision FFT kernels of the transform lengths of group C
// (PF_FFT32_SIZES_C in fft32.cuh), in a translation unit of their own.
#include "fft32.cuh"

namespace pf {

cudaError_t fft32_configure_c()
{
	cudaError_t e = cudaSuccess;
	PF_FFT32_SIZES_C(PF_FFT32_GROUP_CONF)
	return e;
}

bool fft32_launch_c(int pass, int mode, int n, int n_jobs, const ModelDev *models, const Job *jobs, const float *src,
                    const float *psf, float2 *work, float2 *spec, const float *direct, float *out, const float2 *tw,
                    cudaStream_t stream)
{
	switch (n) {
		PF_FFT32_SIZES_C(PF_FFT32_GROUP_LAUNCH)
	}
	return false;
}

}  // namespace pf
