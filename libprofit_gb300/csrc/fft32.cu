// FFT convolution of the single-precision batched path (kernels in
// fft32.cuh): the lengths, the twiddle tables, the launches of the first
// group of lengths and the dispatch to the other groups' translation units.
#include "fft32.cuh"

namespace pf {

namespace {

__constant__ int c_sizes[kNumSizes] = {PF_FFT32_SIZES(PF_FFT32_LIST)};

// every length's table: tw[tw_offset(n) + k] = exp(-2 pi i k / n)
__global__ void twiddle32_kernel(float2 *tw)
{
	int k = blockIdx.x * blockDim.x + threadIdx.x;
	if (k >= kTwTotal) return;
	float2 *out = tw + k;
	int n = 0;
	for (int i = 0; i < kNumSizes; i++) {
		n = c_sizes[i];
		if (k < n) break;
		k -= n;
	}
	double s, c;
	sincospi(-2.0 * k / n, &s, &c);
	*out = make_float2((float)c, (float)s);
}

bool fft32_launch_a(int pass, int mode, int n, int n_jobs, const ModelDev *models, const Job *jobs, const float *src,
                    const float *psf, float2 *work, float2 *spec, const float *direct, float *out, const float2 *tw,
                    cudaStream_t stream)
{
	switch (n) {
		PF_FFT32_SIZES_A(PF_FFT32_GROUP_LAUNCH)
	}
	return false;
}

}  // namespace

// Rows per row-pass job and bin columns per column-pass job for transforms of
// n points (0: no transform of that length).
int fft32_rows_per_job(int n)
{
	switch (n) {
#define PF_FFT32_ROWS(N) \
	case N: return 2 * row_ffts<N>();
		PF_FFT32_SIZES(PF_FFT32_ROWS)
	}
	return 0;
}

int fft32_cols_per_job(int n)
{
	switch (n) {
#define PF_FFT32_COLS(N) \
	case N: return col_ffts<N>();
		PF_FFT32_SIZES(PF_FFT32_COLS)
	}
	return 0;
}

// the smallest transform length >= n (0: none)
int fft32_size_at_least(int n)
{
	for (int i = 0; i < kNumSizes; i++)
		if (kSizes[i] >= n) return kSizes[i];
	return 0;
}

int fft32_twiddle_len() { return kTwTotal; }

cudaError_t fft32_configure()
{
	cudaError_t e = cudaSuccess;
	PF_FFT32_SIZES_A(PF_FFT32_GROUP_CONF)
	if (e == cudaSuccess) e = fft32_configure_b();
	if (e == cudaSuccess) e = fft32_configure_c();
	return e;
}

void launch_fft32_twiddles(void *tw, cudaStream_t stream)
{
	twiddle32_kernel<<<(kTwTotal + 255) / 256, 256, 0, stream>>>((float2 *)tw);
}

// pass 0 rows, 1 columns, 2 inverse rows; mode 0 forward, 1 adjoint, 2 PSF
// spectrum (passes 0 and 1 only); n the transform length of the pass (M_x for
// rows, M_y for columns); jobs {model, first, count, 0} of that length.
void launch_fft32(int pass, int mode, int n, const void *jobs, int n_jobs, const ModelDev *models, const float *src,
                  const float *psf, void *work, void *spec, const float *direct, float *out, const void *tw,
                  cudaStream_t stream)
{
	if (n_jobs <= 0) return;
	const Job *j = (const Job *)jobs;
	float2 *w = (float2 *)work, *s = (float2 *)spec;
	const float2 *t = (const float2 *)tw;
	if (fft32_launch_b(pass, mode, n, n_jobs, models, j, src, psf, w, s, direct, out, t, stream)) return;
	if (fft32_launch_c(pass, mode, n, n_jobs, models, j, src, psf, w, s, direct, out, t, stream)) return;
	fft32_launch_a(pass, mode, n, n_jobs, models, j, src, psf, w, s, direct, out, t, stream);
}

}  // namespace pf
