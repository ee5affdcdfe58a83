// FFT convolution of the batched path (FFTConvolver, src/convolve.cpp:233-312,
// restated as a 2-D real convolution).
//
// The reference forms ext = 2 max(src, krn), places the source at (0,0) and
// the kernel at (src - krn)/2, runs a 1-D r2c FFT of the flattened ext image,
// multiplies, inverts and crops at offset_after_convolution; for the output
// pixels that survive Model::evaluate's crop this equals the direct
// convolution conv(d) = sum_k src(d + k - h) rev(k) (zero outside), i.e.
// conv_full(d + size - 1 - h) with conv_full = src * psf. Here, per model:
//   M_x, M_y = powers of two >= crop + psf - 1 (no wrap-around reaches the
//   cropped outputs);
//   pass 1 (rows):    each source row, zero-padded to M_x, complex FFT,
//                     bins 0..M_x/2 kept (Hermitian);
//   pass 2 (columns): each column of bins, zero-padded to M_y, FFT, times the
//                     PSF spectrum, inverse FFT, only the rows the crop needs
//                     kept (in place);
//   pass 3 (rows):    each kept row, Hermitian-completed, inverse FFT, the
//                     crop's columns scaled by 1/(M_x M_y), plus the direct
//                     image, written to the output (SUM-downsampled if asked:
//                     the fine pixels are left in the source buffer and summed
//                     in the reference's order by a last finishing pass).
// The PSF spectrum is made once per batch by passes 1-2 without the product.
// Every transform is a radix-2 Stockham FFT in shared memory (natural-order
// output, ping-pong buffers), several transforms per block when they are
// short; twiddles come from an FP64-computed table.
#include <cstdint>

#include "pf_device.cuh"

namespace pf {

namespace {

template <typename T>
struct Cx;
template <>
struct Cx<float> {
	using t = float2;
};
template <>
struct Cx<double> {
	using t = double2;
};

template <typename C>
__device__ __forceinline__ C cmul(C a, C b)
{
	C r;
	r.x = a.x * b.x - a.y * b.y;
	r.y = a.x * b.y + a.y * b.x;
	return r;
}

template <typename C>
__device__ __forceinline__ C cadd(C a, C b)
{
	C r;
	r.x = a.x + b.x;
	r.y = a.y + b.y;
	return r;
}

template <typename C>
__device__ __forceinline__ C csub(C a, C b)
{
	C r;
	r.x = a.x - b.x;
	r.y = a.y - b.y;
	return r;
}

// cnt transforms of length n (a power of two) held back to back in x; y is
// scratch of the same size. tw[m] = exp(-2 pi i m / nmax), m < nmax / 2.
// Returns the buffer that holds the result.
template <typename C>
__device__ C *stockham(C *x, C *y, int n, int cnt, const C *__restrict__ tw, int nmax, bool inverse)
{
	const int half = n >> 1;
	for (int ns = 1; ns < n; ns <<= 1) {
		const int tws = nmax / (2 * ns);
		for (int idx = threadIdx.x; idx < cnt * half; idx += blockDim.x) {
			const int t = idx / half, j = idx - t * half;
			const C v0 = x[t * n + j];
			C v1 = x[t * n + j + half];
			const int k = j & (ns - 1);
			C w = tw[k * tws];
			if (inverse) w.y = -w.y;
			v1 = cmul(v1, w);
			const int d = ((j - k) << 1) + k;
			y[t * n + d] = cadd(v0, v1);
			y[t * n + d + ns] = csub(v0, v1);
		}
		__syncthreads();
		C *s = x;
		x = y;
		y = s;
	}
	return x;
}

// Jobs: {model, first row or column, count}.
struct FftJob {
	int model, first, count, pad;
};

// pass 1: rows of the source (or of the PSF for the spectrum)
template <typename T>
__global__ void fft_rows_kernel(const ModelDev *__restrict__ models, const FftJob *__restrict__ jobs,
                                const T *__restrict__ src_img, const T *__restrict__ psf,
                                typename Cx<T>::t *__restrict__ work, const typename Cx<T>::t *__restrict__ tw,
                                int nmax, int spectrum)
{
	using C = typename Cx<T>::t;
	extern __shared__ __align__(16) unsigned char smem_raw[];
	C *buf = reinterpret_cast<C *>(smem_raw);
	const FftJob jb = jobs[blockIdx.x];
	const ModelDev &m = models[jb.model];
	const int n = (int)m.fft_mx, nb = n / 2 + 1;
	C *x = buf, *y = buf + jb.count * n;
	const int w = spectrum ? (int)m.psf_w : (int)m.draw_w;
	for (int i = threadIdx.x; i < jb.count * n; i += blockDim.x) {
		const int t = i / n, c = i - t * n, r = jb.first + t;
		C v;
		v.x = 0;
		v.y = 0;
		if (c < w) v.x = spectrum ? psf[m.psf_off + (size_t)r * m.psf_w + c] : src_img[m.draw_off + (size_t)r * m.draw_w + c];
		x[i] = v;
	}
	__syncthreads();
	C *res = stockham(x, y, n, jb.count, tw, nmax, false);
	C *dst = work + (spectrum ? m.fft_spec_off : m.fft_work_off);
	for (int i = threadIdx.x; i < jb.count * nb; i += blockDim.x) {
		const int t = i / nb, c = i - t * nb;
		dst[(size_t)(jb.first + t) * nb + c] = res[t * n + c];
	}
}

// pass 2: columns of bins; forward FFT, then (convolution) product with the
// spectrum, inverse FFT and the kept rows, or (spectrum) the full column
template <typename T>
__global__ void fft_cols_kernel(const ModelDev *__restrict__ models, const FftJob *__restrict__ jobs,
                                typename Cx<T>::t *__restrict__ work, typename Cx<T>::t *__restrict__ spec,
                                const typename Cx<T>::t *__restrict__ tw, int nmax, int spectrum)
{
	using C = typename Cx<T>::t;
	extern __shared__ __align__(16) unsigned char smem_raw[];
	C *buf = reinterpret_cast<C *>(smem_raw);
	const FftJob jb = jobs[blockIdx.x];
	const ModelDev &m = models[jb.model];
	const int n = (int)m.fft_my, nb = (int)m.fft_mx / 2 + 1;
	const int rows_in = spectrum ? (int)m.psf_h : (int)m.draw_h;
	C *x = buf, *y = buf + jb.count * n;
	C *col = (spectrum ? spec + m.fft_spec_off : work + m.fft_work_off);
	// transform t, element r: column jb.first + t, row r (coalesced across t)
	for (int i = threadIdx.x; i < jb.count * n; i += blockDim.x) {
		const int r = i / jb.count, t = i - r * jb.count;
		C v;
		v.x = 0;
		v.y = 0;
		if (r < rows_in) v = col[(size_t)r * nb + jb.first + t];
		x[t * n + r] = v;
	}
	__syncthreads();
	C *res = stockham(x, y, n, jb.count, tw, nmax, false);
	if (spectrum) {
		for (int i = threadIdx.x; i < jb.count * n; i += blockDim.x) {
			const int r = i / jb.count, t = i - r * jb.count;
			col[(size_t)r * nb + jb.first + t] = res[t * n + r];
		}
		return;
	}
	const C *sp = spec + m.fft_spec_off;
	for (int i = threadIdx.x; i < jb.count * n; i += blockDim.x) {
		const int r = i / jb.count, t = i - r * jb.count;
		res[t * n + r] = cmul(res[t * n + r], sp[(size_t)r * nb + jb.first + t]);
	}
	__syncthreads();
	C *other = res == x ? y : x;
	res = stockham(res, other, n, jb.count, tw, nmax, true);
	// the output rows: the crop's, from its offset in the linear convolution;
	// with the uncropped frame, its own rows (zero where the convolution is)
	const int off_y = m.uncropped ? m.ufy0 : (int)m.pad_y + (int)m.psf_h - 1 - (int)m.psf_h / 2;
	const int rows_out = m.uncropped ? (int)m.out_h : (int)m.crop_h;
	const int full_h = (int)m.draw_h + (int)m.psf_h - 1;
	for (int i = threadIdx.x; i < jb.count * rows_out; i += blockDim.x) {
		const int r = i / jb.count, t = i - r * jb.count;
		const int ry = r + off_y;
		C v;
		v.x = 0;
		v.y = 0;
		if (ry >= 0 && ry < full_h && ry < n) v = res[t * n + ry];
		col[(size_t)r * nb + jb.first + t] = v;
	}
}

// pass 3: kept rows, inverse, crop, scale, plus the direct image. A model
// SUM-downsampled: with `fine` given, each fine pixel's value is stored there
// at its drawing position, and the downsampling sums them afterwards in the
// reference's order (finish64_kernel); without, added to its output pixel.
template <typename T>
__global__ void fft_irows_kernel(const ModelDev *__restrict__ models, const FftJob *__restrict__ jobs,
                                 const typename Cx<T>::t *__restrict__ work, const T *__restrict__ direct,
                                 T *__restrict__ out, T *__restrict__ fine, const typename Cx<T>::t *__restrict__ tw,
                                 int nmax)
{
	using C = typename Cx<T>::t;
	extern __shared__ __align__(16) unsigned char smem_raw[];
	C *buf = reinterpret_cast<C *>(smem_raw);
	const FftJob jb = jobs[blockIdx.x];
	const ModelDev &m = models[jb.model];
	const int n = (int)m.fft_mx, nb = n / 2 + 1;
	C *x = buf, *y = buf + jb.count * n;
	const C *src = work + m.fft_work_off;
	for (int i = threadIdx.x; i < jb.count * n; i += blockDim.x) {
		const int t = i / n, c = i - t * n;
		const int r = jb.first + t;
		C v;
		if (c < nb) {
			v = src[(size_t)r * nb + c];
		}
		else {
			v = src[(size_t)r * nb + (n - c)];
			v.y = -v.y;
		}
		x[i] = v;
	}
	__syncthreads();
	C *res = stockham(x, y, n, jb.count, tw, nmax, true);
	const T scale = (T)1 / ((T)m.fft_mx * (T)m.fft_my);
	const int off_x = (int)m.pad_x + (int)m.psf_w - 1 - (int)m.psf_w / 2;
	const bool downsample = m.fs > 1 && !m.return_fs;
	if (m.uncropped) {
		// the uncropped frame (Model::evaluate with crop = false): the linear
		// convolution at (c + ufx0, row), the direct image at drawing pixel
		// (c + udx0, r + udy0); the convolution masked by the calculation mask
		// extended over the frame (mask_and_crop, src/convolve.cpp:81-94)
		const int full_w = (int)m.draw_w + (int)m.psf_w - 1;
		for (int i = threadIdx.x; i < jb.count * (int)m.out_w; i += blockDim.x) {
			const int t = i / m.out_w, c = i - t * m.out_w;
			const int r = jb.first + t;
			const int fx = c + m.ufx0, dxp = c + m.udx0, dyp = r + m.udy0;
			const bool in_draw = dxp >= 0 && dyp >= 0 && dxp < (int)m.draw_w && dyp < (int)m.draw_h;
			T conv = fx >= 0 && fx < full_w && fx < n ? res[t * n + fx].x * scale : (T)0;
			if (m.mask_eval && !(in_draw && evaluated(m, dxp, dyp))) conv = (T)0;
			const T dir = in_draw && m.direct_required ? direct[m.draw_off + (size_t)dyp * m.draw_w + dxp] : (T)0;
			out[m.out_off + (size_t)r * m.out_w + c] = dir + conv;
		}
		return;
	}
	for (int i = threadIdx.x; i < jb.count * (int)m.crop_w; i += blockDim.x) {
		const int t = i / m.crop_w, c = i - t * m.crop_w;
		const int r = jb.first + t;
		// the convolution zero where the calculation mask is; the model's mask at the end
		const T conv = evaluated(m, c + (int)m.pad_x, r + (int)m.pad_y) ? res[t * n + c + off_x].x * scale : (T)0;
		const T dir = m.direct_required ? direct[m.draw_off + (size_t)(r + m.pad_y) * m.draw_w + c + m.pad_x] : (T)0;
		const T v = dir + conv;
		if (downsample && fine) {
			fine[m.draw_off + (size_t)(r + m.pad_y) * m.draw_w + c + m.pad_x] = v;
		}
		else if (downsample) {
			if (kept(m, c / (int)m.fs, r / (int)m.fs)) atomicAdd(&out[m.out_off + (size_t)(r / m.fs) * m.out_w + c / m.fs], v);
		}
		else out[m.out_off + (size_t)r * m.out_w + c] = kept(m, c, r) ? v : (T)0;
	}
}

template <typename C>
__global__ void twiddle_kernel(C *tw, int nmax)
{
	const int k = blockIdx.x * blockDim.x + threadIdx.x;
	if (k >= nmax / 2) return;
	double s, c;
	sincospi(-2.0 * k / nmax, &s, &c);
	tw[k].x = c;
	tw[k].y = s;
}

}  // namespace

int fft_job_size() { return (int)sizeof(FftJob); }

template <typename T>
size_t fft_smem(int n, int count)
{
	return 2 * sizeof(typename Cx<T>::t) * (size_t)n * count;
}

template <typename T>
cudaError_t fft_configure(size_t smem)
{
	cudaError_t e = cudaFuncSetAttribute(fft_rows_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
	if (e == cudaSuccess)
		e = cudaFuncSetAttribute(fft_cols_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
	if (e == cudaSuccess)
		e = cudaFuncSetAttribute(fft_irows_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
	return e;
}

template <typename T>
void launch_twiddles(void *tw, int nmax, cudaStream_t stream)
{
	twiddle_kernel<<<(nmax / 2 + 255) / 256, 256, 0, stream>>>((typename Cx<T>::t *)tw, nmax);
}

// pass: 0 rows (source), 1 columns (convolution), 2 inverse rows, 3 rows (PSF
// spectrum), 4 columns (PSF spectrum)
template <typename T>
void launch_fft_pass(int pass, const ModelDev *models, const void *jobs, int n_jobs, const T *src, const T *psf,
                     void *work, void *spec, const T *direct, T *out, T *fine, const void *tw, int nmax, size_t smem,
                     cudaStream_t stream)
{
	using C = typename Cx<T>::t;
	if (n_jobs <= 0) return;
	const FftJob *j = (const FftJob *)jobs;
	const int threads = 256;
	switch (pass) {
	case 0:
		fft_rows_kernel<T><<<n_jobs, threads, smem, stream>>>(models, j, src, psf, (C *)work, (const C *)tw, nmax, 0);
		break;
	case 1:
		fft_cols_kernel<T><<<n_jobs, threads, smem, stream>>>(models, j, (C *)work, (C *)spec, (const C *)tw, nmax, 0);
		break;
	case 2:
		fft_irows_kernel<T><<<n_jobs, threads, smem, stream>>>(models, j, (const C *)work, direct, out, fine,
		                                                        (const C *)tw, nmax);
		break;
	case 3:
		fft_rows_kernel<T><<<n_jobs, threads, smem, stream>>>(models, j, src, psf, (C *)spec, (const C *)tw, nmax, 1);
		break;
	case 4:
		fft_cols_kernel<T><<<n_jobs, threads, smem, stream>>>(models, j, (C *)work, (C *)spec, (const C *)tw, nmax, 1);
		break;
	}
}

template size_t fft_smem<float>(int, int);
template size_t fft_smem<double>(int, int);
template cudaError_t fft_configure<float>(size_t);
template cudaError_t fft_configure<double>(size_t);
template void launch_twiddles<float>(void *, int, cudaStream_t);
template void launch_twiddles<double>(void *, int, cudaStream_t);
template void launch_fft_pass<float>(int, const ModelDev *, const void *, int, const float *, const float *, void *,
                                     void *, const float *, float *, float *, const void *, int, size_t,
                                     cudaStream_t);
template void launch_fft_pass<double>(int, const ModelDev *, const void *, int, const double *, const double *,
                                      void *, void *, const double *, double *, double *, const void *, int, size_t,
                                      cudaStream_t);

}  // namespace pf
