// FFT convolution of the single-precision batched path: forward (the
// reference's FFTConvolver, src/convolve.cpp:233-312, restated as a 2-D real
// convolution) and its adjoint (the cotangent correlated with the PSF).
//
// Per model, with M_x, M_y the smallest supported lengths >= crop + psf (no
// wrap-around reaches a kept output; lengths 2^a and 3, 5, 9 x 2^a):
//   forward  out  = crop(IFFT(FFT(src) * S)) / (M_x M_y) + direct
//   adjoint  gsrc = drawing(IFFT(FFT(embed(gout)) * conj(S))) / (M_x M_y)
// where S is the PSF's spectrum (made once per batch) and embed places the
// cotangent where the forward crop takes its outputs. Three passes:
//   rows    two real rows per complex transform (z = a + i b), bins 0..M_x/2
//           of both unpacked from Z(k) and conj(Z(M_x - k));
//   columns 16 bin columns per block (fewer when long), forward transform,
//           product with the spectrum, inverse transform, the kept rows back
//           in place;
//   rows    two Hermitian rows per inverse transform (Z = A + i B), the real
//           and imaginary parts the two output rows.
// Transforms: Stockham autosort stages in shared memory (formulation of
// Govindaraju et al., "High performance discrete Fourier transforms on
// graphics processors", SC 2008): the odd factor first (radix 3, 5 or two
// radix-3 stages), then radix 8 with a radix-4 or -2 stage last; N / 8
// threads per transform, each taking its butterflies of a stage in registers.
// Twiddles from per-length tables of exp(-2 pi i k / N) computed in FP64.
// Shared-memory element i of a transform sits at i + i / 8, so the stride-8
// stores of the first stages hit distinct banks.
#pragma once
#include <cstdint>

#include "pf_device.cuh"

namespace pf {

// one job of a pass: transforms of model `model` starting at row or bin column `first`
struct Job {
	int model, first, count, pad;
};

namespace {

// The transform lengths: 2^a (64 .. 8192) and 3, 5, 9 x 2^a (2^a >= 32, up to
// 6144, 5120, 4608), ascending.
// The kernels of each group are instantiated in a translation unit of their
// own (fft32.cu, fft32_b.cu, fft32_c.cu), compiled in parallel.
#define PF_FFT32_SIZES_A(X) X(64) X(96) X(128) X(160) X(192) X(256) X(288) X(320) X(384)
#define PF_FFT32_SIZES_B(X) X(512) X(576) X(640) X(768) X(1024) X(1152) X(1280) X(1536)
#define PF_FFT32_SIZES_C(X) X(2048) X(2304) X(2560) X(3072) X(4096) X(4608) X(5120) X(6144) X(8192)
#define PF_FFT32_SIZES(X) PF_FFT32_SIZES_A(X) PF_FFT32_SIZES_B(X) PF_FFT32_SIZES_C(X)
#define PF_FFT32_LIST(n) n,
constexpr int kSizes[] = {PF_FFT32_SIZES(PF_FFT32_LIST)};
constexpr int kNumSizes = sizeof(kSizes) / sizeof(kSizes[0]);

// offset of length n's twiddle table (exp(-2 pi i k / n), k < n) in the
// concatenated tables; kTwTotal, their total length
__host__ __device__ constexpr int tw_offset(int n)
{
	int o = 0;
	for (int i = 0; i < kNumSizes && kSizes[i] != n; i++) o += kSizes[i];
	return o;
}
constexpr int kTwTotal = tw_offset(-1);

// the odd factor of a transform length: 1, 3, 5 or 9
__host__ __device__ constexpr int odd_part(int n) { return n % 9 == 0 ? 9 : n % 5 == 0 ? 5 : n % 3 == 0 ? 3 : 1; }

enum { F_FORWARD = 0, F_ADJOINT = 1, F_SPECTRUM = 2 };

__device__ __forceinline__ float2 cmulf(float2 a, float2 b)
{
	return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ float2 caddf(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 csubf(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
// a * (-i) (forward) or a * (+i) (inverse)
template <bool INV>
__device__ __forceinline__ float2 rot90(float2 a)
{
	return INV ? make_float2(-a.y, a.x) : make_float2(a.y, -a.x);
}

__device__ __forceinline__ int pidx(int i) { return i + (i >> 3); }

template <bool INV>
__device__ __forceinline__ float2 twiddle(const float2 *__restrict__ table, int k)  // table[k], conjugated inverse
{
	float2 w = __ldg(table + k);
	if (INV) w.y = -w.y;
	return w;
}

template <bool INV>
__device__ __forceinline__ void dft2(float2 *v)
{
	const float2 a = v[0], b = v[1];
	v[0] = caddf(a, b);
	v[1] = csubf(a, b);
}

template <bool INV>
__device__ __forceinline__ void dft4(float2 *v)
{
	const float2 p0 = caddf(v[0], v[2]), p1 = csubf(v[0], v[2]);
	const float2 p2 = caddf(v[1], v[3]), p3 = rot90<INV>(csubf(v[1], v[3]));
	v[0] = caddf(p0, p2);
	v[2] = csubf(p0, p2);
	v[1] = caddf(p1, p3);
	v[3] = csubf(p1, p3);
}

// 3-point DFT: X1, X2 = x0 - (x1 + x2) / 2 -+ i sin(2 pi / 3) (x1 - x2) (forward)
template <bool INV>
__device__ __forceinline__ void dft3(float2 *v)
{
	constexpr float s3 = 0.86602540378443865f;  // sin(2 pi / 3)
	const float2 t1 = caddf(v[1], v[2]);
	const float2 t2 = make_float2(v[0].x - 0.5f * t1.x, v[0].y - 0.5f * t1.y);
	const float2 t3 = rot90<INV>(make_float2(s3 * (v[1].x - v[2].x), s3 * (v[1].y - v[2].y)));
	v[0] = caddf(v[0], t1);
	v[1] = caddf(t2, t3);
	v[2] = csubf(t2, t3);
}

// 5-point DFT: with a1 = x1 + x4, a2 = x2 + x3, b1 = x1 - x4, b2 = x2 - x3,
// X1, X4 = x0 + c1 a1 + c2 a2 -+ i (s1 b1 + s2 b2) and X2, X3 = x0 + c2 a1 +
// c1 a2 -+ i (s2 b1 - s1 b2) (forward), c_k = cos(2 pi k / 5), s_k = sin(2 pi k / 5)
template <bool INV>
__device__ __forceinline__ void dft5(float2 *v)
{
	constexpr float c1 = 0.30901699437494742f, c2 = -0.80901699437494742f;
	constexpr float s1 = 0.95105651629515357f, s2 = 0.58778525229247313f;
	const float2 x0 = v[0];
	const float2 a1 = caddf(v[1], v[4]), a2 = caddf(v[2], v[3]);
	const float2 b1 = csubf(v[1], v[4]), b2 = csubf(v[2], v[3]);
	const float2 t1 = make_float2(x0.x + c1 * a1.x + c2 * a2.x, x0.y + c1 * a1.y + c2 * a2.y);
	const float2 t2 = make_float2(x0.x + c2 * a1.x + c1 * a2.x, x0.y + c2 * a1.y + c1 * a2.y);
	const float2 u1 = rot90<INV>(make_float2(s1 * b1.x + s2 * b2.x, s1 * b1.y + s2 * b2.y));
	const float2 u2 = rot90<INV>(make_float2(s2 * b1.x - s1 * b2.x, s2 * b1.y - s1 * b2.y));
	v[0] = caddf(x0, caddf(a1, a2));
	v[1] = caddf(t1, u1);
	v[4] = csubf(t1, u1);
	v[2] = caddf(t2, u2);
	v[3] = csubf(t2, u2);
}

// 8-point DFT, natural order in and out (decimation in frequency)
template <bool INV>
__device__ __forceinline__ void dft8(float2 *v)
{
	constexpr float h = 0.70710678118654752f;
	float2 u[4], w[4];
#pragma unroll
	for (int n = 0; n < 4; n++) {
		u[n] = caddf(v[n], v[n + 4]);
		w[n] = csubf(v[n], v[n + 4]);
	}
	// w[n] *= exp(-+ 2 pi i n / 8)
	w[1] = INV ? make_float2(h * (w[1].x - w[1].y), h * (w[1].x + w[1].y))
	           : make_float2(h * (w[1].x + w[1].y), h * (w[1].y - w[1].x));
	w[2] = rot90<INV>(w[2]);
	w[3] = INV ? make_float2(-h * (w[3].x + w[3].y), h * (w[3].x - w[3].y))
	           : make_float2(h * (w[3].y - w[3].x), -h * (w[3].x + w[3].y));
	dft4<INV>(u);
	dft4<INV>(w);
#pragma unroll
	for (int k = 0; k < 4; k++) {
		v[2 * k] = u[k];
		v[2 * k + 1] = w[k];
	}
}

template <int R, bool INV>
__device__ __forceinline__ void dft(float2 *v)
{
	if constexpr (R == 8) dft8<INV>(v);
	else if constexpr (R == 5) dft5<INV>(v);
	else if constexpr (R == 4) dft4<INV>(v);
	else if constexpr (R == 3) dft3<INV>(v);
	else dft2<INV>(v);
}

// One radix-R Stockham stage over the N points of buf (padded layout) after
// stages whose radices multiply to NS, by thread t < N / 8 of the transform:
// butterfly j (of N / R) takes points j + r N / R, twiddled by
// exp(-+2 pi i (j mod NS) r / (NS R)), and writes its outputs to
// (j - j mod NS) R + j mod NS + r NS. All threads of the block take part.
template <int N, int R, int NS, bool INV>
__device__ __forceinline__ void stage(float2 *buf, int t, const float2 *__restrict__ table)
{
	constexpr int T = N / 8, NB = N / R;  // threads, butterflies
	constexpr int G = (NB + T - 1) / T;   // butterflies per thread
	constexpr bool ragged = NB % T != 0;  // radix 3 and 5: the last ones on some threads only
	float2 v[G * R];
#pragma unroll
	for (int q = 0; q < G; q++) {
		const int j = t + q * T;
		if (!ragged || j < NB) {
#pragma unroll
			for (int r = 0; r < R; r++) v[q * R + r] = buf[pidx(j + r * NB)];
		}
	}
	__syncthreads();
#pragma unroll
	for (int q = 0; q < G; q++) {
		const int j = t + q * T;
		if (ragged && j >= NB) continue;
		const int jm = j % NS;
		if constexpr (NS > 1) {
#pragma unroll
			for (int r = 1; r < R; r++)
				v[q * R + r] = cmulf(v[q * R + r], twiddle<INV>(table, tw_offset(N) + jm * r * (N / (NS * R))));
		}
		dft<R, INV>(v + q * R);
		const int base = (j - jm) * R + jm;
#pragma unroll
		for (int r = 0; r < R; r++) buf[pidx(base + r * NS)] = v[q * R + r];
	}
	__syncthreads();
}

// the power-of-two stages after the odd factor's (NS = their product so far)
template <int N, int NS, bool INV>
__device__ __forceinline__ void pow2_stages(float2 *buf, int t, const float2 *__restrict__ table)
{
	constexpr int rem = N / NS;
	if constexpr (rem >= 8) {
		stage<N, 8, NS, INV>(buf, t, table);
		pow2_stages<N, NS * 8, INV>(buf, t, table);
	}
	else if constexpr (rem == 4) stage<N, 4, NS, INV>(buf, t, table);
	else if constexpr (rem == 2) stage<N, 2, NS, INV>(buf, t, table);
}

// In-place FFT of the N points of buf (natural order in and out).
template <int N, bool INV>
__device__ __forceinline__ void fft(float2 *buf, int t, const float2 *__restrict__ table)
{
	constexpr int F = odd_part(N);
	static_assert(N % 8 == 0 && (N / F) >= 32 && ((N / F) & (N / F - 1)) == 0, "lengths 2^a, 3, 5, 9 x 2^a");
	if constexpr (F == 3) stage<N, 3, 1, INV>(buf, t, table);
	if constexpr (F == 5) stage<N, 5, 1, INV>(buf, t, table);
	if constexpr (F == 9) {
		stage<N, 3, 1, INV>(buf, t, table);
		stage<N, 3, 3, INV>(buf, t, table);
	}
	pow2_stages<N, F, INV>(buf, t, table);
}

template <int N>
__host__ __device__ constexpr int row_ffts() { return (N / 8) >= 256 ? 1 : 256 / (N / 8); }  // transforms per row block
// Column-pass blocks: at most PF_FFT_COL_THREADS threads (16 transforms at
// most), PF_FFT_COL_MINB blocks per SM for the launch bounds when they have
// at most 576 threads.
#ifndef PF_FFT_COL_THREADS
#define PF_FFT_COL_THREADS 288
#endif
#ifndef PF_FFT_COL_MINB
#define PF_FFT_COL_MINB 2
#endif
// Lengths whose column pass runs as warp transforms (cols_w_kernel): N = 32 P
// with P points per lane, P one of the register DFTs' sizes.
template <int N>
__host__ __device__ constexpr bool warp_cols()
{
	return N == 64 || N == 96 || N == 128 || N == 160 || N == 256 || N == 288 || N == 512;
}

template <int N>
__host__ __device__ constexpr int col_ffts()
{
	if (warp_cols<N>()) return 8;  // one warp per bin column, 8 per block
	return PF_FFT_COL_THREADS / (N / 8) < 1 ? 1 : PF_FFT_COL_THREADS / (N / 8) > 16 ? 16 : PF_FFT_COL_THREADS / (N / 8);
}
template <int N>
__host__ __device__ constexpr int row_stride() { return N + N / 8; }                     // padded length
template <int N>
__host__ __device__ constexpr int col_stride() { return N + N / 8 + 1; }                 // = 1 or 9 mod 16: columns on distinct banks


// cotangent of crop pixel (cx, cy) (SUM-downsampling aware; zero where the
// calculation mask zeroed the forward convolution)
__device__ __forceinline__ float cot_crop(const ModelDev &m, const float *gout, int cx, int cy)
{
	if (!evaluated(m, cx + (int)m.pad_x, cy + (int)m.pad_y)) return 0.f;
	if (m.fs > 1 && !m.return_fs) return gout[m.out_off + (size_t)(cy / m.fs) * m.out_w + cx / m.fs];
	return gout[m.out_off + (size_t)cy * m.out_w + cx];
}

// Pass 1: rows. Job rows first .. first + count - 1 (of the source image,
// the cotangent or the PSF), two per transform; bins 0..N/2 to dst rows.
template <int N, int MODE>
__global__ void __launch_bounds__(row_ffts<N>() * (N / 8))
rows_kernel(const ModelDev *__restrict__ models, const Job *__restrict__ jobs, const float *__restrict__ src,
            const float *__restrict__ psf, float2 *__restrict__ work, float2 *__restrict__ spec,
            const float2 *__restrict__ table)
{
	constexpr int F = row_ffts<N>(), PS = row_stride<N>(), NB = N / 2 + 1;
	extern __shared__ float2 fsm[];
	float2 *buf = fsm;
	const Job jb = jobs[blockIdx.x];
	const ModelDev &m = models[jb.model];
	const int f = threadIdx.x / (N / 8), t = threadIdx.x % (N / 8);
	// source columns and their offset in the transform
	int w, xoff = 0;
	if (MODE == F_FORWARD) w = (int)m.draw_w;
	else if (MODE == F_ADJOINT) {
		w = (int)m.crop_w;
		xoff = (int)m.pad_x + (int)m.psf_w - 1 - (int)m.psf_w / 2;
	}
	else w = (int)m.psf_w;
	// the block has F * N / 8 threads: eight points each, all loads issued
	// before the shared-memory stores
	float2 v[8];
#pragma unroll
	for (int q = 0; q < 8; q++) {
		const int i = (int)threadIdx.x + q * (F * (N / 8));
		const int ff = i / N, c = i % N;
		const int r0 = jb.first + 2 * ff, r1 = r0 + 1;
		const int x = c - xoff;
		v[q] = make_float2(0.f, 0.f);
		if (x >= 0 && x < w) {
			if (MODE == F_FORWARD) {
				const float *s = src + m.draw_off;
				if (r0 < jb.first + jb.count) v[q].x = s[(size_t)r0 * m.draw_w + x];
				if (r1 < jb.first + jb.count) v[q].y = s[(size_t)r1 * m.draw_w + x];
			}
			else if (MODE == F_ADJOINT) {
				if (r0 < jb.first + jb.count) v[q].x = cot_crop(m, src, x, r0);
				if (r1 < jb.first + jb.count) v[q].y = cot_crop(m, src, x, r1);
			}
			else {
				const float *k = psf + m.psf_off;
				if (r0 < jb.first + jb.count) v[q].x = k[(size_t)r0 * m.psf_w + x];
				if (r1 < jb.first + jb.count) v[q].y = k[(size_t)r1 * m.psf_w + x];
			}
		}
	}
#pragma unroll
	for (int q = 0; q < 8; q++) {
		const int i = (int)threadIdx.x + q * (F * (N / 8));
		buf[(i / N) * PS + pidx(i % N)] = v[q];
	}
	__syncthreads();
	fft<N, false>(buf + f * PS, t, table);
	// unpack: A(k) = (Z(k) + conj Z(N-k)) / 2, B(k) = (Z(k) - conj Z(N-k)) / (2 i)
	float2 *dst = work + m.fft_work_off;  // the PSF's row spectra too: the column pass writes the spectrum
	const int nbr = (int)m.fft_mx / 2 + 1;  // = NB
	for (int i = threadIdx.x; i < F * NB; i += blockDim.x) {
		const int ff = i / NB, k = i % NB;
		const int r0 = jb.first + 2 * ff;
		const float2 z = buf[ff * PS + pidx(k)], zm = buf[ff * PS + pidx(k == 0 ? 0 : N - k)];
		if (r0 < jb.first + jb.count) dst[(size_t)r0 * nbr + k] = make_float2(0.5f * (z.x + zm.x), 0.5f * (z.y - zm.y));
		if (r0 + 1 < jb.first + jb.count) dst[(size_t)(r0 + 1) * nbr + k] = make_float2(0.5f * (z.y + zm.y), 0.5f * (zm.x - z.x));
	}
}

// Pass 2: columns of bins. Job: bin columns first .. first + count - 1.
template <int N>
__host__ __device__ constexpr int col_min_blocks() { return col_ffts<N>() * (N / 8) <= 576 ? PF_FFT_COL_MINB : 1; }

template <int N, int MODE>
__global__ void __launch_bounds__(col_ffts<N>() * (N / 8), col_min_blocks<N>())
cols_kernel(const ModelDev *__restrict__ models, const Job *__restrict__ jobs, float2 *__restrict__ work,
            float2 *__restrict__ spec, const float2 *__restrict__ table)
{
	constexpr int F = col_ffts<N>(), PS = col_stride<N>();
	extern __shared__ float2 fsm[];
	float2 *cbuf = fsm;
	const Job jb = jobs[blockIdx.x];
	const ModelDev &m = models[jb.model];
	const int nb = (int)m.fft_mx / 2 + 1;
	const int f = threadIdx.x / (N / 8), t = threadIdx.x % (N / 8);
	float2 *col = work + m.fft_work_off;
	// rows present in the input and their place in the transform
	int rows_in, yoff = 0;
	if (MODE == F_FORWARD) rows_in = (int)m.draw_h;
	else if (MODE == F_ADJOINT) {
		rows_in = (int)m.crop_h;
		yoff = (int)m.pad_y + (int)m.psf_h - 1 - (int)m.psf_h / 2;
	}
	else rows_in = (int)m.psf_h;
	// the block has F * N / 8 threads: eight points each, all loads issued
	// before the shared-memory stores
	float2 v[8];
#pragma unroll
	for (int q = 0; q < 8; q++) {
		const int i = (int)threadIdx.x + q * (F * (N / 8));
		const int rg = i / F, ff = i % F;  // transform row, column within the job
		const int r = rg - yoff;
		v[q] = make_float2(0.f, 0.f);
		if (ff < jb.count && r >= 0 && r < rows_in) v[q] = col[(size_t)r * nb + jb.first + ff];
	}
#pragma unroll
	for (int q = 0; q < 8; q++) {
		const int i = (int)threadIdx.x + q * (F * (N / 8));
		cbuf[(i % F) * PS + pidx(i / F)] = v[q];
	}
	__syncthreads();
	fft<N, false>(cbuf + f * PS, t, table);
	if (MODE == F_SPECTRUM) {
		float2 *sp_out = spec + m.fft_spec_off;
		for (int i = threadIdx.x; i < F * N; i += blockDim.x) {
			const int rg = i / F, ff = i % F;
			if (ff < jb.count) sp_out[(size_t)rg * nb + jb.first + ff] = cbuf[ff * PS + pidx(rg)];
		}
		return;
	}
	const float2 *sp = spec + m.fft_spec_off;
#pragma unroll
	for (int q = 0; q < 8; q++) {
		const int i = (int)threadIdx.x + q * (F * (N / 8));
		const int rg = i / F, ff = i % F;
		v[q] = ff < jb.count ? sp[(size_t)rg * nb + jb.first + ff] : make_float2(0.f, 0.f);
	}
#pragma unroll
	for (int q = 0; q < 8; q++) {
		const int i = (int)threadIdx.x + q * (F * (N / 8));
		const int rg = i / F, ff = i % F;
		if (ff >= jb.count) continue;
		float2 sq = v[q];
		if (MODE == F_ADJOINT) sq.y = -sq.y;
		cbuf[ff * PS + pidx(rg)] = cmulf(cbuf[ff * PS + pidx(rg)], sq);
	}
	__syncthreads();
	fft<N, true>(cbuf + f * PS, t, table);
	// kept rows: forward, the crop's (from its offset); adjoint, the drawing area's
	const int rows_out = MODE == F_FORWARD ? (int)m.crop_h : (int)m.draw_h;
	const int keep = MODE == F_FORWARD ? (int)m.pad_y + (int)m.psf_h - 1 - (int)m.psf_h / 2 : 0;
#pragma unroll 4
	for (int i = threadIdx.x; i < F * rows_out; i += blockDim.x) {
		const int r = i / F, ff = i % F;
		if (ff < jb.count) col[(size_t)r * nb + jb.first + ff] = cbuf[ff * PS + pidx(r + keep)];
	}
}

// ---- the column pass as warp transforms (lengths N = 32 P, warp_cols<N>())
//
// One warp per bin column, lane l holding points l + 32 p (p < P). With
// n = 32 n1 + n2 and k = k1 + P k2 (Cooley-Tukey, N = P x 32):
//   forward  a P-point DFT in registers over n1, the twiddle W_N^(l k1), and
//            a 32-point decimation-in-frequency DFT across the lanes (shuffles),
//            which leaves X[k1 + P bitrev5(l)] in lane l's k1-th register;
//   product  with the PSF spectrum stored in that same order (the spectrum pass
//            runs the same forward transform), so no permutation is needed;
//   inverse  the lane network undone stage by stage, the conjugate twiddle and
//            the inverse register DFT: back to natural order, unnormalised.

// exp(-2 pi i m / P) (forward; conjugated for the inverse) for the register
// DFTs of 9 and 16 points, m < 10
template <int P, bool INV>
__device__ __forceinline__ float2 small_twiddle(int m)
{
	constexpr float c9[5] = {1.f, 0.76604444311897804f, 0.17364817766693035f, -0.5f, -0.93969262078590838f};
	constexpr float s9[5] = {0.f, 0.64278760968653933f, 0.98480775301220802f, 0.86602540378443865f,
	                         0.34202014332566873f};
	constexpr float c16[10] = {1.f, 0.92387953251128674f, 0.70710678118654752f, 0.38268343236508978f, 0.f,
	                           -0.38268343236508978f, -0.70710678118654752f, -0.92387953251128674f, -1.f,
	                           -0.92387953251128674f};
	constexpr float s16[10] = {0.f, 0.38268343236508978f, 0.70710678118654752f, 0.92387953251128674f, 1.f,
	                           0.92387953251128674f, 0.70710678118654752f, 0.38268343236508978f, 0.f,
	                           -0.38268343236508978f};
	const float c = P == 9 ? c9[m] : c16[m], sn = P == 9 ? s9[m] : s16[m];
	return make_float2(c, INV ? sn : -sn);
}

// A B-point DFT in registers, natural order in and out (Cooley-Tukey A x B):
// A-point DFTs of the stride-B subsequences, twiddles W_(AB)^(n2 k1), B-point
// DFTs across them.
template <int A, int B, bool INV>
__device__ __forceinline__ void dft_ct(float2 *v)
{
	constexpr int P = A * B;
	float2 y[P];
#pragma unroll
	for (int n2 = 0; n2 < B; n2++) {
		float2 t[A];
#pragma unroll
		for (int n1 = 0; n1 < A; n1++) t[n1] = v[B * n1 + n2];
		dft<A, INV>(t);
#pragma unroll
		for (int k1 = 0; k1 < A; k1++) y[n2 * A + k1] = n2 * k1 ? cmulf(t[k1], small_twiddle<P, INV>(n2 * k1)) : t[k1];
	}
#pragma unroll
	for (int k1 = 0; k1 < A; k1++) {
		float2 t[B];
#pragma unroll
		for (int n2 = 0; n2 < B; n2++) t[n2] = y[n2 * A + k1];
		dft<B, INV>(t);
#pragma unroll
		for (int k2 = 0; k2 < B; k2++) v[k1 + A * k2] = t[k2];
	}
}

template <int P, bool INV>
__device__ __forceinline__ void dft_reg(float2 *v)
{
	if constexpr (P == 9) dft_ct<3, 3, INV>(v);
	else if constexpr (P == 16) dft_ct<4, 4, INV>(v);
	else dft<P, INV>(v);
}

__device__ __forceinline__ float2 shfl_xor2(float2 v, int m)
{
	return make_float2(__shfl_xor_sync(0xffffffffu, v.x, m), __shfl_xor_sync(0xffffffffu, v.y, m));
}

// forward: v[p] = x[lane + 32 p] in, X[k1 + P bitrev5(lane)] in v[k1] out
template <int N>
__device__ __forceinline__ void warp_fft_forward(float2 (&v)[N / 32], int lane, const float2 *__restrict__ table)
{
	constexpr int P = N / 32;
	dft_reg<P, false>(v);
#pragma unroll
	for (int k1 = 1; k1 < P; k1++) v[k1] = cmulf(v[k1], twiddle<false>(table, tw_offset(N) + lane * k1));
#pragma unroll
	for (int h = 16; h >= 1; h >>= 1) {
		const bool upper = lane & h;
		const float2 w = twiddle<false>(table, tw_offset(N) + (lane & (h - 1)) * (N / (2 * h)));
#pragma unroll
		for (int k1 = 0; k1 < P; k1++) {
			const float2 o = shfl_xor2(v[k1], h);
			v[k1] = upper ? cmulf(csubf(o, v[k1]), w) : caddf(v[k1], o);
		}
	}
}

// inverse of warp_fft_forward times N (the unnormalised inverse DFT)
template <int N>
__device__ __forceinline__ void warp_fft_inverse(float2 (&v)[N / 32], int lane, const float2 *__restrict__ table)
{
	constexpr int P = N / 32;
#pragma unroll
	for (int h = 1; h <= 16; h <<= 1) {
		const bool upper = lane & h;
		const float2 w = twiddle<true>(table, tw_offset(N) + (lane & (h - 1)) * (N / (2 * h)));
#pragma unroll
		for (int k1 = 0; k1 < P; k1++) {
			const float2 o = shfl_xor2(v[k1], h);
			// lower lane: its own sum term, the partner's difference term; upper: the reverse
			const float2 t = cmulf(upper ? v[k1] : o, w);
			v[k1] = upper ? csubf(o, t) : caddf(v[k1], t);
		}
	}
#pragma unroll
	for (int k1 = 1; k1 < P; k1++) v[k1] = cmulf(v[k1], twiddle<true>(table, tw_offset(N) + lane * k1));
	dft_reg<P, true>(v);
}

// Pass 2 for warp_cols<N>() lengths: 8 bin columns per block, one per warp.
// The spectrum pass (F_SPECTRUM) stores its columns' transforms in the
// warps' own order (column c at spec[c N + 32 k1 + lane]).
template <int N, int MODE>
__global__ void __launch_bounds__(256)
cols_w_kernel(const ModelDev *__restrict__ models, const Job *__restrict__ jobs, float2 *__restrict__ work,
              float2 *__restrict__ spec, const float2 *__restrict__ table)
{
	constexpr int F = 8, P = N / 32, PS = N + 1;
	extern __shared__ float2 fsm[];
	float2 *cbuf = fsm;
	const Job jb = jobs[blockIdx.x];
	const ModelDev &m = models[jb.model];
	const int nb = (int)m.fft_mx / 2 + 1;
	const int warp = (int)threadIdx.x >> 5, lane = (int)threadIdx.x & 31;
	float2 *col = work + m.fft_work_off;
	int rows_in, yoff = 0;
	if (MODE == F_FORWARD) rows_in = (int)m.draw_h;
	else if (MODE == F_ADJOINT) {
		rows_in = (int)m.crop_h;
		yoff = (int)m.pad_y + (int)m.psf_h - 1 - (int)m.psf_h / 2;
	}
	else rows_in = (int)m.psf_h;
	// coalesced loads of the job's columns (F x 8 bytes per row), P per thread,
	// all issued before the shared-memory stores
	float2 v[P];
#pragma unroll
	for (int q = 0; q < P; q++) {
		const int i = (int)threadIdx.x + q * 256;
		const int rg = i / F, ff = i % F;
		const int r = rg - yoff;
		v[q] = make_float2(0.f, 0.f);
		if (ff < jb.count && r >= 0 && r < rows_in) v[q] = col[(size_t)r * nb + jb.first + ff];
	}
#pragma unroll
	for (int q = 0; q < P; q++) {
		const int i = (int)threadIdx.x + q * 256;
		cbuf[(i % F) * PS + i / F] = v[q];
	}
	__syncthreads();
	const bool live = warp < jb.count;
	const int c = jb.first + warp;
	float2 x[P];
#pragma unroll
	for (int p = 0; p < P; p++) x[p] = cbuf[warp * PS + lane + 32 * p];
	warp_fft_forward<N>(x, lane, table);
	if (MODE == F_SPECTRUM) {
		if (live) {
			float2 *sp = spec + m.fft_spec_off + (size_t)c * N;
#pragma unroll
			for (int k1 = 0; k1 < P; k1++) sp[32 * k1 + lane] = x[k1];
		}
		return;
	}
	if (live) {
		const float2 *sp = spec + m.fft_spec_off + (size_t)c * N;
		float2 sv[P];
#pragma unroll
		for (int k1 = 0; k1 < P; k1++) sv[k1] = sp[32 * k1 + lane];
#pragma unroll
		for (int k1 = 0; k1 < P; k1++) {
			if (MODE == F_ADJOINT) sv[k1].y = -sv[k1].y;
			x[k1] = cmulf(x[k1], sv[k1]);
		}
	}
	warp_fft_inverse<N>(x, lane, table);
#pragma unroll
	for (int p = 0; p < P; p++) cbuf[warp * PS + lane + 32 * p] = x[p];
	__syncthreads();
	// kept rows: forward, the crop's (from its offset); adjoint, the drawing area's
	const int rows_out = MODE == F_FORWARD ? (int)m.crop_h : (int)m.draw_h;
	const int keep = MODE == F_FORWARD ? (int)m.pad_y + (int)m.psf_h - 1 - (int)m.psf_h / 2 : 0;
#pragma unroll 4
	for (int i = threadIdx.x; i < F * rows_out; i += blockDim.x) {
		const int r = i / F, ff = i % F;
		if (ff < jb.count) col[(size_t)r * nb + jb.first + ff] = cbuf[ff * PS + r + keep];
	}
}

// Pass 3: inverse rows. Job rows first .. first + count - 1 of the kept rows,
// two per transform: Z(k) = A(k) + i B(k) over all k, A and B Hermitian.
template <int N, int MODE>
__global__ void __launch_bounds__(row_ffts<N>() * (N / 8))
irows_kernel(const ModelDev *__restrict__ models, const Job *__restrict__ jobs, const float2 *__restrict__ work,
             const float *__restrict__ direct, float *__restrict__ out, const float2 *__restrict__ table)
{
	constexpr int F = row_ffts<N>(), PS = row_stride<N>();
	extern __shared__ float2 fsm[];
	float2 *buf = fsm;
	const Job jb = jobs[blockIdx.x];
	const ModelDev &m = models[jb.model];
	const int nb = (int)m.fft_mx / 2 + 1;
	const int f = threadIdx.x / (N / 8), t = threadIdx.x % (N / 8);
	const float2 *src = work + m.fft_work_off;
	// each stored bin k <= N/2 of the two rows loaded once (all loads issued
	// before the shared-memory stores), Z(k) = A(k) + i B(k) written at k and,
	// from A(N-k) = conj A(k), B(N-k) = conj B(k), at N - k
	constexpr int NB = N / 2 + 1, T = F * (N / 8), Q = (F * NB + T - 1) / T;
	float2 a[Q], b[Q];
#pragma unroll
	for (int q = 0; q < Q; q++) {
		const int i = (int)threadIdx.x + q * T;
		const int ff = i / NB, k = i % NB;
		const int r0 = jb.first + 2 * ff, r1 = r0 + 1;
		a[q] = b[q] = make_float2(0.f, 0.f);
		if (i < F * NB) {
			if (r0 < jb.first + jb.count) a[q] = src[(size_t)r0 * nb + k];
			if (r1 < jb.first + jb.count) b[q] = src[(size_t)r1 * nb + k];
		}
	}
#pragma unroll
	for (int q = 0; q < Q; q++) {
		const int i = (int)threadIdx.x + q * T;
		if (i >= F * NB) continue;
		const int ff = i / NB, k = i % NB;
		buf[ff * PS + pidx(k)] = make_float2(a[q].x - b[q].y, a[q].y + b[q].x);
		if (k > 0 && k < N - k) buf[ff * PS + pidx(N - k)] = make_float2(a[q].x + b[q].y, b[q].x - a[q].y);
	}
	__syncthreads();
	fft<N, true>(buf + f * PS, t, table);
	const float scale = 1.f / ((float)m.fft_mx * (float)m.fft_my);
	if (MODE == F_FORWARD) {
		const int off_x = (int)m.pad_x + (int)m.psf_w - 1 - (int)m.psf_w / 2;
		const bool downsample = m.fs > 1 && !m.return_fs;
		const int cw = (int)m.crop_w;
#pragma unroll 4
		for (int i = threadIdx.x; i < F * 2 * cw; i += blockDim.x) {
			const int ff = i / (2 * cw), rem = i % (2 * cw), half = rem / cw, c = rem % cw;
			const int r = jb.first + 2 * ff + half;
			if (r >= jb.first + jb.count) continue;
			const float2 z = buf[ff * PS + pidx(c + off_x)];
			// the convolution is zero where the calculation mask is; the output
			// is multiplied by the model's mask at the end
			const float conv = evaluated(m, c + (int)m.pad_x, r + (int)m.pad_y) ? (half ? z.y : z.x) * scale : 0.f;
			const float dir = m.direct_required ? direct[m.draw_off + (size_t)(r + m.pad_y) * m.draw_w + c + m.pad_x] : 0.f;
			const float v = dir + conv;
			if (downsample) {
				if (kept(m, c / (int)m.fs, r / (int)m.fs))
					atomicAdd(&out[m.out_off + (size_t)(r / m.fs) * m.out_w + c / m.fs], v);
			}
			else out[m.out_off + (size_t)r * m.out_w + c] = kept(m, c, r) ? v : 0.f;
		}
	}
	else {
		const int dw = (int)m.draw_w;
		for (int i = threadIdx.x; i < F * 2 * dw; i += blockDim.x) {
			const int ff = i / (2 * dw), rem = i % (2 * dw), half = rem / dw, c = rem % dw;
			const int r = jb.first + 2 * ff + half;
			if (r >= jb.first + jb.count) continue;
			const float2 z = buf[ff * PS + pidx(c)];
			out[m.draw_off + (size_t)r * m.draw_w + c] = (half ? z.y : z.x) * scale;
		}
	}
}

template <int N>
constexpr size_t rows_smem() { return sizeof(float2) * row_ffts<N>() * row_stride<N>(); }
template <int N>
constexpr size_t cols_smem()
{
	return warp_cols<N>() ? sizeof(float2) * 8 * (N + 1) : sizeof(float2) * col_ffts<N>() * col_stride<N>();
}

template <int N>
cudaError_t configure_n()
{
	const int rs = (int)rows_smem<N>(), cs = (int)cols_smem<N>();
	const cudaFuncAttribute a = cudaFuncAttributeMaxDynamicSharedMemorySize;
	cudaError_t e = cudaFuncSetAttribute(rows_kernel<N, F_FORWARD>, a, rs);
	if (e == cudaSuccess) e = cudaFuncSetAttribute(rows_kernel<N, F_ADJOINT>, a, rs);
	if (e == cudaSuccess) e = cudaFuncSetAttribute(rows_kernel<N, F_SPECTRUM>, a, rs);
	if (e == cudaSuccess) e = cudaFuncSetAttribute(irows_kernel<N, F_FORWARD>, a, rs);
	if (e == cudaSuccess) e = cudaFuncSetAttribute(irows_kernel<N, F_ADJOINT>, a, rs);
	if constexpr (warp_cols<N>()) {
		if (e == cudaSuccess) e = cudaFuncSetAttribute(cols_w_kernel<N, F_FORWARD>, a, cs);
		if (e == cudaSuccess) e = cudaFuncSetAttribute(cols_w_kernel<N, F_ADJOINT>, a, cs);
		if (e == cudaSuccess) e = cudaFuncSetAttribute(cols_w_kernel<N, F_SPECTRUM>, a, cs);
	}
	else {
		if (e == cudaSuccess) e = cudaFuncSetAttribute(cols_kernel<N, F_FORWARD>, a, cs);
		if (e == cudaSuccess) e = cudaFuncSetAttribute(cols_kernel<N, F_ADJOINT>, a, cs);
		if (e == cudaSuccess) e = cudaFuncSetAttribute(cols_kernel<N, F_SPECTRUM>, a, cs);
	}
	return e;
}

template <int N>
void launch_n(int pass, int mode, int n_jobs, const ModelDev *models, const Job *jobs, const float *src,
              const float *psf, float2 *work, float2 *spec, const float *direct, float *out, const float2 *tw,
              cudaStream_t stream)
{
	const int rthreads = row_ffts<N>() * (N / 8), cthreads = col_ffts<N>() * (N / 8);
	const size_t rsmem = rows_smem<N>(), csmem = cols_smem<N>();
	if (pass == 0) {
		if (mode == F_FORWARD) rows_kernel<N, F_FORWARD><<<n_jobs, rthreads, rsmem, stream>>>(models, jobs, src, psf, work, spec, tw);
		else if (mode == F_ADJOINT) rows_kernel<N, F_ADJOINT><<<n_jobs, rthreads, rsmem, stream>>>(models, jobs, src, psf, work, spec, tw);
		else rows_kernel<N, F_SPECTRUM><<<n_jobs, rthreads, rsmem, stream>>>(models, jobs, src, psf, work, spec, tw);
	}
	else if (pass == 1) {
		if constexpr (warp_cols<N>()) {
			if (mode == F_FORWARD) cols_w_kernel<N, F_FORWARD><<<n_jobs, 256, csmem, stream>>>(models, jobs, work, spec, tw);
			else if (mode == F_ADJOINT) cols_w_kernel<N, F_ADJOINT><<<n_jobs, 256, csmem, stream>>>(models, jobs, work, spec, tw);
			else cols_w_kernel<N, F_SPECTRUM><<<n_jobs, 256, csmem, stream>>>(models, jobs, work, spec, tw);
		}
		else {
			if (mode == F_FORWARD) cols_kernel<N, F_FORWARD><<<n_jobs, cthreads, csmem, stream>>>(models, jobs, work, spec, tw);
			else if (mode == F_ADJOINT) cols_kernel<N, F_ADJOINT><<<n_jobs, cthreads, csmem, stream>>>(models, jobs, work, spec, tw);
			else cols_kernel<N, F_SPECTRUM><<<n_jobs, cthreads, csmem, stream>>>(models, jobs, work, spec, tw);
		}
	}
	else {
		if (mode == F_FORWARD) irows_kernel<N, F_FORWARD><<<n_jobs, rthreads, rsmem, stream>>>(models, jobs, work, direct, out, tw);
		else irows_kernel<N, F_ADJOINT><<<n_jobs, rthreads, rsmem, stream>>>(models, jobs, work, direct, out, tw);
	}
}

// The launches of one group's lengths: false if n is not one of them.
#define PF_FFT32_GROUP_LAUNCH(N) \
	case N: launch_n<N>(pass, mode, n_jobs, models, jobs, src, psf, work, spec, direct, out, tw, stream); return true;
#define PF_FFT32_GROUP_CONF(N) \
	if (e == cudaSuccess) e = configure_n<N>();

}  // namespace

cudaError_t fft32_configure_b();
cudaError_t fft32_configure_c();
bool fft32_launch_b(int pass, int mode, int n, int n_jobs, const ModelDev *models, const Job *jobs, const float *src,
                    const float *psf, float2 *work, float2 *spec, const float *direct, float *out, const float2 *tw,
                    cudaStream_t stream);
bool fft32_launch_c(int pass, int mode, int n, int n_jobs, const ModelDev *models, const Job *jobs, const float *src,
                    const float *psf, float2 *work, float2 *spec, const float *direct, float *out, const float2 *tw,
                    cudaStream_t stream);

}  // namespace pf
