// Register-blocked direct convolution on the CUDA cores, for the batched path:
// the kernels, included by conv.cu (the PSF row stride read per model) and by
// conv_k*.cu (one row stride each, known at compile time).
//
// Both directions of the PSF convolution of Model::produce_image
// (src/model.cpp:344-356; the convolution itself is the brute-force one of
// src/convolve.cpp:158-231, zero outside the source):
//   forward  out(o) = direct(o + pad) + sum_{k,l} src(o + pad + (k,l) - h) rev(k,l)
//            over the output pixels, then the crop, optionally SUM-downsampled;
//   adjoint  g_src(q) = sum_{k,l} G(q + (k,l) - h') psf(k,l), h' = size - 1 - h,
//            over the drawing area, G = the output cotangent placed at the crop.
// A block stages a source patch and the (reversed or not) PSF, zero-padded to
// a multiple of 4 columns, in shared memory. Each thread owns a C-wide (4 or
// 8) by R-tall block of outputs; it reads every source row of its patch once,
// as 16-byte vectors, and applies it to all the kernel rows that touch it,
// taking four kernel taps per 16-byte broadcast read, so that a shared-memory
// read feeds up to C R FMAs.
#pragma once

#include <cstdint>
#include <type_traits>

#include "pf_device.cuh"

namespace pf {

namespace {

// Block shapes: TX x TY threads, each C columns by R rows of outputs.
//   float  0: 16 x 16, 4 x 8 -> 64 x 128 outputs
//   float  1: 14 x 14, 4 x 5 -> 56 x 70
//   float  2: 16 x 12, 4 x 8 -> 64 x 96
//   float  3: 14 x 10, 4 x 7 -> 56 x 70
//   float  4: 35 x 7, 4 x 8  -> 140 x 56
//   double 0: 16 x 8, 4 x 4  -> 64 x 32
// (8 columns per thread, 64 x 128 and 128 x 64 tiles, measured slower in
// both directions on the 1024-model step.)
// The host picks, per batch and direction, the shape that wastes the least
// tile area over the images it convolves, or, for large single-precision
// batches, the one the autotuner timed fastest.
struct Shape {
	int tx, ty, r, c;
};
__host__ __device__ constexpr Shape shape_of(bool dbl, int id)
{
	return dbl ? Shape{16, 8, 4, 4}
	           : id == 1 ? Shape{14, 14, 5, 4}
	           : id == 2 ? Shape{16, 12, 8, 4}
	           : id == 3 ? Shape{14, 10, 7, 4}
	           : id == 4 ? Shape{35, 7, 8, 4}
	                     : Shape{16, 16, 8, 4};
}

template <typename T>
struct Vec4;
template <>
struct Vec4<float> {
	using type = float4;
};
template <>
struct Vec4<double> {
	using type = double4_16a;
};

enum ConvMode { CONV_FORWARD = 0, CONV_ADJOINT = 1 };

__device__ __forceinline__ int find_tile_model(const long long *base, int n_models, long long tile)
{
	int lo = 0, hi = n_models - 1;
	while (lo < hi) {
		int mid = (lo + hi + 1) >> 1;
		if (base[mid] <= tile) lo = mid; else hi = mid - 1;
	}
	return lo;
}

// cotangent of drawing pixel (x, y) (0 in the padding, SUM-downsampling aware)
template <typename T>
__device__ __forceinline__ T cot_at(const ModelDev &m, const T *gout, int x, int y)
{
	const int cx = x - (int)m.pad_x, cy = y - (int)m.pad_y;
	if (cx < 0 || cy < 0 || cx >= (int)m.crop_w || cy >= (int)m.crop_h) return (T)0;
	if (!evaluated(m, x, y)) return (T)0;  // the forward convolution is zero there
	if (m.fs > 1 && !m.return_fs) return gout[m.out_off + (size_t)(cy / m.fs) * m.out_w + cx / m.fs];
	return gout[m.out_off + (size_t)cy * m.out_w + cx];
}

// C + 4 source values from srow: the thread's C columns and the next 4
template <typename T, int C>
__device__ __forceinline__ void load_src(const T *srow, T (&w)[C + 4])
{
	using V4 = typename Vec4<T>::type;
#pragma unroll
	for (int v = 0; v < C / 4 + 1; v++) {
		const V4 x = *reinterpret_cast<const V4 *>(srow + 4 * v);
		w[4 * v] = x.x;
		w[4 * v + 1] = x.y;
		w[4 * v + 2] = x.z;
		w[4 * v + 3] = x.w;
	}
}

// The multiply-adds of one source row (srow, this thread's C + 4 columns)
// into output rows r0..r1 (kernel row s - r), over the kw4 = 4 floor(kw / 4)
// taps of whole groups of four; with r0 and r1 known at compile time after
// unrolling, the row loop carries no tests. KWP > 0: the kernel's row stride
// in shared memory, known at compile time, so that the R kernel rows' reads
// are immediate offsets from one address per tap group.
template <typename T, int R, int C, int KWP>
__device__ __forceinline__ void conv_rows(const T *srow, const T *s_k, int s, int kwp, int kw4, int r0, int r1,
                                          T (&acc)[R][C])
{
	using V4 = typename Vec4<T>::type;
	if constexpr (KWP > 0) {
		// not unrolled: fully unrolled ramps took over a minute to compile per
		// stride and outgrew the instruction cache
		const T *krow = s_k + s * KWP;
#pragma unroll 1
		for (int kb = 0; kb < kw4; kb += 4) {
			T w[C + 4];
			load_src<T, C>(srow + kb, w);
#pragma unroll
			for (int r = 0; r < R; r++) {
				if (r < r0 || r > r1) continue;
				const V4 kv4 = *reinterpret_cast<const V4 *>(krow - r * KWP + kb);
				const T kv[4] = {kv4.x, kv4.y, kv4.z, kv4.w};
#pragma unroll
				for (int c = 0; c < C; c++)
#pragma unroll
					for (int q = 0; q < 4; q++) acc[r][c] = fma(w[c + q], kv[q], acc[r][c]);
			}
		}
	}
	else {
		for (int kb = 0; kb < kw4; kb += 4) {
			T w[C + 4];
			load_src<T, C>(srow + kb, w);
#pragma unroll
			for (int r = 0; r < R; r++) {
				if (r < r0 || r > r1) continue;
				const V4 kv4 = *reinterpret_cast<const V4 *>(s_k + (s - r) * kwp + kb);
				const T kv[4] = {kv4.x, kv4.y, kv4.z, kv4.w};
#pragma unroll
				for (int c = 0; c < C; c++)
#pragma unroll
					for (int q = 0; q < 4; q++) acc[r][c] = fma(w[c + q], kv[q], acc[r][c]);
			}
		}
	}
}

// The kw mod 4 taps past kw4 (tail of them), one by one, in a pass of their
// own after every source row's whole groups: fewer multiply-adds than a
// zero-padded group (measured 2.75 -> 2.68 ms for the adjoint of 1024 models
// of 280 x 280 with a 25 x 25 PSF, the forward unchanged). KWP > 0: kw4 =
// KWP - 4 whenever there is a tail.
template <typename T, int R, int C, int KWP>
__device__ __forceinline__ void conv_tail(const T *srow, const T *s_k, int s, int kwp, int kw4, int tail, int r0,
                                          int r1, T (&acc)[R][C])
{
	constexpr bool fixed = KWP > 0;
	const int k4 = fixed ? KWP - 4 : kw4;
	const T *krow = s_k + s * (fixed ? KWP : kwp) + k4;
	T w[C + 4];
	load_src<T, C>(srow + k4, w);
#pragma unroll
	for (int q = 0; q < 3; q++) {
		if (q >= tail) break;
#pragma unroll
		for (int r = 0; r < R; r++) {
			if (r < r0 || r > r1) continue;
			const T kv = krow[q - r * (fixed ? KWP : kwp)];
#pragma unroll
			for (int c = 0; c < C; c++) acc[r][c] = fma(w[c + q], kv, acc[r][c]);
		}
	}
}

// Register cap per thread of the convolution kernels (0: the compiler's
// choice), as a minimum of resident blocks per SM.
#ifndef PF_CONV_REGS
#define PF_CONV_REGS 0
#endif
#if PF_CONV_REGS > 0
__host__ __device__ constexpr int conv_min_blocks(int threads) { return 65536 / (threads * PF_CONV_REGS); }
#define PF_CONV_BOUNDS(threads) __launch_bounds__(threads, conv_min_blocks(threads))
#else
#define PF_CONV_BOUNDS(threads) __launch_bounds__(threads)
#endif
template <typename T, int MODE, int TX, int TY, int R, int C, int KWP>
__global__ void PF_CONV_BOUNDS(TX * TY)
conv_kernel(const ModelDev *__restrict__ models, int n_models, const T *__restrict__ psf, const T *__restrict__ in,
            const T *__restrict__ direct, T *__restrict__ out, const long long *__restrict__ tile_base,
            long long n_tiles)
{
	constexpr int BW = TX * C, BH = TY * R;  // outputs per block
	using V4 = typename Vec4<T>::type;
	extern __shared__ __align__(16) unsigned char smem_raw[];
	T *smem = reinterpret_cast<T *>(smem_raw);
	const int tx = threadIdx.x % TX, ty = threadIdx.x / TX;
	for (long long tile = blockIdx.x; tile < n_tiles; tile += gridDim.x) {
		const int mi = find_tile_model(tile_base, n_models, tile);
		const ModelDev &m = models[mi];
		if (!m.conv_required && MODE == CONV_ADJOINT) continue;
		const long long local = tile - tile_base[mi];
		const int ow = MODE == CONV_FORWARD ? (int)m.crop_w : (int)m.draw_w;
		const int oh = MODE == CONV_FORWARD ? (int)m.crop_h : (int)m.draw_h;
		const int tiles_x = (ow + BW - 1) / BW;
		const int x0 = (int)(local % tiles_x) * BW, y0 = (int)(local / tiles_x) * BH;
		T acc[R][C];
#pragma unroll
		for (int r = 0; r < R; r++)
#pragma unroll
			for (int c = 0; c < C; c++) acc[r][c] = 0;
		if (m.conv_required) {
			const int kw = (int)m.psf_w, kh = (int)m.psf_h;
			const int kwp = KWP > 0 ? KWP : (kw + 3) & ~3;  // the host checks KWP against kw
			const int pw = BW + kwp, ph = BH + kh - 1;
			T *s_src = smem;
			T *s_k = smem + pw * ph;
			// patch origin in the source (drawing) image
			int sx0, sy0;
			if (MODE == CONV_FORWARD) {
				sx0 = x0 + (int)m.pad_x - kw / 2;
				sy0 = y0 + (int)m.pad_y - kh / 2;
			}
			else {
				sx0 = x0 - (kw - 1 - kw / 2);
				sy0 = y0 - (kh - 1 - kh / 2);
			}
			const T *src = in + (MODE == CONV_FORWARD ? m.draw_off : 0);
			if (MODE == CONV_FORWARD) {
				// one full warp per patch row, lanes along it (coalesced, no index
				// division); the threads of a partial last warp take no part
				const int lane = threadIdx.x & 31, nwarp = (TX * TY) >> 5;
				for (int py = (int)threadIdx.x >> 5; py < ph && ((int)threadIdx.x >> 5) < nwarp; py += nwarp) {
					const int yy = sy0 + py;
					const bool row_in = yy >= 0 && yy < (int)m.draw_h;
					T *dst = s_src + py * pw;
					for (int px = lane; px < pw; px += 32) {
						const int xx = sx0 + px;
						T v = 0;
						if (px < BW + kw - 1 && row_in && xx >= 0 && xx < (int)m.draw_w) {
							v = src[(size_t)yy * m.draw_w + xx];
						}
						dst[px] = v;
					}
				}
			}
			else {
				// the cotangent placed at the crop (measured faster flattened over
				// every thread of the block than row by row)
				for (int i = threadIdx.x; i < pw * ph; i += blockDim.x) {
					const int px = i % pw;
					s_src[i] = px < BW + kw - 1 ? cot_at(m, in, sx0 + px, sy0 + i / pw) : (T)0;
				}
			}
			const T *k = psf + m.psf_off;
			const int kn = kw * kh;
			for (int i = threadIdx.x; i < kwp * kh; i += blockDim.x) {
				const int kx = i % kwp, ky = i / kwp;
				T v = 0;
				if (kx < kw) v = MODE == CONV_FORWARD ? k[kn - 1 - (ky * kw + kx)] : k[ky * kw + kx];
				s_k[i] = v;
			}
			__syncthreads();
			const int xb = tx * C, yb = ty * R;
			const int kw4 = kw & ~3, tail = kw & 3;
			if (kh >= R) {
				// source row s feeds output rows r with kernel row l = s - r in
				// [0, kh): rows 0..s while s < R - 1, all rows up to s = kh - 1,
				// rows s - kh + 1 .. R - 1 after; the ramps are unrolled so that no
				// row test is left in the multiply-add stream
#pragma unroll
				for (int s0 = 0; s0 < R - 1; s0++)
					conv_rows<T, R, C, KWP>(s_src + (yb + s0) * pw + xb, s_k, s0, kwp, kw4, 0, s0, acc);
				for (int s0 = R - 1; s0 < kh; s0++)
					conv_rows<T, R, C, KWP>(s_src + (yb + s0) * pw + xb, s_k, s0, kwp, kw4, 0, R - 1, acc);
#pragma unroll
				for (int d = 0; d < R - 1; d++) {
					conv_rows<T, R, C, KWP>(s_src + (yb + kh + d) * pw + xb, s_k, kh + d, kwp, kw4, d + 1, R - 1, acc);
				}
			}
			else {
				for (int s0 = 0; s0 < R + kh - 1; s0++) {
					conv_rows<T, R, C, KWP>(s_src + (yb + s0) * pw + xb, s_k, s0, kwp, kw4, max(0, s0 - kh + 1),
					                   min(R - 1, s0), acc);
				}
			}
			if (tail) {
				for (int s0 = 0; s0 < R + kh - 1; s0++) {
					conv_tail<T, R, C, KWP>(s_src + (yb + s0) * pw + xb, s_k, s0, kwp, kw4, tail, max(0, s0 - kh + 1),
					                   min(R - 1, s0), acc);
				}
			}
			__syncthreads();
		}
		const int xo = x0 + tx * C;
#pragma unroll
		for (int r = 0; r < R; r++) {
			const int yo = y0 + ty * R + r;
			if (yo >= oh) continue;
#pragma unroll
			for (int c = 0; c < C; c++) {
				const int x = xo + c;
				if (x >= ow) continue;
				if (MODE == CONV_FORWARD) {
					// the convolution is zero where the calculation mask is, and the
					// output is multiplied by the model's mask at the end
					const bool conv_here = evaluated(m, x + (int)m.pad_x, yo + (int)m.pad_y);
					const T dir =
					    m.direct_required ? direct[m.draw_off + (size_t)(yo + m.pad_y) * m.draw_w + x + m.pad_x] : (T)0;
					const T v = dir + (conv_here ? acc[r][c] : (T)0);
					if (m.fs > 1 && !m.return_fs) {
						if (kept(m, x / (int)m.fs, yo / (int)m.fs))
							atomicAdd(&out[m.out_off + (size_t)(yo / m.fs) * m.out_w + x / m.fs], v);
					}
					else out[m.out_off + (size_t)yo * m.out_w + x] = kept(m, x, yo) ? v : (T)0;
				}
				else {
					out[m.draw_off + (size_t)yo * m.draw_w + x] = acc[r][c];
				}
			}
		}
	}
}


// The kernels of the five single-precision block shapes (or the one double
// shape) for row stride KWP (0: read per model): shared memory sizing and
// launch.
template <typename T, int KWP>
cudaError_t configure_kernels(size_t smem, int shape)
{
	const auto set = [smem](auto kernel) {
		return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
	};
#define PF_CONV_SET(TX, TY, R, C)                                                     \
	do {                                                                              \
		cudaError_t e = set(conv_kernel<T, CONV_FORWARD, TX, TY, R, C, KWP>);         \
		return e != cudaSuccess ? e : set(conv_kernel<T, CONV_ADJOINT, TX, TY, R, C, KWP>); \
	} while (0)
	if constexpr (std::is_same<T, double>::value) {
		PF_CONV_SET(16, 8, 4, 4);
	}
	else {
		if (shape == 1) PF_CONV_SET(14, 14, 5, 4);
		if (shape == 2) PF_CONV_SET(16, 12, 8, 4);
		if (shape == 3) PF_CONV_SET(14, 10, 7, 4);
		if (shape == 4) PF_CONV_SET(35, 7, 8, 4);
		PF_CONV_SET(16, 16, 8, 4);
	}
#undef PF_CONV_SET
}

template <typename T, int KWP>
void launch_kernels(int mode, int shape, const ModelDev *models, int n_models, const T *psf, const T *in,
                    const T *direct, T *out, const long long *tile_base, long long n_tiles, size_t smem, int n_sm,
                    cudaStream_t stream)
{
	int blocks = (int)(n_tiles < (long long)n_sm * 8 ? n_tiles : (long long)n_sm * 8);
	if (blocks < 1) blocks = 1;
#define PF_CONV_GO(TX, TY, R, C)                                                                             \
	do {                                                                                                     \
		if (mode == CONV_FORWARD)                                                                            \
			conv_kernel<T, CONV_FORWARD, TX, TY, R, C, KWP><<<blocks, TX * TY, smem, stream>>>(              \
			    models, n_models, psf, in, direct, out, tile_base, n_tiles);                                 \
		else                                                                                                 \
			conv_kernel<T, CONV_ADJOINT, TX, TY, R, C, KWP><<<blocks, TX * TY, smem, stream>>>(              \
			    models, n_models, psf, in, direct, out, tile_base, n_tiles);                                 \
		return;                                                                                              \
	} while (0)
	if constexpr (std::is_same<T, double>::value) {
		PF_CONV_GO(16, 8, 4, 4);
	}
	else {
		if (shape == 1) PF_CONV_GO(14, 14, 5, 4);
		if (shape == 2) PF_CONV_GO(16, 12, 8, 4);
		if (shape == 3) PF_CONV_GO(14, 10, 7, 4);
		if (shape == 4) PF_CONV_GO(35, 7, 8, 4);
		PF_CONV_GO(16, 16, 8, 4);
	}
#undef PF_CONV_GO
}

}  // namespace

// Single-precision entry points for one compiled-in row stride K (defined in
// conv_kK.cu).
#define PF_CONV_FIXED_DECL(K)                                                                                   \
	cudaError_t conv_configure_f##K(size_t smem, int shape);                                                   \
	void launch_conv_f##K(int mode, int shape, const ModelDev *models, int n_models, const float *psf,          \
	                      const float *in, const float *direct, float *out, const long long *tile_base,         \
	                      long long n_tiles, size_t smem, int n_sm, cudaStream_t stream);
#define PF_CONV_FIXED_DEF(K)                                                                                    \
	cudaError_t conv_configure_f##K(size_t smem, int shape) { return configure_kernels<float, K>(smem, shape); } \
	void launch_conv_f##K(int mode, int shape, const ModelDev *models, int n_models, const float *psf,          \
	                      const float *in, const float *direct, float *out, const long long *tile_base,         \
	                      long long n_tiles, size_t smem, int n_sm, cudaStream_t stream)                        \
	{                                                                                                          \
		launch_kernels<float, K>(mode, shape, models, n_models, psf, in, direct, out, tile_base, n_tiles, smem,   \
		                         n_sm, stream);                                                                \
	}
// the row strides compiled in: PSF widths 13 to 32
#define PF_CONV_FIXED_ALL(X) X(16) X(20) X(24) X(28) X(32)
PF_CONV_FIXED_ALL(PF_CONV_FIXED_DECL)

}  // namespace pf
