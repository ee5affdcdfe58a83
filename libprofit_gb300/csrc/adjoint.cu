// Adjoint (vector-Jacobian product) of the rendered images with respect to
// every profile parameter, and of chi^2 = sum ((model - data) / sigma)^2.
// libprofit has no derivatives; this follows its forward definition:
//
//   out(o)  = direct(o + pad) + sum_k src(o + pad + k - h) rev(k)         (finish)
//   src(q)  = sum_profiles flux_scale_p * v_p(q)                          (eval)
//   v_p(q)  = f_p(q) or sum over the leaves of q's subsampling tree of
//             w_leaf f_p(leaf), w_leaf = res^-2(level+1)                   (subsample_pixel)
//
// With the cotangent g_out = d L / d out:
//   1. g_src = the transposed convolution of g_out (drawing area, a direct
//      convolution with the unreversed PSF);
//   2. for each profile, over its pixels, S_v = sum g v and
//      S_theta = sum g sum_leaves w f d ln f / d theta, the subsampling tree
//      recomputed exactly as the forward pass builds it and held fixed;
//   3. d L / d theta = flux_scale (S_theta + d ln flux_scale / d theta * S_v).
// Per-item partial sums are written in FP64 and reduced in a fixed order, so
// gradients and chi^2 are deterministic.
//
// Profiles supported by the adjoint: sersic (all eight parameters xcen, ycen,
// mag, ang, axrat, box, re, nser; not rescale_flux) and sky (bg).
#include <cstdint>
#include <type_traits>

#include "pf_device.cuh"
#include "profiles_f32.cuh"
#include "profiles_f64.cuh"

namespace pf {

namespace {

constexpr int kBandRows = 16;    // drawing rows per backward work item
constexpr int kWarpsB = 8;
// the forward pass's guard bands (eval_f32.cu), so that both take the same decisions
constexpr float kGuardAccB = 1.2e-5f;
constexpr float kGuardRadiusB = 2e-6f;

template <typename T>
__device__ __forceinline__ T warp_sum_t(T v)
{
#pragma unroll
	for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
	return v;
}

// ------------------------------------------------------------ chi^2, g_out

template <typename T>
__global__ void chi2_kernel(const ModelDev *__restrict__ models, const T *__restrict__ img, const T *__restrict__ data,
                            const T *__restrict__ sigma, const T *__restrict__ cot, T *__restrict__ gout,
                            double *__restrict__ chi2)
{
	const ModelDev &m = models[blockIdx.x];
	const long long n = (long long)m.out_w * m.out_h;
	double s = 0;
	for (long long i = threadIdx.x; i < n; i += blockDim.x) {
		const long long g = m.out_off + i;
		if (cot) {
			gout[g] = cot[g];
		}
		else {
			const T r = img[g] - data[g];
			const T w = sigma ? (T)1 / (sigma[g] * sigma[g]) : (T)1;
			s += (double)w * (double)r * (double)r;
			gout[g] = (T)2 * w * r;
		}
	}
	__shared__ double part[256];
	part[threadIdx.x] = s;
	__syncthreads();
	for (int w = blockDim.x / 2; w > 0; w >>= 1) {
		if ((int)threadIdx.x < w) part[threadIdx.x] += part[threadIdx.x + w];
		__syncthreads();
	}
	if (threadIdx.x == 0 && chi2) chi2[blockIdx.x] = cot ? 0. : part[0];
}

// cotangent of drawing pixel (x, y): the output pixel it lands in after the
// crop (and the SUM downsampling), 0 in the padding
template <typename T>
__device__ __forceinline__ T g_direct(const ModelDev &m, const T *gout, int x, int y)
{
	const int cx = x - (int)m.pad_x, cy = y - (int)m.pad_y;
	if (cx < 0 || cy < 0 || cx >= (int)m.crop_w || cy >= (int)m.crop_h) return (T)0;
	if (m.fs > 1 && !m.return_fs) {
		return gout[m.out_off + (size_t)(cy / m.fs) * m.out_w + cx / m.fs];
	}
	return gout[m.out_off + (size_t)cy * m.out_w + cx];
}


// value and shape derivatives d ln f / d theta of the sersic profile at
// profile coordinates (xp, yp); acc[] += weight * f * (1, d/dxcen, d/dycen,
// d/dang, d/daxrat, d/dbox, d/dre, d/dnser)
template <typename T>
__device__ __forceinline__ void sersic_grad(const ProfileDev &P, T xp, T yp, T weight, T *acc)
{
	constexpr bool dbl = std::is_same<T, double>::value;
	const T n = dbl ? (T)P.par[7] : (T)P.fnser;
	const T re = dbl ? (T)P.par[6] : (T)P.fre;
	const T bn = dbl ? (T)P.bn : (T)P.fbn;
	const T dbn = dbl ? (T)P.dbn : (T)P.fdbn;
	const T B = dbl ? (T)(P.par[PF_P_BOX] + 2) : (T)P.fpar[FP_B];
	const T q = dbl ? (T)P.par[PF_P_AXRAT] : (T)1 / P.finv_axrat;
	const T c = dbl ? (T)P.cos_ang : (T)P.fcos;
	const T s = dbl ? (T)P.sin_ang : (T)P.fsin;
	const T ux = fabs(xp) / re, uy = fabs(yp) / re;
	const T lux = log(ux), luy = log(uy);
	const T ax = exp(B * lux), ay = exp(B * luy);
	const T base = ax + ay;
	const T lbase = log(base);
	const T rf = exp(lbase / (n * B));
	const T f = exp(-bn * (rf - (T)1));
	const T wf = weight * f;
	acc[G_V] += wf;
	if (!(base > (T)0)) {
		acc[G_X1] += wf * dbn;  // d/dn at the exact centre: rf = 0
		return;
	}
	const T A = -bn * rf;
	const T Dx = xp != (T)0 ? A * ax / (n * xp * base) : (T)0;
	const T Dy = yp != (T)0 ? A * ay / (n * yp * base) : (T)0;
	const T xl = ax > (T)0 ? ax * lux : (T)0, yl = ay > (T)0 ? ay * luy : (T)0;
	const T dB = A * ((xl + yl) / (n * B * base) - lbase / (n * B * B));
	const T deg = (T)(3.14159265358979323846 / 180.0);
	acc[G_XCEN] += wf * (-c * Dx + (s / q) * Dy);
	acc[G_YCEN] += wf * (-s * Dx - (c / q) * Dy);
	acc[G_ANG] += wf * deg * (q * yp * Dx - (xp / q) * Dy);
	acc[G_AXRAT] += wf * (-(yp / q) * Dy);
	acc[G_BOX] += wf * dB;
	acc[G_X0] += wf * (-A / (n * re));
	acc[G_X1] += wf * (A * (-lbase / (n * n * B)) - dbn * (rf - (T)1));
}

// ------------------------------------------------------------- backward eval

// A sub-pixel box as in eval_f32.cu: its corner relative to the profile
// centre as an unevaluated sum hi + lo in T (lo stays 0 in double), its size
// and its eight running totals.
template <typename T>
struct FrameG {
	T xhi, xlo, yhi, ylo, bx, by;
	T tot[kGradSlots];
	unsigned int mask[kMaskWords];
};

template <typename T>
struct WarpScratchG {
	FrameG<T> fr[kMaxLevels];
};

template <typename T>
__device__ __forceinline__ void two_sum_t(T a, T b, T &s, T &e)
{
	s = a + b;
	const T bb = s - a;
	e = (a - (s - bb)) + (b - bb);
}

// hi + lo = i * (s_hi + s_lo) - (c_hi + c_lo), the product formed error-free
__device__ __forceinline__ void corner_pair_b(float i, float s_hi, float s_lo, float c_hi, float c_lo, float &hi,
                                              float &lo)
{
	const float p = i * s_hi;
	const float ep = fmaf(i, s_hi, -p) + i * s_lo;
	float e;
	two_sum_t<float>(p, -c_hi, hi, e);
	lo = (e + ep) - c_lo;
}

template <typename T>
__device__ __forceinline__ T value_at(const ProfileDev &P, T xp, T yp)
{
	if constexpr (std::is_same<T, double>::value) return f64::evaluate_at(P, xp, yp);
	else return f32::evaluate_at(P, xp, yp);
}

__device__ __noinline__ bool test_f64b(const ProfileDev &P, double dx, double dy, double xbin, double ybin)
{
	const double xp = dx * P.cos_ang + dy * P.sin_ang;
	const double yp = (-dx * P.sin_ang + dy * P.cos_ang) / P.par[PF_P_AXRAT];
	const double sv = f64::evaluate_at(P, xp, yp);
	const double dyp = (-xbin * P.sin_ang + ybin * P.cos_ang) / P.par[PF_P_AXRAT];
	const double t = f64::evaluate_at(P, fabs(xp), fabs(yp) + fabs(dyp));
	return fabs(t / sv - 1.0) > P.acc;
}

template <typename T>
__device__ void eval_frame_g(const ProfileDev &P, WarpScratchG<T> &ws, int L, unsigned int res, T inv_res,
                             unsigned int max_rec, int lane)
{
	constexpr bool dbl = std::is_same<T, double>::value;
	FrameG<T> &f = ws.fr[L];
	const T xhi = f.xhi, xlo = f.xlo, yhi = f.yhi, ylo = f.ylo;
	const T txbin = f.bx * inv_res, tybin = f.by * inv_res;
	const bool recurse = res > 1 && (unsigned int)L < max_rec;
	const unsigned int n = res * res;
	const T c = dbl ? (T)P.cos_ang : (T)P.fcos, s = dbl ? (T)P.sin_ang : (T)P.fsin;
	const T iq = dbl ? (T)1 / (T)P.par[PF_P_AXRAT] : (T)P.finv_axrat;
	const T acc_t = dbl ? (T)P.acc : (T)P.facc;
	const T tdyp = fabs((-txbin * s + tybin * c) * iq);
	T part[kGradSlots];
#pragma unroll
	for (int k = 0; k < kGradSlots; k++) part[k] = 0;
	for (unsigned int base = 0; base < n; base += 32) {
		const unsigned int idx = base + lane;
		bool fail = false;
		if (idx < n) {
			const unsigned int i = div_res(idx, res_magic(res)), j = idx - i * res;
			const T ox = ((T)small_int_to_float(i) + (T)0.5) * txbin, oy = ((T)small_int_to_float(j) + (T)0.5) * tybin;
			const T dx = (xhi + ox) + xlo;
			const T dy = (yhi + oy) + ylo;
			const T xp = dx * c + dy * s;
			const T yp = (dy * c - dx * s) * iq;
			if (recurse) {
				const T sv = value_at<T>(P, xp, yp);
				const T t = value_at<T>(P, fabs(xp), fabs(yp) + tdyp);
				const T d = fabs(t / sv - (T)1);
				if (!dbl && (!(isfinite(d) && isfinite(sv)) || fabs(d - acc_t) <= (T)kGuardAccB * (acc_t + (T)1))) {
					fail = test_f64b(P, ((double)xhi + (double)xlo) + (double)ox,
					                 ((double)yhi + (double)ylo) + (double)oy, (double)txbin, (double)tybin);
				}
				else {
					fail = d > acc_t;
				}
			}
			if (!fail) sersic_grad<T>(P, xp, yp, (T)1, part);
		}
		const unsigned int word = __ballot_sync(0xffffffffu, fail);
		if (lane == 0) f.mask[base >> 5] = word;
	}
#pragma unroll
	for (int k = 0; k < kGradSlots; k++) part[k] = warp_sum_t(part[k]);
	if (lane == 0) {
		for (int k = 0; k < kGradSlots; k++) f.tot[k] = part[k];
	}
	__syncwarp();
}

template <typename T>
__device__ void warp_subsample_g(const ProfileDev &P, WarpScratchG<T> &ws, T xhi, T xlo, T yhi, T ylo, T bx, T by,
                                 unsigned int res, unsigned int max_rec, int lane, T *out)
{
	if (lane == 0) {
		ws.fr[0].xhi = xhi;
		ws.fr[0].xlo = xlo;
		ws.fr[0].yhi = yhi;
		ws.fr[0].ylo = ylo;
		ws.fr[0].bx = bx;
		ws.fr[0].by = by;
	}
	__syncwarp();
	const T inv_res = (T)1 / (T)res;
	const T inv_res2 = (T)1 / (T)(res * res);
	int L = 0;
	eval_frame_g<T>(P, ws, 0, res, inv_res, max_rec, lane);
	const unsigned int nwords = (res * res + 31) / 32;
	while (true) {
		FrameG<T> &f = ws.fr[L];
		int k = -1;
		for (unsigned int w = 0; w < nwords; w++) {
			const unsigned int mw = f.mask[w];
			if (mw) {
				k = (int)(w * 32 + __ffs(mw) - 1);
				break;
			}
		}
		__syncwarp();
		if (k >= 0) {
			if (lane == 0) {
				const unsigned int i = div_res((unsigned int)k, res_magic(res)), j = (unsigned int)k - i * res;
				const T cbx = f.bx * inv_res, cby = f.by * inv_res;
				f.mask[k >> 5] &= ~(1u << (k & 31));
				FrameG<T> &ch = ws.fr[L + 1];
				T e;
				two_sum_t<T>(f.xhi, (T)small_int_to_float(i) * cbx, ch.xhi, e);
				ch.xlo = f.xlo + e;
				two_sum_t<T>(f.yhi, (T)small_int_to_float(j) * cby, ch.yhi, e);
				ch.ylo = f.ylo + e;
				ch.bx = cbx;
				ch.by = cby;
			}
			__syncwarp();
			L++;
			eval_frame_g<T>(P, ws, L, res, inv_res, max_rec, lane);
		}
		else {
			if (L == 0) {
				for (int s = 0; s < kGradSlots; s++) out[s] = f.tot[s] * inv_res2;
				return;
			}
			L--;
			if (lane == 0) {
				for (int s = 0; s < kGradSlots; s++) ws.fr[L].tot[s] += f.tot[s] * inv_res2;
			}
			__syncwarp();
		}
	}
}

// One work item = one band of kBandRows drawing rows of one model. For each
// profile of the model, the warps share the band's 32-pixel tiles, the
// per-warp sums are reduced in a fixed order and written as FP64 partials.
template <typename T>
__global__ void __launch_bounds__(kWarpsB * 32)
backward_kernel(const ModelDev *__restrict__ models, int n_models, const ProfileDev *__restrict__ profs,
                const T *__restrict__ gout, const T *__restrict__ gsrc, const long long *__restrict__ band_base,
                const long long *__restrict__ part_base, long long n_items, double *__restrict__ partial)
{
	constexpr bool dbl = std::is_same<T, double>::value;
	__shared__ WarpScratchG<T> scratch[kWarpsB];
	__shared__ double red[kWarpsB][kGradSlots];
	__shared__ unsigned int tile_next;
	const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
	WarpScratchG<T> &ws = scratch[warp];
	for (long long item = blockIdx.x; item < n_items; item += gridDim.x) {
		int lo = 0, hi = n_models - 1;
		while (lo < hi) {
			int mid = (lo + hi + 1) >> 1;
			if (band_base[mid] <= item) lo = mid; else hi = mid - 1;
		}
		const ModelDev &m = models[lo];
		const int band = (int)(item - band_base[lo]);
		const int r0 = band * kBandRows, r1 = min(r0 + kBandRows, (int)m.draw_h);
		const int tiles_per_row = (int)m.tiles_per_row;
		for (int q = 0; q < m.n_profiles; q++) {
			const ProfileDev &P = profs[m.first_profile + q];
			double *dst = partial + part_base[lo] + ((long long)band * m.n_profiles + q) * kGradSlots;
			const bool is_radial = P.kind == PF_SERSIC;
			int br0 = r0, br1 = r1, bc0 = 0, bc1 = tiles_per_row;
			if (is_radial) {
				br0 = max(r0, P.bby0);
				br1 = min(r1, P.bby1 + 1);
				bc0 = max(0, P.bbx0 / 32);
				bc1 = min(tiles_per_row, P.bbx1 / 32 + 1);
			}
			const bool work = (P.kind == PF_SKY || is_radial) && br0 < br1 && bc0 < bc1;
			if (!work) {
				if (threadIdx.x < kGradSlots) dst[threadIdx.x] = 0.;
				continue;
			}
			if (threadIdx.x == 0) tile_next = 0;
			__syncthreads();
			const int ncols = bc1 - bc0;
			const unsigned int n_tiles = (unsigned int)((br1 - br0) * ncols);
			const T *gimg = P.convolve ? gsrc + m.draw_off : nullptr;
			T acc[kGradSlots];
#pragma unroll
			for (int k = 0; k < kGradSlots; k++) acc[k] = 0;
			while (true) {
				unsigned int t = 0;
				if (lane == 0) t = atomicAdd(&tile_next, 1u);
				t = __shfl_sync(0xffffffffu, t, 0);
				if (t >= n_tiles) break;
				const int trow = (int)(t / (unsigned int)ncols);
				const int tcol = bc0 + (int)(t - (unsigned int)(trow * ncols));
				const int row = br0 + trow;
				const int px = tcol * 32 + lane;
				const bool active = px < (int)m.draw_w;
				T g = 0;
				if (active) {
					g = gimg ? gimg[(size_t)row * m.draw_w + px] : g_direct(m, gout, px, row);
				}
				if (P.kind == PF_SKY) {
					acc[G_V] += g;
					continue;
				}
				// the forward pass's decisions for this pixel (eval_f32.cu / eval_f64.cu)
				T xp, yp;
				float fdx = 0.f, fdy = 0.f;
				bool beyond, outside;
				if (dbl) {
					const double x = m.sx / 2. + px * m.sx, y = m.sy / 2. + row * m.sy;
					double xp64, yp64;
					f64::to_profile(P, x, y, xp64, yp64);
					xp = (T)xp64;
					yp = (T)yp64;
					const double r64 = sqrt(xp64 * xp64 + yp64 * yp64);
					beyond = P.rscale_max > 0 && r64 / P.rscale > P.rscale_max;
					outside = r64 / P.rscale > P.rscale_switch;
				}
				else {
					const float cx = small_int_to_float(px) + 0.5f, cy = small_int_to_float(row) + 0.5f;
					const float xh = cx * m.fsx_hi, yh = cy * m.fsy_hi;
					const float xl = fmaf(cx, m.fsx_hi, -xh) + cx * m.fsx_lo;
					const float yl = fmaf(cy, m.fsy_hi, -yh) + cy * m.fsy_lo;
					const float dx = (xh - P.fxc_hi) + (xl - P.fxc_lo);
					const float dy = (yh - P.fyc_hi) + (yl - P.fyc_lo);
					fdx = dx;
					fdy = dy;
					xp = (T)(dx * P.fcos + dy * P.fsin);
					yp = (T)((dy * P.fcos - dx * P.fsin) * P.finv_axrat);
					const float rr = sqrtf((float)(xp * xp + yp * yp)) * P.finv_rscale;
					beyond = P.frmax > 0.f && rr > P.frmax;
					outside = rr > P.fswitch;
					const bool amb = (P.frmax > 0.f && fabsf(rr - P.frmax) <= kGuardRadiusB * P.frmax) ||
					                 fabsf(rr - P.fswitch) <= kGuardRadiusB * P.fswitch || !isfinite(rr);
					if (amb && active) {
						const double x = m.sx / 2. + px * m.sx, y = m.sy / 2. + row * m.sy;
						double xp64, yp64;
						f64::to_profile(P, x, y, xp64, yp64);
						const double r64 = sqrt(xp64 * xp64 + yp64 * yp64);
						beyond = P.rscale_max > 0 && r64 / P.rscale > P.rscale_max;
						outside = r64 / P.rscale > P.rscale_switch;
					}
				}
				bool need_ss = false;
				if (active && g != (T)0 && !beyond) {
					if (P.rough || outside) {
						T tmp[kGradSlots];
#pragma unroll
						for (int k = 0; k < kGradSlots; k++) tmp[k] = 0;
						sersic_grad<T>(P, xp, yp, (T)1, tmp);
#pragma unroll
						for (int k = 0; k < kGradSlots; k++) acc[k] += g * tmp[k];
					}
					else {
						need_ss = true;
					}
				}
				unsigned int pending = __ballot_sync(0xffffffffu, need_ss);
				while (pending) {
					const int src = __ffs(pending) - 1;
					pending &= pending - 1;
					const int spx = tcol * 32 + src;
					const float sdx = __shfl_sync(0xffffffffu, fdx, src);
					const float sdy = __shfl_sync(0xffffffffu, fdy, src);
					unsigned int res = P.resolution, max_rec = P.max_recursions;
					if (P.center_boost) {  // sersic central pixel (src/sersic.cpp:331-347)
						bool center;
						if (!dbl && fabsf(fabsf(sdx) - m.fscale_x) > 1e-5f * m.fscale_x &&
						    fabsf(fabsf(sdy) - m.fscale_y) > 1e-5f * m.fscale_y) {
							center = fabsf(sdx) < m.fscale_x && fabsf(sdy) < m.fscale_y;
						}
						else {
							const double x = m.sx / 2. + spx * m.sx, y = m.sy / 2. + row * m.sy;
							center = fabs(x - P.xc) < m.scale_x && fabs(y - P.yc) < m.scale_y;
						}
						if (center) {
							res = 8;
							max_rec = 10;
						}
					}
					if (res > (unsigned int)kMaxRes) res = kMaxRes;
					if (max_rec > (unsigned int)kMaxLevels - 1) max_rec = kMaxLevels - 1;
					T bxh, bxl, byh, byl;
					if constexpr (dbl) {
						bxh = (T)((double)spx * m.sx - P.xc);
						byh = (T)((double)row * m.sy - P.yc);
						bxl = byl = 0;
					}
					else {
						corner_pair_b(small_int_to_float(spx), m.fsx_hi, m.fsx_lo, P.fxc_hi, P.fxc_lo, bxh, bxl);
						corner_pair_b(small_int_to_float(row), m.fsy_hi, m.fsy_lo, P.fyc_hi, P.fyc_lo, byh, byl);
					}
					T sums[kGradSlots];
					warp_subsample_g<T>(P, ws, bxh, bxl, byh, byl, dbl ? (T)m.sx : (T)m.fsx_hi,
					                    dbl ? (T)m.sy : (T)m.fsy_hi, res, max_rec, lane, sums);
					const T gs = __shfl_sync(0xffffffffu, g, src);
					if (lane == 0) {
#pragma unroll
						for (int k = 0; k < kGradSlots; k++) acc[k] += gs * sums[k];
					}
				}
			}
#pragma unroll
			for (int k = 0; k < kGradSlots; k++) {
				const double v = warp_sum_t((double)acc[k]);
				if (lane == 0) red[warp][k] = v;
			}
			__syncthreads();
			if (threadIdx.x < kGradSlots) {
				double s = 0;
				for (int w = 0; w < kWarpsB; w++) s += red[w][threadIdx.x];
				dst[threadIdx.x] = s;
			}
			__syncthreads();
		}
	}
}

// d L / d par for every profile: partials summed over the model's bands in
// order, then scaled by the flux scale and its logarithmic derivatives.
__global__ void grad_reduce_kernel(const ModelDev *__restrict__ models, const ProfileDev *__restrict__ profs,
                                   int n_profiles, const long long *__restrict__ part_base,
                                   const double *__restrict__ partial, double *__restrict__ grad)
{
	const int i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= n_profiles) return;
	const ProfileDev &P = profs[i];
	const ModelDev &m = models[P.model];
	double *g = grad + (size_t)i * PF_NPAR;
	for (int k = 0; k < PF_NPAR; k++) g[k] = 0.;
	if (P.kind != PF_SERSIC && P.kind != PF_SKY) return;
	const int q = i - m.first_profile;
	const int n_bands = (m.draw_h + kBandRows - 1) / kBandRows;
	double S[kGradSlots];
	for (int k = 0; k < kGradSlots; k++) S[k] = 0.;
	for (int b = 0; b < n_bands; b++) {
		const double *src = partial + part_base[P.model] + ((long long)b * m.n_profiles + q) * kGradSlots;
		for (int k = 0; k < kGradSlots; k++) S[k] += src[k];
	}
	if (P.kind == PF_SKY) {
		g[6] = S[G_V] / (m.fs * m.fs);  // d/d bg of bg / fs^2 on every pixel (src/sky.cpp:42-45)
		return;
	}
	const double fs_ = P.flux_scale;
	g[PF_P_XCEN] = fs_ * S[G_XCEN];
	g[PF_P_YCEN] = fs_ * S[G_YCEN];
	g[PF_P_MAG] = fs_ * P.dlnfs[PF_P_MAG] * S[G_V];
	g[PF_P_ANG] = fs_ * S[G_ANG];
	g[PF_P_AXRAT] = fs_ * (S[G_AXRAT] + P.dlnfs[PF_P_AXRAT] * S[G_V]);
	g[PF_P_BOX] = fs_ * (S[G_BOX] + P.dlnfs[PF_P_BOX] * S[G_V]);
	g[6] = fs_ * (S[G_X0] + P.dlnfs[6] * S[G_V]);
	g[7] = fs_ * (S[G_X1] + P.dlnfs[7] * S[G_V]);
}

}  // namespace

int backward_band_rows() { return kBandRows; }

template <typename T>
void launch_chi2(const ModelDev *models, int n_models, const void *img, const void *data, const void *sigma,
                 const void *cot, void *gout, double *chi2, cudaStream_t stream)
{
	chi2_kernel<T><<<n_models, 256, 0, stream>>>(models, (const T *)img, (const T *)data, (const T *)sigma,
	                                             (const T *)cot, (T *)gout, chi2);
}


template <typename T>
void launch_backward(const ModelDev *models, int n_models, const ProfileDev *profs, int n_profiles, const void *gout,
                     const void *gsrc, const long long *band_base, const long long *part_base, long long n_items,
                     double *partial, double *grad, int n_sm, cudaStream_t stream)
{
	int blocks = (int)(n_items < (long long)n_sm * 8 ? n_items : (long long)n_sm * 8);
	if (blocks < 1) blocks = 1;
	backward_kernel<T><<<blocks, kWarpsB * 32, 0, stream>>>(models, n_models, profs, (const T *)gout,
	                                                        (const T *)gsrc, band_base, part_base, n_items, partial);
	grad_reduce_kernel<<<(n_profiles + 127) / 128, 128, 0, stream>>>(models, profs, n_profiles, part_base, partial,
	                                                                 grad);
}

template void launch_chi2<float>(const ModelDev *, int, const void *, const void *, const void *, const void *, void *,
                                 double *, cudaStream_t);
template void launch_chi2<double>(const ModelDev *, int, const void *, const void *, const void *, const void *,
                                  void *, double *, cudaStream_t);
template void launch_backward<float>(const ModelDev *, int, const ProfileDev *, int, const void *, const void *,
                                     const long long *, const long long *, long long, double *, double *, int,
                                     cudaStream_t);
template void launch_backward<double>(const ModelDev *, int, const ProfileDev *, int, const void *, const void *,
                                      const long long *, const long long *, long long, double *, double *, int,
                                      cudaStream_t);

}  // namespace pf
