// Batched single-precision path: FP32 profile values, FP64 where precision
// decides the result.
//
// Same structure as the plain FP64 path (eval_f64.cu): one warp per 32-pixel
// row tile of a model's drawing area, the model's profiles in order, and a
// warp-cooperative depth-first recursion for the pixels that
// RadialProfile::evaluate_cpu subsamples (src/radial.cpp:291-344,
// subsample_pixel src/radial.cpp:55-135). The differences:
//   * profile values are computed in FP32 (profiles_f32.cuh), coordinates
//     relative to the profile centre, the pixel centre formed with an
//     error-free float product so that it keeps full relative precision;
//   * each sub-pixel box is tracked in FP64 relative to the profile centre
//     (corner and bin), so that boxes 8^-11 pixel wide at the centre of a
//     high-index Sersic profile keep their geometry; the points inside a box
//     are FP32 offsets from its corner;
//   * every decision the reference takes by comparison -- the accuracy test
//     |testval/subval - 1| > acc, r/rscale > rscale_max, r/rscale >
//     rscale_switch, the sersic central-pixel test -- is re-taken in FP64
//     when the FP32 operands fall inside a guard band around the threshold or
//     are not finite, so the subsampling tree is the FP64 tree;
//   * box totals are warp reductions in FP32; the final images are FP32.
#include <cstdint>

#include "pf_device.cuh"
#include "profiles_f32.cuh"
#include "profiles_f64.cuh"
#include "psf_profile.cuh"

namespace pf {

namespace {

constexpr int kWarps32 = 8;
// Half-width of the band around a threshold inside which an FP32 comparison is
// re-taken in FP64. The FP32 profile values carry at most ~3e-6 relative
// error (the exp2 argument K (1 - rf) reaches ~40, ~2.4e-6 of rounding, plus
// the MUFU approximations), so |testval/subval - 1| is within 6e-6 (1 + d) of
// its FP64 value; the band is twice that. Radii carry a few 1e-7.
constexpr float kGuardAcc = 1.2e-5f;
constexpr float kGuardRadius = 2e-6f;

// A sub-pixel box: its corner relative to the profile centre as an
// unevaluated float sum (hi + lo), exact at the pixel level and updated with
// an error-free addition per level, so that boxes far below float resolution
// of the pixel coordinate keep their position; its size; its running total.
struct FrameM {
	float xhi, xlo, yhi, ylo;  // corner relative to the profile centre
	float bx, by;              // box size
	float total;               // sum of the accepted sub-point values, then children
	unsigned int mask[kMaskWords];
};

// s + e = a + b exactly (Knuth's two-sum)
__device__ __forceinline__ void two_sum(float a, float b, float &s, float &e)
{
	s = a + b;
	const float bb = s - a;
	e = (a - (s - bb)) + (b - bb);
}

// hi + lo = i * (s_hi + s_lo) - (c_hi + c_lo), the product formed error-free
__device__ __forceinline__ void corner_pair(float i, float s_hi, float s_lo, float c_hi, float c_lo, float &hi,
                                            float &lo)
{
	const float p = i * s_hi;
	const float ep = fmaf(i, s_hi, -p) + i * s_lo;
	float e;
	two_sum(p, -c_hi, hi, e);
	lo = (e + ep) - c_lo;
}

struct WarpScratchM {
	FrameM fr[kMaxLevels];
};

__device__ __forceinline__ float warp_sum(float v)
{
#pragma unroll
	for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
	return v;
}

// FP64 value and accuracy test of one sub-point (the rare re-taken decisions)
__device__ __noinline__ bool test_f64(const ProfileDev &P, double dx, double dy, double xbin, double ybin, float &subval)
{
	const double xp = dx * P.cos_ang + dy * P.sin_ang;
	const double yp = (-dx * P.sin_ang + dy * P.cos_ang) / P.par[PF_P_AXRAT];
	const double s = f64::evaluate_at(P, xp, yp);
	const double dyp = (-xbin * P.sin_ang + ybin * P.cos_ang) / P.par[PF_P_AXRAT];
	const double t = f64::evaluate_at(P, fabs(xp), fabs(yp) + fabs(dyp));
	subval = (float)s;
	return fabs(t / s - 1.0) > P.acc;
}

__device__ __noinline__ float value_f64(const ProfileDev &P, double dx, double dy)
{
	const double xp = dx * P.cos_ang + dy * P.sin_ang;
	const double yp = (-dx * P.sin_ang + dy * P.cos_ang) / P.par[PF_P_AXRAT];
	return (float)f64::evaluate_at(P, xp, yp);
}

__device__ void eval_frame_m(const ProfileDev &P, WarpScratchM &ws, int L, unsigned int res, float inv_res,
                             unsigned int max_rec, int lane, unsigned long long *counts)
{
	FrameM &f = ws.fr[L];
	const float xhi = f.xhi, xlo = f.xlo, yhi = f.yhi, ylo = f.ylo;
	const float fxbin = f.bx * inv_res, fybin = f.by * inv_res;
	const bool recurse = res > 1 && (unsigned int)L < max_rec;
	const unsigned int n = res * res;
	const float c = P.fcos, s = P.fsin, iq = P.finv_axrat;
	const float fdyp = fabsf((-fxbin * s + fybin * c) * iq);
	if (counts && lane == 0 && L < kLevelCounts) {
		atomicAdd(&counts[L], 1ull);
		atomicAdd(&counts[kCountSubEvals], (unsigned long long)(recurse ? 2 * n : n));
	}
	float part = 0.f;
	const unsigned int magic = res_magic(res);
	for (unsigned int base = 0; base < n; base += 32) {
		const unsigned int idx = base + lane;
		bool fail = false;
		if (idx < n) {
			const unsigned int i = div_res(idx, magic), j = idx - i * res;
			const float ox = (small_int_to_float(i) + 0.5f) * fxbin, oy = (small_int_to_float(j) + 0.5f) * fybin;
			const float dx = (xhi + ox) + xlo;
			const float dy = (yhi + oy) + ylo;
			const float xp = dx * c + dy * s;
			const float yp = (dy * c - dx * s) * iq;
			float sub = f32::evaluate_at(P, xp, yp);
			if (recurse) {
				const float t = f32::evaluate_at(P, fabsf(xp), fabsf(yp) + fdyp);
				const float d = fabsf(t / sub - 1.f);
				if (!(isfinite(d) && isfinite(sub)) || fabsf(d - P.facc) <= kGuardAcc * (P.facc + 1.f)) {
					// re-taken in FP64 (rare): the point from the exact corner
					fail = test_f64(P, ((double)xhi + (double)xlo) + (double)ox, ((double)yhi + (double)ylo) + (double)oy,
					                (double)fxbin, (double)fybin, sub);
				}
				else {
					fail = d > P.facc;
				}
			}
			else if (!isfinite(sub)) {
				sub = value_f64(P, ((double)xhi + (double)xlo) + (double)ox, ((double)yhi + (double)ylo) + (double)oy);
			}
			if (!fail) part += sub;
		}
		const unsigned int word = __ballot_sync(0xffffffffu, fail);
		if (lane == 0) f.mask[base >> 5] = word;
	}
	part = warp_sum(part);
	if (lane == 0) f.total = part;
	__syncwarp();
}

// subsample_pixel on a box given relative to the profile centre
__device__ float warp_subsample_m(const ProfileDev &P, WarpScratchM &ws, float xhi, float xlo, float yhi, float ylo,
                                  float bx, float by, unsigned int res, unsigned int max_rec, int lane,
                                  unsigned long long *counts, int &deepest)
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
	const float inv_res = __frcp_rn((float)res);
	const float inv_res2 = __frcp_rn((float)(res * res));
	int L = 0;
	deepest = 1;
	eval_frame_m(P, ws, 0, res, inv_res, max_rec, lane, counts);
	const unsigned int nwords = (res * res + 31) / 32;
	while (true) {
		FrameM &f = ws.fr[L];
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
				const float cbx = f.bx * inv_res, cby = f.by * inv_res;
				f.mask[k >> 5] &= ~(1u << (k & 31));
				FrameM &ch = ws.fr[L + 1];
				float e;
				two_sum(f.xhi, small_int_to_float(i) * cbx, ch.xhi, e);
				ch.xlo = f.xlo + e;
				two_sum(f.yhi, small_int_to_float(j) * cby, ch.yhi, e);
				ch.ylo = f.ylo + e;
				ch.bx = cbx;
				ch.by = cby;
			}
			__syncwarp();
			L++;
			if (L + 1 > deepest) deepest = L + 1;
			eval_frame_m(P, ws, L, res, inv_res, max_rec, lane, counts);
		}
		else {
			const float v = f.total * inv_res2;
			if (L == 0) {
				return v;
			}
			L--;
			if (lane == 0) ws.fr[L].total += v;
			__syncwarp();
		}
	}
}

__global__ void __launch_bounds__(kWarps32 * 32, 2)
eval_tiles32_kernel(const ModelDev *__restrict__ models, int n_models, const ProfileDev *__restrict__ profs,
                    const double *__restrict__ psf_pool, float *__restrict__ conv_img, float *__restrict__ direct_img,
                    long long n_tiles, unsigned int *tile_counter, DebugRec dbg)
{
	__shared__ WarpScratchM scratch[kWarps32];
	const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
	WarpScratchM &ws = scratch[warp];
	while (true) {
		unsigned int t = 0;
		if (lane == 0) t = atomicAdd(tile_counter, 1u);
		const long long tile = (long long)__shfl_sync(0xffffffffu, t, 0);
		if (tile >= n_tiles) break;
		const int mi = find_model(models, n_models, tile);
		const ModelDev &m = models[mi];
		const long long local = tile - m.tile_base;
		const unsigned int row = (unsigned int)local / m.tiles_per_row;
		const int col0 = (int)((unsigned int)local - row * m.tiles_per_row) * 32;
		const int col1 = min(col0 + 31, (int)m.draw_w - 1);
		const unsigned int px = (unsigned int)col0 + lane;
		const bool active = px < m.draw_w;
		const double *psf = m.psf_off >= 0 ? psf_pool + m.psf_off : nullptr;
		// pixel centre (i + 1/2) * scale as an unevaluated float sum
		const float cx = small_int_to_float(px) + 0.5f, cy = small_int_to_float(row) + 0.5f;
		const float xh = cx * m.fsx_hi, yh = cy * m.fsy_hi;
		const float xl = fmaf(cx, m.fsx_hi, -xh) + cx * m.fsx_lo;
		const float yl = fmaf(cy, m.fsy_hi, -yh) + cy * m.fsy_lo;
		float acc_conv = 0.f, acc_direct = 0.f;

		for (int q = 0; q < m.n_profiles; q++) {
			const int pi = m.first_profile + q;
			const ProfileDev &P = profs[pi];
			float add = 0.f;
			bool has = false;
			if (P.kind == PF_SKY) {
				add = P.fbg;
				has = active;
			}
			else if (P.kind == PF_PSF) {
				double v = 0;
				if (active && psf && psf_pixel64(P, m, psf, px, row, v)) {
					add = (float)v;
					has = true;
				}
			}
			else if (P.kind <= PF_BROKENEXP) {
				if ((int)row < P.bby0 || (int)row > P.bby1 || col1 < P.bbx0 || col0 > P.bbx1) {
					continue;
				}
				const float dx = (xh - P.fxc_hi) + (xl - P.fxc_lo);
				const float dy = (yh - P.fyc_hi) + (yl - P.fyc_lo);
				const float xp = dx * P.fcos + dy * P.fsin;
				const float yp = (dy * P.fcos - dx * P.fsin) * P.finv_axrat;
				const float rr = sqrtf(xp * xp + yp * yp) * P.finv_rscale;
				bool beyond = P.frmax > 0.f && rr > P.frmax;
				bool outside = rr > P.fswitch;
				const bool amb = (P.frmax > 0.f && fabsf(rr - P.frmax) <= kGuardRadius * P.frmax) ||
				                 fabsf(rr - P.fswitch) <= kGuardRadius * P.fswitch || !isfinite(rr);
				if (amb && active) {
					// the reference's r_prof, in FP64 (src/radial.cpp:313-326)
					const double x = m.sx / 2. + px * m.sx, y = m.sy / 2. + row * m.sy;
					double xp64, yp64;
					f64::to_profile(P, x, y, xp64, yp64);
					const double r64 = sqrt(xp64 * xp64 + yp64 * yp64);
					beyond = P.rscale_max > 0 && r64 / P.rscale > P.rscale_max;
					outside = r64 / P.rscale > P.rscale_switch;
				}
				float pixel_val = 0.f;
				int depth = 0;
				bool need_ss = false;
				if (beyond) {
					depth = -1;
				}
				else if (P.rough || outside) {
					pixel_val = f32::evaluate_at(P, xp, yp);
					if (!isfinite(pixel_val)) pixel_val = value_f64(P, (double)dx, (double)dy);
				}
				else {
					need_ss = true;
				}
				unsigned int pending = __ballot_sync(0xffffffffu, need_ss && active);
				unsigned long long *counts = dbg.counts ? dbg.counts + (size_t)pi * kLevelCounts : nullptr;
				if (counts) {
					const unsigned int nd = __popc(__ballot_sync(0xffffffffu, active && !beyond && !need_ss));
					if (lane == 0 && nd) atomicAdd(&counts[kCountDirectEvals], (unsigned long long)nd);
				}
				while (pending) {
					const int src = __ffs(pending) - 1;
					pending &= pending - 1;
					const unsigned int spx = (unsigned int)col0 + src;
					const float sdx = __shfl_sync(0xffffffffu, dx, src);
					const float sdy = __shfl_sync(0xffffffffu, dy, src);
					unsigned int res = P.resolution, max_rec = P.max_recursions;
					if (P.center_boost) {  // src/sersic.cpp:331-347
						bool center = fabsf(sdx) < m.fscale_x && fabsf(sdy) < m.fscale_y;
						if (fabsf(fabsf(sdx) - m.fscale_x) <= 1e-5f * m.fscale_x ||
						    fabsf(fabsf(sdy) - m.fscale_y) <= 1e-5f * m.fscale_y) {
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
					// pixel box corner (i * scale - centre) as an exact float pair
					float bxh, bxl, byh, byl;
					corner_pair(small_int_to_float(spx), m.fsx_hi, m.fsx_lo, P.fxc_hi, P.fxc_lo, bxh, bxl);
					corner_pair(small_int_to_float(row), m.fsy_hi, m.fsy_lo, P.fyc_hi, P.fyc_lo, byh, byl);
					int deepest = 0;
					const float v = warp_subsample_m(P, ws, bxh, bxl, byh, byl, m.fsx_hi, m.fsy_hi, res, max_rec, lane,
					                                 counts, deepest);
					if (lane == src) {
						pixel_val = v;
						depth = deepest;
					}
				}
				if (dbg.depth && active) {
					dbg.depth[P.depth_off + (size_t)row * m.draw_w + px] = (int8_t)depth;
				}
				add = P.fflux_scale * pixel_val;
				has = active;
			}
			if (has) {
				if (P.convolve) acc_conv += add;
				else acc_direct += add;
			}
		}
		if (active) {
			const size_t idx = (size_t)m.draw_off + (size_t)row * m.draw_w + px;
			if (m.conv_required) conv_img[idx] = acc_conv;
			direct_img[idx] = acc_direct;
		}
	}
}

__global__ void psf_to_float_kernel(const double *in, float *out, long long n)
{
	for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
		out[i] = (float)in[i];
}

}  // namespace

void launch_eval32(const ModelDev *models, int n_models, const ProfileDev *profs, const double *psf_pool,
                   float *conv_img, float *direct_img, long long n_tiles, unsigned int *tile_counter, DebugRec dbg,
                   int n_sm, cudaStream_t stream)
{
	int blocks = n_sm * 4;
	long long need = (n_tiles + kWarps32 - 1) / kWarps32;
	if (need < blocks) blocks = (int)(need > 0 ? need : 1);
	eval_tiles32_kernel<<<blocks, kWarps32 * 32, 0, stream>>>(models, n_models, profs, psf_pool, conv_img, direct_img,
	                                                          n_tiles, tile_counter, dbg);
}

void launch_psf_to_float(const double *in, float *out, long long n, cudaStream_t stream)
{
	if (n <= 0) return;
	psf_to_float_kernel<<<(int)((n + 255) / 256 < 4096 ? (n + 255) / 256 : 4096), 256, 0, stream>>>(in, out, n);
}

}  // namespace pf
