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
// Per (profile, row) partial sums are written in FP64 and reduced in a fixed
// order, so gradients and chi^2 are deterministic.
//
// Profiles supported by the adjoint: the six radial profiles with all their
// parameters (xcen, ycen, mag, ang, axrat, box and the profile's own: sersic
// re, nser (rescale_flux included); coresersic re, nser, rb, a, b; moffat fwhm,
// con; ferrer rout, a, b; king rc, rt, a; brokenexp h1, h2, rb, a) and sky
// (bg). A batch whose radial profiles are all sersics runs kernels with eight
// gradient slots per partial (value, five geometric, re, nser); any other
// batch runs the same kernels with twelve (value, five geometric, par[6..11]),
// the other kinds' terms coming from profiles_grad.cuh. The psf profile
// (point source, src/psf.cpp:58-145): xcen, ycen (its stamp's overlaps are
// piecewise linear in the centre) and mag.
#include <cstdint>
#include <type_traits>

#include "pf_device.cuh"
#include "profiles_f32.cuh"
#include "profiles_f64.cuh"
#include "profiles_grad.cuh"
#include "psf_profile.cuh"

namespace pf {

namespace {

// Warps per block and blocks per SM of the backward pass's register budget
// (4 and 4: 128 registers, 16 warps per SM; the kernel is latency-bound:
// 2.99 ms on the 1024-model step against 3.21 ms at 12 warps and 166
// registers without spills).
#ifndef PF_BACKWARD_WARPS
#define PF_BACKWARD_WARPS 4
#endif
#ifndef PF_BACKWARD_MIN_BLOCKS
#define PF_BACKWARD_MIN_BLOCKS 4
#endif
// phase-A (ring tile) items a warp claims at once (a divisor of 32): 8
// measured best on the 1024-model step (backward 2.57 ms, against 2.87 at 32
// and 2.68 at 2)
#ifndef PF_BACKWARD_RING_CHUNK
#define PF_BACKWARD_RING_CHUNK 8
#endif
constexpr int kWarpsB = PF_BACKWARD_WARPS;
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

// Sums v[0..7] over the warp by a transposed butterfly: at each of the first
// three steps a lane keeps half of its slots and receives its partner's other
// half, so 8 slots cost 9 shuffles and 9 additions instead of 40 each. Returns,
// in every lane, the total of slot (lane >> 2) & 7. The order of the
// additions is fixed: the result is deterministic.
template <typename T>
__device__ __forceinline__ T warp_sum8(const T *v, int lane)
{
	const bool b4 = (lane & 16) != 0, b3 = (lane & 8) != 0, b2 = (lane & 4) != 0;
	T w[4], u[2];
#pragma unroll
	for (int j = 0; j < 4; j++) {
		const T send = b4 ? v[j] : v[j + 4];
		const T keep = b4 ? v[j + 4] : v[j];
		w[j] = keep + __shfl_xor_sync(0xffffffffu, send, 16);
	}
#pragma unroll
	for (int j = 0; j < 2; j++) {
		const T send = b3 ? w[j] : w[j + 2];
		const T keep = b3 ? w[j + 2] : w[j];
		u[j] = keep + __shfl_xor_sync(0xffffffffu, send, 8);
	}
	T t = (b2 ? u[1] : u[0]) + __shfl_xor_sync(0xffffffffu, b2 ? u[0] : u[1], 4);
	t += __shfl_xor_sync(0xffffffffu, t, 2);
	t += __shfl_xor_sync(0xffffffffu, t, 1);
	return t;
}

// Gradient slots per partial of a kernel built for the profile kinds KINDS.
template <unsigned int KINDS>
__host__ __device__ constexpr int slots_of()
{
	return KINDS == f32::kSersicOnly ? (int)kGradSlots : grad::kSlots;
}

__host__ __device__ constexpr bool is_radial_kind(int kind) { return kind >= PF_SERSIC && kind <= PF_BROKENEXP; }

// Sums v[0..NS-1] over the warp (NS = 8 or 12, warp_sum8 once or twice) and
// stores the totals to dst[0..NS-1] from the lanes that hold them.
template <int NS, typename T, typename D>
__device__ __forceinline__ void warp_store_slots(const T *v, int lane, D *dst)
{
	const T lo = warp_sum8(v, lane);
	if constexpr (NS == 8) {
		if ((lane & 3) == 0) dst[lane >> 2] = (D)lo;
	}
	else {
		static_assert(NS > 8 && NS <= 16, "two passes of eight slots");
		T rest[8];
#pragma unroll
		for (int k = 0; k < 8; k++) rest[k] = 8 + k < NS ? v[8 + k] : (T)0;
		const T hi = warp_sum8(rest, lane);
		if ((lane & 3) == 0) {
			dst[lane >> 2] = (D)lo;
			if ((lane >> 2) < NS - 8) dst[8 + (lane >> 2)] = (D)hi;
		}
	}
}

// ------------------------------------------------------------ chi^2, g_out

// Block (model, c) of gridDim.y = `parts` blocks per model takes the model's
// output pixels [c * chunk, (c + 1) * chunk), chunk a multiple of 4. With one
// block per model it writes chi2[model] itself; with several, each writes its
// FP64 partial and the last block of the model to finish (a per-model counter,
// reset by that block) adds the partials in block order, so the result does
// not depend on the blocks' timing. `vec`: every buffer starts on a 16-byte
// boundary, so that single-precision models whose pixels do too (and that have
// no final mask) are read and written four pixels at a time (16-byte
// accesses: twice the bytes in flight of one pixel per thread, which left the
// pass at about 3 TB/s).
template <typename T>
__global__ void chi2_kernel(const ModelDev *__restrict__ models, const T *__restrict__ img, const T *__restrict__ data,
                            const T *__restrict__ sigma, const T *__restrict__ cot, T *__restrict__ gout,
                            double *__restrict__ chi2, double *__restrict__ partial, unsigned int *__restrict__ done,
                            bool vec)
{
	const ModelDev &m = models[blockIdx.x];
	const long long n = (long long)m.out_w * m.out_h;
	const int parts = gridDim.y;
	const long long chunk = ((n + parts - 1) / parts + 3) & ~3ll;
	const long long i0 = min(n, (long long)blockIdx.y * chunk), i1 = min(n, i0 + chunk);
	// per thread: a compensated (Kahan) sum in T, so that single precision
	// costs no FP64 work per pixel; across threads: FP64
	T s = 0, comp = 0;
	long long first = i0;  // the pixels from here on go one at a time
	if constexpr (std::is_same<T, float>::value) {
		if (vec && !cot && !m.mask_final && (m.out_off & 3) == 0) {
			const long long nq = (i1 - i0) >> 2;
			const long long g0 = (m.out_off + i0) >> 2;
			const float4 *img4 = reinterpret_cast<const float4 *>(img) + g0;
			const float4 *data4 = reinterpret_cast<const float4 *>(data) + g0;
			const float4 *sig4 = sigma ? reinterpret_cast<const float4 *>(sigma) + g0 : nullptr;
			float4 *gout4 = reinterpret_cast<float4 *>(gout) + g0;
			for (long long q = threadIdx.x; q < nq; q += blockDim.x) {
				const float4 a = img4[q], d = data4[q];
				const float4 sg = sig4 ? sig4[q] : make_float4(1.f, 1.f, 1.f, 1.f);
				const float av[4] = {a.x, a.y, a.z, a.w}, dv[4] = {d.x, d.y, d.z, d.w};
				const float sv[4] = {sg.x, sg.y, sg.z, sg.w};
				float gv[4];
#pragma unroll
				for (int k = 0; k < 4; k++) {
					const float r = av[k] - dv[k];
					const float wr = (sig4 ? 1.f / (sv[k] * sv[k]) : 1.f) * r;
					const float y = wr * r - comp;
					const float t = s + y;
					comp = (t - s) - y;
					s = t;
					gv[k] = 2.f * wr;
				}
				gout4[q] = make_float4(gv[0], gv[1], gv[2], gv[3]);
			}
			first = i0 + 4 * nq;
		}
	}
	for (long long i = first + threadIdx.x; i < i1; i += blockDim.x) {
		const long long g = m.out_off + i;
		// output pixels the final masking zeroes do not depend on the parameters
		const bool live = !m.mask_final || kept(m, (int)(i % m.out_w), (int)(i / m.out_w));
		if (cot) {
			gout[g] = live ? cot[g] : (T)0;
		}
		else {
			const T r = img[g] - data[g];
			const T w = sigma ? (T)1 / (sigma[g] * sigma[g]) : (T)1;
			const T wr = w * r;
			const T y = wr * r - comp;
			const T t = s + y;
			comp = (t - s) - y;
			s = t;
			gout[g] = live ? (T)2 * wr : (T)0;
		}
	}
	__shared__ double part[256];
	part[threadIdx.x] = (double)s - (double)comp;
	__syncthreads();
	for (int w = blockDim.x / 2; w > 0; w >>= 1) {
		if ((int)threadIdx.x < w) part[threadIdx.x] += part[threadIdx.x + w];
		__syncthreads();
	}
	if (threadIdx.x != 0 || !chi2) return;
	if (parts == 1) {
		chi2[blockIdx.x] = cot ? 0. : part[0];
		return;
	}
	partial[(size_t)blockIdx.x * parts + blockIdx.y] = part[0];
	__threadfence();
	if (atomicAdd(&done[blockIdx.x], 1u) + 1 != (unsigned int)parts) return;
	__threadfence();
	double total = 0.;
	const volatile double *pp = partial + (size_t)blockIdx.x * parts;
	for (int c = 0; c < parts; c++) total += pp[c];
	chi2[blockIdx.x] = cot ? 0. : total;
	done[blockIdx.x] = 0;
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

// FP32 sersic value and f * (1, d ln f / d theta) at profile coordinates
// (xp, yp), into t[]: the quantities of sersic_grad<float>, from one chain of
// base-2 logarithms and powers (special-function unit) shared by the value and
// every derivative. Returns f.
__device__ __forceinline__ float sersic_terms_f(const f32::Shape &P, float xp, float yp, float *t)
{
	constexpr float kLn2 = 0.6931471805599453f;
	constexpr float kDeg = 0.017453292519943295f;
	const float *c = P.c;
	const float inv_re = c[FP_S_INV_RE];
	const float ux = fabsf(xp) * inv_re, uy = fabsf(yp) * inv_re;
	const float lx = f32::lg2(ux), ly = f32::lg2(uy);  // -inf at 0
	float axm, aym;                                     // u^(B - 1)
	if (!P.boxy) {
		axm = ux;
		aym = uy;
	}
	else {
		const float bm1 = c[FP_B] - 1.f;
		axm = f32::ex2(bm1 * lx);
		aym = f32::ex2(bm1 * ly);
	}
	const float ax = axm * ux, ay = aym * uy;          // u^B
	const float base = ax + ay;
	const float lb = f32::lg2(base);
	const float inv_nb = c[FP_S_INV_NB];
	const float rf = f32::ex2(lb * inv_nb);             // base^(1 / (n B))
	const float K = c[FP_S_K];
	const float f = f32::ex2(K - K * rf);              // exp(-bn (rf - 1))
	t[G_V] = f;
	if (!(base > 0.f)) {  // the exact centre: rf = 0
#pragma unroll
		for (int k = 1; k < kGradSlots; k++) t[k] = 0.f;
		t[G_X1] = f * P.dbn;
		return f;
	}
	const float inv_n = 2.f * c[FP_S_HALF_INV_N];
	const float A = -P.bn * rf;
	const float inv_base = __fdividef(1.f, base);
	const float anb = A * inv_n * inv_base;
	const float dx = anb * copysignf(axm * inv_re, xp);  // A ax / (n xp base)
	const float dy = anb * copysignf(aym * inv_re, yp);
	const float lbase = lb * kLn2;
	const float xl = ax > 0.f ? ax * lx * kLn2 : 0.f, yl = ay > 0.f ? ay * ly * kLn2 : 0.f;
	const float db = A * inv_nb * ((xl + yl) * inv_base - lbase * c[FP_INVB]);
	const float cs = P.cs, sn = P.sn, iq = P.iq;
	const float q = __fdividef(1.f, iq);
	t[G_XCEN] = f * (-cs * dx + (sn * iq) * dy);
	t[G_YCEN] = f * (-sn * dx - (cs * iq) * dy);
	t[G_ANG] = f * kDeg * (q * yp * dx - (xp * iq) * dy);
	t[G_AXRAT] = f * (-(yp * iq) * dy);
	t[G_BOX] = f * db;
	t[G_X0] = f * (-A * inv_n * inv_re);
	t[G_X1] = f * (A * (-lbase * inv_n * inv_nb) - P.dbn * (rf - 1.f));
	return f;
}

// A sub-pixel box as in eval_f32.cu: its corner relative to the profile
// centre as an unevaluated sum hi + lo in T (lo stays 0 in double), its size
// and its eight running totals.
template <typename T, int NS>
struct FrameG {
	T xhi, xlo, yhi, ylo, bx, by;
	T tot[NS];
	unsigned int mask[kMaskWords];
};

template <typename T, int NS>
struct WarpScratchG {
	FrameG<T, NS> fr[kMaxLevels];
	unsigned int amb[kMaskWords];  // sub-points of the frame being evaluated whose decision is re-taken in FP64
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

// The FP32 path's rare FP64 re-takes. They take only single-precision and
// integer arguments, so that no double-precision work is scheduled on the
// common path. The one of the subsampling recursion is inlined (a call there
// costs the whole kernel registers).

// accuracy test of one sub-point, the point (xhi + xlo) + ox, (yhi + ylo) + oy
template <unsigned int KINDS>
__device__ __forceinline__ bool test_f64b(const ProfileDev &P, float xhi, float xlo, float yhi, float ylo, float ox,
                                       float oy, float xbin, float ybin)
{
	const double dx = ((double)xhi + (double)xlo) + (double)ox;
	const double dy = ((double)yhi + (double)ylo) + (double)oy;
	const double xp = dx * P.cos_ang + dy * P.sin_ang;
	const double yp = (-dx * P.sin_ang + dy * P.cos_ang) / P.par[PF_P_AXRAT];
	const double dyp = (-(double)xbin * P.sin_ang + (double)ybin * P.cos_ang) / P.par[PF_P_AXRAT];
	double sv, t;
	if constexpr (KINDS == f32::kSersicOnly) {
		sv = f64::sersic(P, xp, yp);
		t = f64::sersic(P, fabs(xp), fabs(yp) + fabs(dyp));
	}
	else {
		sv = f64::evaluate_at(P, xp, yp);
		t = f64::evaluate_at(P, fabs(xp), fabs(yp) + fabs(dyp));
	}
	return fabs(t / sv - 1.0) > P.acc;
}

// the reference's r_prof decisions for drawing pixel (px, row)
// (src/radial.cpp:313-326): bit 0 beyond rscale_max, bit 1 beyond rscale_switch
__device__ __noinline__ unsigned int radius_f64(const ProfileDev &P, const ModelDev &m, int px, int row)
{
	const double x = m.sx / 2. + px * m.sx, y = m.sy / 2. + row * m.sy;
	double xp, yp;
	f64::to_profile(P, x, y, xp, yp);
	const double r = sqrt(xp * xp + yp * yp);
	return (P.rscale_max > 0 && r / P.rscale > P.rscale_max ? 1u : 0u) | (r / P.rscale > P.rscale_switch ? 2u : 0u);
}

// the sersic central-pixel test (src/sersic.cpp:331-347)
__device__ __noinline__ bool center_f64(const ProfileDev &P, const ModelDev &m, int px, int row)
{
	const double x = m.sx / 2. + px * m.sx, y = m.sy / 2. + row * m.sy;
	return fabs(x - P.xc) < m.scale_x && fabs(y - P.yc) < m.scale_y;
}

// The value and gradient terms of one point for a kernel built for KINDS:
// t[0..slots_of<KINDS>() - 1]. Returns the value.
template <typename T, unsigned int KINDS>
__device__ __forceinline__ T point_terms(const ProfileDev &P, const f32::Shape &sh, const grad::GShape<T> &gs, T xp,
                                         T yp, T *t)
{
	constexpr bool dbl = std::is_same<T, double>::value;
	constexpr int NS = slots_of<KINDS>();
	if constexpr (KINDS != f32::kSersicOnly) {
		if (P.kind != PF_SERSIC) return grad::terms<T>(gs, xp, yp, t);
	}
	if constexpr (NS > kGradSlots) {
#pragma unroll
		for (int k = kGradSlots; k < NS; k++) t[k] = (T)0;
	}
	if constexpr (dbl) {
#pragma unroll
		for (int k = 0; k < kGradSlots; k++) t[k] = (T)0;
		sersic_grad<T>(P, xp, yp, (T)1, t);
		return t[G_V];
	}
	else {
		return sersic_terms_f(sh, xp, yp, t);
	}
}

template <typename T, unsigned int KINDS>
__device__ void eval_frame_g(const ProfileDev &P, const f32::Shape &sh, const grad::GShape<T> &gs,
                             WarpScratchG<T, slots_of<KINDS>()> &ws, int L, unsigned int res, T inv_res,
                             unsigned int max_rec, int lane)
{
	constexpr bool dbl = std::is_same<T, double>::value;
	constexpr int NS = slots_of<KINDS>();
	FrameG<T, NS> &f = ws.fr[L];
	const T xhi = f.xhi, xlo = f.xlo, yhi = f.yhi, ylo = f.ylo;
	const T txbin = f.bx * inv_res, tybin = f.by * inv_res;
	const bool recurse = res > 1 && (unsigned int)L < max_rec;
	const unsigned int n = res * res;
	const T c = dbl ? (T)P.cos_ang : (T)sh.cs, s = dbl ? (T)P.sin_ang : (T)sh.sn;
	const T iq = dbl ? (T)1 / (T)P.par[PF_P_AXRAT] : (T)sh.iq;
	const T acc_t = dbl ? (T)P.acc : (T)sh.acc;
	const T tdyp = fabs((-txbin * s + tybin * c) * iq);
	const unsigned int magic = res_magic(res);
	T part[NS];
#pragma unroll
	for (int k = 0; k < NS; k++) part[k] = 0;
	unsigned int amb_any = 0;
	for (unsigned int base = 0; base < n; base += 32) {
		const unsigned int idx = base + lane;
		bool fail = false, amb = false;
		if (idx < n) {
			const unsigned int i = div_res(idx, magic), j = idx - i * res;
			const T ox = ((T)small_int_to_float(i) + (T)0.5) * txbin, oy = ((T)small_int_to_float(j) + (T)0.5) * tybin;
			const T dx = (xhi + ox) + xlo;
			const T dy = (yhi + oy) + ylo;
			const T xp = dx * c + dy * s;
			const T yp = (dy * c - dx * s) * iq;
			if constexpr (dbl) {
				if (recurse) {
					const T sv = f64::evaluate_at(P, xp, yp);
					const T t = f64::evaluate_at(P, fabs(xp), fabs(yp) + tdyp);
					fail = fabs(t / sv - (T)1) > acc_t;
				}
				if (!fail) {
					T terms[NS];
					point_terms<T, KINDS>(P, sh, gs, xp, yp, terms);
#pragma unroll
					for (int k = 0; k < NS; k++) part[k] += terms[k];
				}
			}
			else if constexpr (KINDS == f32::kSersicOnly) {
				float terms[kGradSlots];
				const float sv = sersic_terms_f(sh, xp, yp, terms);
				if (recurse) {
					const float t = f32::value<f32::kSersicOnly>(sh, fabsf(xp), fabsf(yp) + tdyp);
					const float d = fabsf(__fdividef(t, sv) - 1.f);
					amb = !(isfinite(d) && isfinite(sv)) || fabsf(d - acc_t) <= kGuardAccB * (acc_t + 1.f);
					fail = !amb && d > acc_t;
				}
				if (!fail && !amb) {
#pragma unroll
					for (int k = 0; k < kGradSlots; k++) part[k] += terms[k];
				}
			}
			else {
				// the forward pass's decision from its own values, then the terms
				if (recurse) {
					const float sv = f32::value<KINDS>(sh, xp, yp);
					const float t = f32::value<KINDS>(sh, fabsf(xp), fabsf(yp) + tdyp);
					const float d = fabsf(__fdividef(t, sv) - 1.f);
					amb = !(isfinite(d) && isfinite(sv)) || fabsf(d - acc_t) <= kGuardAccB * (acc_t + 1.f);
					fail = !amb && d > acc_t;
				}
				if (!fail && !amb) {
					float terms[NS];
					point_terms<float, KINDS>(P, sh, gs, xp, yp, terms);
#pragma unroll
					for (int k = 0; k < NS; k++) part[k] += terms[k];
				}
			}
		}
		const unsigned int word = __ballot_sync(0xffffffffu, fail);
		const unsigned int aword = __ballot_sync(0xffffffffu, amb);
		if (lane == 0) {
			f.mask[base >> 5] = word;
			ws.amb[base >> 5] = aword;
		}
		amb_any |= aword;
	}
	if constexpr (!dbl) {
		if (amb_any) {
			// the ambiguous sub-points, re-taken in FP64 (rare) from the exact
			// corner, outside the loop above so that little state is live here
			__syncwarp();
			for (unsigned int base = 0; base < n; base += 32) {
				const unsigned int aword = ws.amb[base >> 5];
				if (!aword) continue;
				bool fail = false;
				if ((aword >> lane) & 1u) {
					const unsigned int idx = base + lane;
					const unsigned int i = div_res(idx, magic), j = idx - i * res;
					const float ox = (small_int_to_float(i) + 0.5f) * txbin, oy = (small_int_to_float(j) + 0.5f) * tybin;
					fail = test_f64b<KINDS>(P, xhi, xlo, yhi, ylo, ox, oy, txbin, tybin);
					if (!fail) {
						const float dx = (xhi + ox) + xlo;
						const float dy = (yhi + oy) + ylo;
						float terms[NS];
						point_terms<float, KINDS>(P, sh, gs, dx * c + dy * s, (dy * c - dx * s) * iq, terms);
#pragma unroll
						for (int k = 0; k < NS; k++) part[k] += terms[k];
					}
				}
				const unsigned int word = __ballot_sync(0xffffffffu, fail);
				if (lane == 0) f.mask[base >> 5] |= word;
			}
		}
	}
	warp_store_slots<NS>(part, lane, f.tot);
	__syncwarp();
}

template <typename T, unsigned int KINDS>
__device__ void warp_subsample_g(const ProfileDev &P, const f32::Shape &sh, const grad::GShape<T> &gs,
                                 WarpScratchG<T, slots_of<KINDS>()> &ws, T xhi, T xlo, T yhi, T ylo, T bx, T by,
                                 unsigned int res, unsigned int max_rec, int lane, T *out)
{
	constexpr int NS = slots_of<KINDS>();
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
	eval_frame_g<T, KINDS>(P, sh, gs, ws, 0, res, inv_res, max_rec, lane);
	const unsigned int nwords = (res * res + 31) / 32;
	while (true) {
		FrameG<T, NS> &f = ws.fr[L];
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
				FrameG<T, NS> &ch = ws.fr[L + 1];
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
			eval_frame_g<T, KINDS>(P, sh, gs, ws, L, res, inv_res, max_rec, lane);
		}
		else {
			if (L == 0) {
				for (int s = 0; s < NS; s++) out[s] = f.tot[s] * inv_res2;
				return;
			}
			L--;
			if (lane == 0) {
				for (int s = 0; s < NS; s++) ws.fr[L].tot[s] += f.tot[s] * inv_res2;
			}
			__syncwarp();
		}
	}
}

// Row items. Item k of the backward pass is row ring(k / n_profiles) of
// profile k % n_profiles, ring(l) = centre row, centre row - 1, centre row + 1,
// centre row - 2, ... of the profile's bounding box: every profile's central
// rows (its subsampled pixels, the costly ones) come first, so that the
// longest items start early and the tail of the pass is made of short ones.
// Returns the drawing row of the item, or -1 if it has none.
__device__ __forceinline__ int item_row(const ProfileDev &P, const ModelDev &m, int l)
{
	int lo, hi, centre;
	if (P.kind == PF_SKY) {
		lo = 0;
		hi = (int)m.draw_h - 1;
		centre = hi / 2;
	}
	else if (is_radial_kind(P.kind)) {
		lo = max(0, P.bby0);
		hi = min((int)m.draw_h - 1, P.bby1);
		centre = (int)floorf(__fdividef(P.fyc_hi, m.fsy_hi));
		centre = min(max(centre, lo), max(lo, hi));
	}
	else if (P.kind == PF_PSF && m.psf_off >= 0) {
		int x0, x1;
		psf_stamp(P, m, x0, x1, lo, hi);
		centre = (lo + hi) / 2;
	}
	else {
		return -1;
	}
	const int half = (l + 1) >> 1;
	const int row = (l & 1) ? centre - half : centre + half;
	return row >= lo && row <= hi ? row : -1;
}

// Tiles [c0, c1] of drawing row `row` of one profile, except tiles [s0, s1]:
// the cotangent-weighted value and shape derivatives of the profile summed
// over their pixels, written as one FP64 partial (slots_of<KINDS>() slots) to dst.
template <typename T, unsigned int KINDS>
__device__ void backward_row(const ModelDev &m, const ProfileDev &P, int row, int c0, int c1, int s0, int s1,
                             const T *__restrict__ gout, const T *__restrict__ gsrc,
                             const double *__restrict__ psf_pool, WarpScratchG<T, slots_of<KINDS>()> &ws, int lane,
                             double *dst)
{
	constexpr bool dbl = std::is_same<T, double>::value;
	constexpr int NS = slots_of<KINDS>();
	const bool is_sky = P.kind == PF_SKY;
	const bool is_psf = P.kind == PF_PSF;
	const T *gimg = P.convolve ? gsrc + m.draw_off : nullptr;
	const f32::Shape sh = f32::load_shape(P);
	grad::GShape<T> gs;
	if constexpr (KINDS != f32::kSersicOnly) {
		if (!is_sky) gs = grad::make_gshape<T>(P);
	}
	T acc[NS];
#pragma unroll
	for (int k = 0; k < NS; k++) acc[k] = 0;
	for (int tcol = c0; tcol <= c1; tcol++) {
		if (tcol >= s0 && tcol <= s1) continue;
		const int px = tcol * 32 + lane;
		// masked drawing pixels were not evaluated: no gradient from them (the
		// psf profile is drawn whatever the mask, src/psf.cpp:58-145)
		const bool active = px < (int)m.draw_w && (is_psf || evaluated(m, px, row));
		T g = 0;
		if (active) {
			g = gimg ? gimg[(size_t)row * m.draw_w + px] : g_direct(m, gout, px, row);
		}
		if (is_sky) {
			acc[G_V] += g;
			continue;
		}
		if (is_psf) {
			double v, dvx, dvy;
			if (active && g != (T)0 &&
			    psf_pixel_grad64(P, m, psf_pool + m.psf_off, (unsigned int)px, (unsigned int)row, v, dvx, dvy)) {
				acc[G_V] += g * (T)v;
				acc[G_XCEN] += g * (T)dvx;
				acc[G_YCEN] += g * (T)dvy;
			}
			continue;
		}
		// the forward pass's decisions for this pixel (eval_f32.cu / eval_f64.cu)
		T xp, yp;
		float fdx = 0.f, fdy = 0.f;
		bool beyond, outside;
		if constexpr (dbl) {
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
			const float cx = small_int_to_float((unsigned int)px) + 0.5f;
			const float cy = small_int_to_float((unsigned int)row) + 0.5f;
			const float xh = cx * m.fsx_hi, yh = cy * m.fsy_hi;
			const float xl = fmaf(cx, m.fsx_hi, -xh) + cx * m.fsx_lo;
			const float yl = fmaf(cy, m.fsy_hi, -yh) + cy * m.fsy_lo;
			const float dx = (xh - P.fxc_hi) + (xl - P.fxc_lo);
			const float dy = (yh - P.fyc_hi) + (yl - P.fyc_lo);
			fdx = dx;
			fdy = dy;
			xp = dx * sh.cs + dy * sh.sn;
			yp = (dy * sh.cs - dx * sh.sn) * sh.iq;
			const float rr = sqrtf(xp * xp + yp * yp) * P.finv_rscale;
			beyond = P.frmax > 0.f && rr > P.frmax;
			outside = rr > P.fswitch;
			const bool amb = (P.frmax > 0.f && fabsf(rr - P.frmax) <= kGuardRadiusB * P.frmax) ||
			                 fabsf(rr - P.fswitch) <= kGuardRadiusB * P.fswitch || !isfinite(rr);
			if (amb && active) {
				const unsigned int d = radius_f64(P, m, px, row);
				beyond = (d & 1u) != 0;
				outside = (d & 2u) != 0;
			}
		}
		bool need_ss = false;
		if (active && g != (T)0 && !beyond) {
			if (P.rough || outside) {
				T tmp[NS];
				point_terms<T, KINDS>(P, sh, gs, xp, yp, tmp);
#pragma unroll
				for (int k = 0; k < NS; k++) acc[k] += g * tmp[k];
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
					center = center_f64(P, m, spx, row);
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
				corner_pair_b(small_int_to_float((unsigned int)spx), m.fsx_hi, m.fsx_lo, P.fxc_hi, P.fxc_lo, bxh, bxl);
				corner_pair_b(small_int_to_float((unsigned int)row), m.fsy_hi, m.fsy_lo, P.fyc_hi, P.fyc_lo, byh, byl);
			}
			T sums[NS];
			warp_subsample_g<T, KINDS>(P, sh, gs, ws, bxh, bxl, byh, byl, dbl ? (T)m.sx : (T)m.fsx_hi,
			                           dbl ? (T)m.sy : (T)m.fsy_hi, res, max_rec, lane, sums);
			const T gsrc_px = __shfl_sync(0xffffffffu, g, src);
			if (lane == 0) {
#pragma unroll
				for (int k = 0; k < NS; k++) acc[k] += gsrc_px * sums[k];
			}
		}
	}
	// the lanes' sums added across the warp in T (single precision: 32 terms,
	// a few ulp), each total stored as this item's FP64 partial; the partials
	// are reduced in FP64 (grad_reduce_kernel)
	warp_store_slots<NS>(acc, lane, dst);
}

// Work items, taken by warps 32 at a time from a global counter (items with
// nothing to do cost one check):
//   phase A, n_profiles * kRingRows * kRingCols items: profile p's ring tile
//     (l, c) (pf_device.cuh), item k = (l * n_profiles + p) * kRingCols + c,
//     each one tile with its own partial, so that the deepest subsampling
//     trees -- the tiles nearest each profile's centre -- are spread over many
//     warps and start first;
//   phase B, n_profiles * n_ring items: profile p's drawing row ring(l) of its
//     bounding box, item n_a + l * n_profiles + p, every tile of the row but
//     its ring tiles, one partial per (profile, row).
template <typename T, unsigned int KINDS>
__global__ void __launch_bounds__(kWarpsB * 32, PF_BACKWARD_MIN_BLOCKS)
backward_kernel(const ModelDev *__restrict__ models, const ProfileDev *__restrict__ profs, unsigned int n_profiles,
                const T *__restrict__ gout, const T *__restrict__ gsrc, const double *__restrict__ psf_pool,
                const long long *__restrict__ prow_base, unsigned int n_ring, unsigned int *counter,
                double *__restrict__ partial, double *__restrict__ ring_partial)
{
	constexpr int NS = slots_of<KINDS>();
	__shared__ WarpScratchG<T, NS> scratch[kWarpsB];
	const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
	WarpScratchG<T, NS> &ws = scratch[warp];
	const unsigned int n_a = n_profiles * (kRingRows * kRingCols);
	const unsigned int n_items = n_a + n_ring * n_profiles;
	// phase A from counter[0], PF_BACKWARD_RING_CHUNK items per claim; phase B
	// from counter[1], 32 per claim (as the evaluation kernel)
	bool ring = n_a > 0;
	while (true) {
		unsigned int chunk = 0;
		if (lane == 0) {
			chunk = atomicAdd(&counter[ring ? 0 : 1], ring ? (unsigned int)PF_BACKWARD_RING_CHUNK : 32u);
		}
		chunk = __shfl_sync(0xffffffffu, chunk, 0);
		if (ring && chunk >= n_a) {
			ring = false;
			continue;
		}
		if (!ring) chunk += n_a;
		if (chunk >= n_items) break;
		const unsigned int k = chunk + (unsigned int)lane;
		int p = 0, row = -1, tc = -1;
		long long slot = 0;
		if (ring && lane >= PF_BACKWARD_RING_CHUNK) {
			// not this claim's item
		}
		else if (k < n_a) {
			const unsigned int per_ring = n_profiles * kRingCols;
			const unsigned int l = k / per_ring;
			const unsigned int rem = k - l * per_ring;
			p = (int)(rem / kRingCols);
			const int c = (int)(rem - (unsigned int)p * kRingCols);
			const ProfileDev &P = profs[p];
			if (!is_radial_kind(P.kind) || !ring_tile_of(P, models[P.model], (int)l, c, row, tc)) row = -1;
			slot = (((long long)p * kRingRows + l) * kRingCols + c) * NS;
		}
		else if (k < n_items) {
			const unsigned int kb = k - n_a;
			const unsigned int l = kb / n_profiles;
			p = (int)(kb - l * n_profiles);
			const ProfileDev &P = profs[p];
			row = item_row(P, models[P.model], (int)l);
		}
		unsigned int todo = __ballot_sync(0xffffffffu, row >= 0);
		while (todo) {
			const int src = __ffs(todo) - 1;
			todo &= todo - 1;
			const int ip = __shfl_sync(0xffffffffu, p, src);
			const int irow = __shfl_sync(0xffffffffu, row, src);
			const int itc = __shfl_sync(0xffffffffu, tc, src);
			const long long islot = __shfl_sync(0xffffffffu, slot, src);
			const ProfileDev &P = profs[ip];
			const ModelDev &m = models[P.model];
			if (itc >= 0) {  // phase A: one ring tile
				backward_row<T, KINDS>(m, P, irow, itc, itc, 0, -1, gout, gsrc, psf_pool, ws, lane,
				                       ring_partial + islot);
			}
			else {           // phase B: the row but its ring tiles
				int c0 = 0, c1 = (int)m.tiles_per_row - 1, s0 = 0, s1 = -1;
				if (P.kind == PF_PSF) {
					int x0, x1, y0, y1;
					psf_stamp(P, m, x0, x1, y0, y1);
					c0 = x0 / 32;
					c1 = x1 / 32;
				}
				else if (P.kind != PF_SKY) {
					c0 = max(0, P.bbx0) / 32;
					c1 = P.bbx1 < 0 ? -1 : min((int)m.draw_w - 1, P.bbx1) / 32;
					ring_cols_of_row(P, m, irow, s0, s1);
				}
				backward_row<T, KINDS>(m, P, irow, c0, c1, s0, s1, gout, gsrc, psf_pool, ws, lane,
				                       partial + (prow_base[ip] + irow) * (long long)NS);
			}
		}
	}
}

// d L / d par for every profile, one warp per profile: the (profile, row)
// and ring-tile partials summed in a fixed order (lane l takes rows l, l + 32,
// ... then ring slots l, l + 32, ...; then a fixed shuffle tree), then scaled
// by the flux scale and its logarithmic derivatives.
template <int NS>
__global__ void grad_reduce_kernel(const ModelDev *__restrict__ models, const ProfileDev *__restrict__ profs,
                                   int n_profiles, const long long *__restrict__ prow_base,
                                   const double *__restrict__ partial, const double *__restrict__ ring_partial,
                                   double *__restrict__ grad)
{
	const int i = (int)((blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5);
	const int lane = threadIdx.x & 31;
	if (i >= n_profiles) return;
	const ProfileDev &P = profs[i];
	const ModelDev &m = models[P.model];
	double *g = grad + (size_t)i * PF_NPAR;
	if (lane < PF_NPAR) g[lane] = 0.;
	const bool radial = is_radial_kind(P.kind);
	const bool psf = P.kind == PF_PSF && m.psf_off >= 0;
	if (!radial && !psf && P.kind != PF_SKY) return;
	int lo = 0, hi = (int)m.draw_h - 1;
	if (radial) {
		lo = max(0, P.bby0);
		hi = min(hi, P.bby1);
	}
	else if (psf) {
		int x0, x1;
		psf_stamp(P, m, x0, x1, lo, hi);
	}
	double S[NS];
	for (int k = 0; k < NS; k++) S[k] = 0.;
	for (int r = lo + lane; r <= hi; r += 32) {
		const double *src = partial + (prow_base[i] + r) * (long long)NS;
		for (int k = 0; k < NS; k++) S[k] += src[k];
	}
	if (radial) {
		for (int q = lane; q < kRingRows * kRingCols; q += 32) {
			int row, tc;
			if (!ring_tile_of(P, m, q / kRingCols, q % kRingCols, row, tc)) continue;
			const double *src = ring_partial + ((long long)i * (kRingRows * kRingCols) + q) * NS;
			for (int k = 0; k < NS; k++) S[k] += src[k];
		}
	}
	__shared__ double tot[8][16];
	double *T8 = tot[threadIdx.x >> 5];
	warp_store_slots<NS>(S, lane, T8);
	__syncwarp();
	if (lane != 0) return;
	if (P.kind == PF_SKY) {
		g[6] = T8[G_V] / (m.fs * m.fs);  // d/d bg of bg / fs^2 on every pixel (src/sky.cpp:42-45)
		return;
	}
	if (psf) {  // value x 10^(-0.4 (mag - magzero)) (src/psf.cpp:66, 141)
		const double sc = P.psf_mag_scale;
		g[PF_P_XCEN] = sc * T8[G_XCEN];
		g[PF_P_YCEN] = sc * T8[G_YCEN];
		g[PF_P_MAG] = -0.4 * log(10.) * sc * T8[G_V];
		return;
	}
	const double fs_ = P.flux_scale;
	g[PF_P_XCEN] = fs_ * T8[G_XCEN];
	g[PF_P_YCEN] = fs_ * T8[G_YCEN];
	g[PF_P_MAG] = fs_ * P.dlnfs[PF_P_MAG] * T8[G_V];
	g[PF_P_ANG] = fs_ * T8[G_ANG];
	g[PF_P_AXRAT] = fs_ * (T8[G_AXRAT] + P.dlnfs[PF_P_AXRAT] * T8[G_V]);
	g[PF_P_BOX] = fs_ * (T8[G_BOX] + P.dlnfs[PF_P_BOX] * T8[G_V]);
	for (int k = PF_P_X0; k < NS; k++) g[k] = fs_ * (T8[k] + P.dlnfs[k] * T8[G_V]);
}

}  // namespace

template <typename T>
void launch_chi2(const ModelDev *models, int n_models, const void *img, const void *data, const void *sigma,
                 const void *cot, void *gout, double *chi2, int parts, double *partial, unsigned int *done,
                 cudaStream_t stream)
{
	if (n_models <= 0) return;
	const auto a16 = [](const void *p) { return ((uintptr_t)p & 15u) == 0; };
	const bool vec = a16(img) && a16(data) && a16(sigma) && a16(gout);
	chi2_kernel<T><<<dim3((unsigned int)n_models, (unsigned int)parts), 256, 0, stream>>>(
	    models, (const T *)img, (const T *)data, (const T *)sigma, (const T *)cot, (T *)gout, chi2, partial, done,
	    vec);
}


template <typename T>
void launch_backward(const ModelDev *models, const ProfileDev *profs, int n_profiles, const void *gout,
                     const void *gsrc, const double *psf_pool, const long long *prow_base, unsigned int n_ring,
                     unsigned int *counter, double *partial, double *ring_partial, double *grad, bool sersic_only,
                     int n_sm, cudaStream_t stream)
{
	if (n_profiles <= 0) return;
	const int blocks = n_sm * PF_BACKWARD_MIN_BLOCKS;
	const int rblocks = (int)(((long long)n_profiles * 32 + 255) / 256);
	if (sersic_only) {
		backward_kernel<T, f32::kSersicOnly><<<blocks, kWarpsB * 32, 0, stream>>>(
		    models, profs, (unsigned int)n_profiles, (const T *)gout, (const T *)gsrc, psf_pool, prow_base, n_ring,
		    counter, partial, ring_partial);
		grad_reduce_kernel<slots_of<f32::kSersicOnly>()><<<rblocks, 256, 0, stream>>>(
		    models, profs, n_profiles, prow_base, partial, ring_partial, grad);
	}
	else {
		backward_kernel<T, f32::kAllKinds><<<blocks, kWarpsB * 32, 0, stream>>>(
		    models, profs, (unsigned int)n_profiles, (const T *)gout, (const T *)gsrc, psf_pool, prow_base, n_ring,
		    counter, partial, ring_partial);
		grad_reduce_kernel<slots_of<f32::kAllKinds>()><<<rblocks, 256, 0, stream>>>(
		    models, profs, n_profiles, prow_base, partial, ring_partial, grad);
	}
}

long long backward_items(long long n_profiles, long long n_ring)
{
	return n_profiles * (kRingRows * kRingCols) + n_profiles * n_ring;
}

int backward_slots(bool sersic_only)
{
	return sersic_only ? slots_of<f32::kSersicOnly>() : slots_of<f32::kAllKinds>();
}

long long backward_ring_slots(bool sersic_only) { return (long long)kRingRows * kRingCols * backward_slots(sersic_only); }

template void launch_chi2<float>(const ModelDev *, int, const void *, const void *, const void *, const void *, void *,
                                 double *, int, double *, unsigned int *, cudaStream_t);
template void launch_chi2<double>(const ModelDev *, int, const void *, const void *, const void *, const void *,
                                  void *, double *, int, double *, unsigned int *, cudaStream_t);
template void launch_backward<float>(const ModelDev *, const ProfileDev *, int, const void *, const void *,
                                     const double *, const long long *, unsigned int, unsigned int *, double *,
                                     double *, double *, bool, int, cudaStream_t);
template void launch_backward<double>(const ModelDev *, const ProfileDev *, int, const void *, const void *,
                                      const double *, const long long *, unsigned int, unsigned int *, double *,
                                      double *, double *, bool, int, cudaStream_t);

}  // namespace pf
