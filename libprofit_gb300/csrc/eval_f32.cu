// Batched single-precision path: FP32 profile values, FP64 where precision
// decides the result.
//
// Same structure as the plain FP64 path (eval_f64.cu): warps over 32-pixel
// row tiles of a model's drawing area (here a row segment of up to 8 tiles
// per work item), the model's profiles in order, and a warp-cooperative
// depth-first recursion for the pixels that RadialProfile::evaluate_cpu
// subsamples (src/radial.cpp:291-344, subsample_pixel src/radial.cpp:55-135).
// The differences:
//   * profile values are computed in FP32 (profiles_f32.cuh), coordinates
//     relative to the profile centre, the pixel centre formed with an
//     error-free float product so that it keeps full relative precision;
//   * each sub-pixel box corner is tracked relative to the profile centre as
//     an unevaluated float pair (hi + lo, an error-free addition per level),
//     so that boxes 8^-11 pixel wide at the centre of a high-index Sersic
//     profile keep their geometry; the points inside a box are FP32 offsets
//     from its corner;
//   * the file is compiled without multiply-add contraction, its
//     multiply-adds written as fmaf, so that every kernel instance rounds
//     alike;
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

// Warps per block, and blocks per SM the register allocation is sized for.
// The kernel that walks the trees in place: 4 blocks, 128 registers and 16
// warps per SM (measured on the 1024-model step with the row segments below:
// 2.41 ms, against 2.82 ms at 20 warps and 96 registers, whose spills fall in
// the subsampling walk, and 3.21 ms at 24 warps). The kernels that split the
// trees off (the tile kernel and split_boxes32_kernel): 5 blocks, 96
// registers, 20 warps (the 4096 uneven models: evaluation 42.9 ms, against
// 48.5 ms at 16 warps: the split boxes need warps more than registers).
#ifndef PF_EVAL32_WARPS
#define PF_EVAL32_WARPS 4
#endif
#ifndef PF_EVAL32_MIN_BLOCKS
#define PF_EVAL32_MIN_BLOCKS 4
#endif
#ifndef PF_EVAL32_SPLIT_MIN_BLOCKS
#define PF_EVAL32_SPLIT_MIN_BLOCKS 5
#endif
// phase-A (ring tile) items a warp claims at once (a divisor of 32; 32, 8
// and 2 measured within 5 % of each other on the 1024-model step)
#ifndef PF_EVAL_RING_CHUNK
#define PF_EVAL_RING_CHUNK 32
#endif
// phase-B tiles a warp claims at once (a divisor of 32; 8 and 2 measured no
// better on the 1024-model step or the 4096 uneven models)
#ifndef PF_EVAL_TILE_CHUNK
#define PF_EVAL_TILE_CHUNK 32
#endif
constexpr int kWarps32 = PF_EVAL32_WARPS;
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
	const float ep = fmaf(i, s_lo, fmaf(i, s_hi, -p));
	float e;
	two_sum(p, -c_hi, hi, e);
	lo = (e + ep) - c_lo;
}

struct WarpScratchM {
	FrameM fr[kMaxLevels];
	unsigned int amb[kMaskWords];  // sub-points of the frame being evaluated whose decision is re-taken in FP64
};

__device__ __forceinline__ float warp_sum(float v)
{
#pragma unroll
	for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
	return v;
}

// The rare FP64 re-takes. They take only single-precision and integer
// arguments, so that no double-precision work is scheduled on the common
// path; the two of the subsampling recursion are inlined (a call there costs
// the whole kernel some 30 registers) and evaluate only the batch's kinds. A
// point is given relative to the profile centre as (xa + xb) + xc,
// (ya + yb) + yc, summed in FP64.

// FP64 profile value for a kernel built for the kinds in KINDS
template <unsigned int KINDS>
__device__ __forceinline__ double value64(const ProfileDev &P, double x, double y)
{
	if constexpr (KINDS == f32::kSersicOnly) return f64::sersic(P, x, y);
	else return f64::evaluate_at(P, x, y);
}

// value and accuracy test of one sub-point
template <unsigned int KINDS>
__device__ __forceinline__ bool test_f64(const ProfileDev &P, float xa, float xb, float xc, float ya, float yb,
                                         float yc, float xbin, float ybin, float &subval)
{
	const double dx = ((double)xa + (double)xb) + (double)xc;
	const double dy = ((double)ya + (double)yb) + (double)yc;
	const double xp = dx * P.cos_ang + dy * P.sin_ang;
	const double yp = (-dx * P.sin_ang + dy * P.cos_ang) / P.par[PF_P_AXRAT];
	const double s = value64<KINDS>(P, xp, yp);
	const double dyp = (-(double)xbin * P.sin_ang + (double)ybin * P.cos_ang) / P.par[PF_P_AXRAT];
	const double t = value64<KINDS>(P, fabs(xp), fabs(yp) + fabs(dyp));
	subval = (float)s;
	return fabs(t / s - 1.0) > P.acc;
}

template <unsigned int KINDS>
__device__ __forceinline__ float value_f64(const ProfileDev &P, float xa, float xb, float xc, float ya, float yb,
                                           float yc)
{
	const double dx = ((double)xa + (double)xb) + (double)xc;
	const double dy = ((double)ya + (double)yb) + (double)yc;
	const double xp = dx * P.cos_ang + dy * P.sin_ang;
	const double yp = (-dx * P.sin_ang + dy * P.cos_ang) / P.par[PF_P_AXRAT];
	return (float)value64<KINDS>(P, xp, yp);
}

// the reference's r_prof decisions for drawing pixel (px, row)
// (src/radial.cpp:313-326): bit 0 beyond rscale_max, bit 1 beyond rscale_switch
__device__ __noinline__ unsigned int radius_f64(const ProfileDev &P, const ModelDev &m, unsigned int px,
                                                unsigned int row)
{
	const double x = m.sx / 2. + px * m.sx, y = m.sy / 2. + row * m.sy;
	double xp, yp;
	f64::to_profile(P, x, y, xp, yp);
	const double r = sqrt(xp * xp + yp * yp);
	return (P.rscale_max > 0 && r / P.rscale > P.rscale_max ? 1u : 0u) | (r / P.rscale > P.rscale_switch ? 2u : 0u);
}

// the sersic central-pixel test (src/sersic.cpp:331-347)
__device__ __noinline__ bool center_f64(const ProfileDev &P, const ModelDev &m, unsigned int px, unsigned int row)
{
	const double x = m.sx / 2. + px * m.sx, y = m.sy / 2. + row * m.sy;
	return fabs(x - P.xc) < m.scale_x && fabs(y - P.yc) < m.scale_y;
}

// the psf profile's stamp value at drawing pixel (px, row); false outside it
__device__ __noinline__ bool psf_value(const ProfileDev &P, const ModelDev &m, const double *psf, unsigned int px,
                                       unsigned int row, float &v)
{
	double d = 0;
	const bool in = psf_pixel64(P, m, psf, px, row, d);
	v = (float)d;
	return in;
}

template <unsigned int KINDS>
__device__ void eval_frame_m(const ProfileDev &P, const f32::Shape &sh, WarpScratchM &ws, int L, unsigned int res,
                             float inv_res, unsigned int max_rec, int lane, unsigned long long *counts)
{
	FrameM &f = ws.fr[L];
	const float xhi = f.xhi, xlo = f.xlo, yhi = f.yhi, ylo = f.ylo;
	const float fxbin = f.bx * inv_res, fybin = f.by * inv_res;
	const bool recurse = res > 1 && (unsigned int)L < max_rec;
	const unsigned int n = res * res;
	const float c = sh.cs, s = sh.sn, iq = sh.iq, facc = sh.acc;
	const float fdyp = fabsf(fmaf(fybin, c, -(fxbin * s)) * iq);
	if (counts && lane == 0 && L < kLevelCounts) {
		atomicAdd(&counts[L], 1ull);
		atomicAdd(&counts[kCountSubEvals], (unsigned long long)(recurse ? 2 * n : n));
	}
	float part = 0.f;
	const unsigned int magic = res_magic(res);
	unsigned int amb_any = 0;
	for (unsigned int base = 0; base < n; base += 32) {
		const unsigned int idx = base + lane;
		bool fail = false, amb = false;
		if (idx < n) {
			const unsigned int i = div_res(idx, magic), j = idx - i * res;
			const float ox = (small_int_to_float(i) + 0.5f) * fxbin, oy = (small_int_to_float(j) + 0.5f) * fybin;
			const float dx = (xhi + ox) + xlo;
			const float dy = (yhi + oy) + ylo;
			const float xp = fmaf(dx, c, dy * s);
			const float yp = fmaf(dy, c, -(dx * s)) * iq;
			const float sub = f32::value<KINDS>(sh, xp, yp);
			if (recurse) {
				const float t = f32::value<KINDS>(sh, fabsf(xp), fabsf(yp) + fdyp);
				const float d = fabsf(__fdividef(t, sub) - 1.f);
				amb = !(isfinite(d) && isfinite(sub)) || fabsf(d - facc) <= kGuardAcc * (facc + 1.f);
				fail = !amb && d > facc;
			}
			else {
				amb = !isfinite(sub);
			}
			if (!fail && !amb) part += sub;
		}
		const unsigned int word = __ballot_sync(0xffffffffu, fail);
		const unsigned int aword = __ballot_sync(0xffffffffu, amb);
		if (lane == 0) {
			f.mask[base >> 5] = word;
			ws.amb[base >> 5] = aword;
		}
		amb_any |= aword;
	}
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
				const float ox = (small_int_to_float(i) + 0.5f) * fxbin, oy = (small_int_to_float(j) + 0.5f) * fybin;
				float sub;
				if (recurse) fail = test_f64<KINDS>(P, xhi, xlo, ox, yhi, ylo, oy, fxbin, fybin, sub);
				else sub = value_f64<KINDS>(P, xhi, xlo, ox, yhi, ylo, oy);
				if (!fail) part += sub;
			}
			const unsigned int word = __ballot_sync(0xffffffffu, fail);
			if (lane == 0) f.mask[base >> 5] |= word;
		}
	}
	part = warp_sum(part);
	if (lane == 0) f.total = part;
	__syncwarp();
}

// The depth-first walk of subsample_pixel below frame L0 of the warp's
// scratch, which has been evaluated (its total holds its accepted sub-points,
// its mask the failing ones): each failing sub-point's box evaluated and
// walked in ascending order, its value added to the frame's total. Returns
// the frame's value, total / res^2; `deepest`: the deepest level + 1 reached.
template <unsigned int KINDS>
__device__ float warp_walk_m(const ProfileDev &P, const f32::Shape &sh, WarpScratchM &ws, int L0, unsigned int res,
                             unsigned int max_rec, int lane, unsigned long long *counts, int &deepest)
{
	const float inv_res = __frcp_rn((float)res);
	const float inv_res2 = __frcp_rn((float)(res * res));
	int L = L0;
	deepest = L0 + 1;
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
			eval_frame_m<KINDS>(P, sh, ws, L, res, inv_res, max_rec, lane, counts);
		}
		else {
			const float v = f.total * inv_res2;
			if (L == L0) {
				return v;
			}
			L--;
			if (lane == 0) ws.fr[L].total += v;
			__syncwarp();
		}
	}
}

// subsample_pixel on a box given relative to the profile centre: its frame
// evaluated and walked (the kernels that split no trees)
template <unsigned int KINDS>
__device__ float warp_subsample_m(const ProfileDev &P, const f32::Shape &sh, WarpScratchM &ws, float xhi, float xlo,
                                  float yhi, float ylo, float bx, float by, unsigned int res, unsigned int max_rec,
                                  int lane, unsigned long long *counts, int &deepest)
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
	eval_frame_m<KINDS>(P, sh, ws, 0, res, __frcp_rn((float)res), max_rec, lane, counts);
	return warp_walk_m<KINDS>(P, sh, ws, 0, res, max_rec, lane, counts, deepest);
}

// Frame L of the warp's scratch set to a box relative to the profile centre
__device__ __forceinline__ void set_frame(WarpScratchM &ws, int L, float xhi, float xlo, float yhi, float ylo, float bx,
                                          float by, int lane)
{
	if (lane == 0) {
		ws.fr[L].xhi = xhi;
		ws.fr[L].xlo = xlo;
		ws.fr[L].yhi = yhi;
		ws.fr[L].ylo = ylo;
		ws.fr[L].bx = bx;
		ws.fr[L].by = by;
	}
	__syncwarp();
}

// Exports the failing sub-points of the evaluated level-0 frame of a
// subsampled drawing pixel as level-1 boxes of the split pool (SplitPool in
// pf_device.cuh). Returns false, having exported nothing, when fewer than
// pool.min_fail sub-points fail or the pool has no room; the caller then walks
// the tree itself. Warp-uniform; lane `src` holds the pixel, whose split
// record (prec) and last split root (plast) are updated.
__device__ bool split_root(const SplitPool &pool, const ProfileDev &P, int pi, const ModelDev &m, WarpScratchM &ws,
                           unsigned int res, unsigned int max_rec, int lane, int src, long long canvas_idx,
                           long long depth_idx, int &prec, int &plast)
{
	const FrameM &f = ws.fr[0];
	const unsigned int nwords = (res * res + 31) / 32;
	unsigned int nf = 0;
	for (unsigned int w = 0; w < nwords; w++) nf += __popc(f.mask[w]);
	if (nf == 0 || nf < pool.min_fail) return false;
	const int old_prec = __shfl_sync(0xffffffffu, prec, src), old_last = __shfl_sync(0xffffffffu, plast, src);
	int p = old_prec, r = -1;
	unsigned int b0 = 0, ok = 1;
	if (lane == 0) {
		if (p < 0) {
			const unsigned int q = atomicAdd(&pool.cnt[2], 1u);
			if (q < pool.cap_pix) p = (int)q;
			else ok = 0;
		}
		if (ok) {
			const unsigned int q = atomicAdd(&pool.cnt[1], 1u);
			if (q < pool.cap_root) r = (int)q;
			else ok = 0;
		}
		if (ok) {
			// room for nf boxes, taken without passing the capacity (a lock-free
			// retry: each failed exchange means another warp took room)
			ok = 0;
			unsigned int old = *(volatile unsigned int *)&pool.cnt[0];
			for (int tries = 0; tries < (1 << 16) && old <= pool.cap_box && pool.cap_box - old >= nf; tries++) {
				const unsigned int got = atomicCAS(&pool.cnt[0], old, old + nf);
				if (got == old) {
					b0 = old;
					ok = 1;
					break;
				}
				old = got;
			}
		}
		if (!ok) atomicAdd(&pool.cnt[4], 1u);
	}
	if (!__shfl_sync(0xffffffffu, ok, 0)) return false;
	p = __shfl_sync(0xffffffffu, p, 0);
	r = __shfl_sync(0xffffffffu, r, 0);
	b0 = __shfl_sync(0xffffffffu, b0, 0);
	if (lane == 0) {
		SplitRoot &R = pool.root[r];
		R.accepted = f.total;
		R.first_box = b0;
		R.n_boxes = nf;
		R.pending = nf;
		R.profile = pi;
		R.pixel = p;
		R.next = -1;
		R.depth = 1;
		R.res = res;
		R.fflux = P.fflux_scale;
		R.convolve = P.convolve;
		R.value = 0.f;
		R.depth_idx = depth_idx;
		SplitPixel &X = pool.pix[p];
		if (old_prec < 0) {
			X.idx = canvas_idx;
			X.s_conv = X.s_direct = 0.f;
			X.first_root = r;
			X.pending = 1;
			X.conv_required = m.conv_required;
			X.direct_required = m.direct_required;
		}
		else {
			pool.root[old_last].next = r;
			X.pending += 1;
		}
	}
	// the boxes in ascending sub-point order, placed as the walk would place
	// its child frames
	const float inv_res = __frcp_rn((float)res);
	const float cbx = f.bx * inv_res, cby = f.by * inv_res;
	const unsigned int magic = res_magic(res);
	const uint32_t meta = res | (1u << 8) | (max_rec << 16);
	unsigned int rank = 0;
	for (unsigned int w = 0; w < nwords; w++) {
		const unsigned int bits = f.mask[w];
		if ((bits >> lane) & 1u) {
			const unsigned int k = w * 32 + (unsigned int)lane;
			const unsigned int i = div_res(k, magic), j = k - i * res;
			SplitBox bx;
			float e;
			two_sum(f.xhi, small_int_to_float(i) * cbx, bx.xhi, e);
			bx.xlo = f.xlo + e;
			two_sum(f.yhi, small_int_to_float(j) * cby, bx.yhi, e);
			bx.ylo = f.ylo + e;
			bx.bx = cbx;
			bx.by = cby;
			bx.root = r;
			bx.meta = meta;
			pool.box[b0 + rank + __popc(bits & ((1u << lane) - 1u))] = bx;
		}
		rank += __popc(bits);
	}
	__syncwarp();
	if (lane == src) {
		prec = p;
		plast = r;
	}
	return true;
}

// Tiles a phase-B work item evaluates together: consecutive 32-pixel tiles of
// one drawing row, each profile's constants loaded once for all of them
// (measured on the 1024-model step with every profile rough: 1.54 ms one tile
// at a time, the profile and model data loaded for each tile).
#ifndef PF_EVAL_SEG_TILES
#define PF_EVAL_SEG_TILES 8
#endif
constexpr int kSegTiles = PF_EVAL_SEG_TILES;
// a claim of ring items starts a profile's ring row: its lanes 4g .. 4g + 3
// are one row's kRingCols tiles
static_assert(PF_EVAL_RING_CHUNK % kRingCols == 0, "ring claims hold whole ring rows");

// A warp's per-pixel running sums over a segment's tiles, lane-major in shared
// memory: the conv and direct image values, and (split kernels) the pixel's
// split record and last split root.
template <bool SPLIT>
struct SegScratch {
	float conv[kSegTiles][32], direct[kSegTiles][32];
	int prec[SPLIT ? kSegTiles : 1][32], plast[SPLIT ? kSegTiles : 1][32];
	unsigned int pend[kSegTiles];  // the current profile's subsampled pixels, a bit per lane
};

// Tiles tc0 .. tc0 + nt - 1 (nt <= kSegTiles; the ones whose bit is set in
// `own`) of drawing row `row` of model mi: every profile of the model in
// order, summed into the conv / direct images. A pixel's sum is formed in
// profile order, as one tile at a time forms it. KINDS: the radial profile
// kinds of the batch.
template <unsigned int KINDS, bool SPLIT>
__device__ __forceinline__ void eval_seg(const ModelDev *__restrict__ models, int mi,
                                         const ProfileDev *__restrict__ profs, const double *__restrict__ psf_pool,
                                         float *__restrict__ conv_img, float *__restrict__ direct_img, int row,
                                         int tc0, int nt, unsigned int own, WarpScratchM &ws, SegScratch<SPLIT> &ss,
                                         int lane, const DebugRec &dbg, const SplitPool &pool)
{
	const ModelDev &m = models[mi];
	const int col0 = tc0 * 32;
	const int col1 = min((tc0 + nt) * 32 - 1, (int)m.draw_w - 1);
	const double *psf = m.psf_off >= 0 ? psf_pool + m.psf_off : nullptr;
	for (int j = 0; j < nt; j++) {
		ss.conv[j][lane] = 0.f;
		ss.direct[j][lane] = 0.f;
		if constexpr (SPLIT) {
			ss.prec[j][lane] = -1;
			ss.plast[j][lane] = -1;
		}
	}
	// pixel centre (i + 1/2) * scale as an unevaluated float sum (y: the row's)
	const float cy = small_int_to_float((unsigned int)row) + 0.5f;
	const float yh = cy * m.fsy_hi;
	const float yl = fmaf(cy, m.fsy_lo, fmaf(cy, m.fsy_hi, -yh));

	for (int q0 = 0; q0 < m.n_profiles; q0 += 32) {
		// 32 profiles' culling boxes tested at once, one per lane; the ones
		// that reach the segment drawn one by one, in profile order
		const bool reaches = profile_reaches(profs, m, q0 + lane, row, col0, col1);
		unsigned int todo = __ballot_sync(0xffffffffu, reaches);
		while (todo) {
			const int q = q0 + __ffs(todo) - 1;
			todo &= todo - 1;
			const int pi = m.first_profile + q;
			const ProfileDev &P = profs[pi];
			const int kind = P.kind;
			const bool conv = P.convolve != 0;
			if (kind == PF_SKY || kind == PF_PSF) {
				const float fbg = P.fbg;
				for (int j = 0; j < nt; j++) {
					if (!((own >> j) & 1u)) continue;
					const unsigned int px = (unsigned int)(col0 + 32 * j + lane);
					const bool active = px < m.draw_w;
					float add = 0.f;
					bool has;
					if (kind == PF_SKY) {
						add = fbg;
						has = active && evaluated(m, (int)px, row);
					}
					else {
						has = active && psf && psf_value(P, m, psf, px, (unsigned int)row, add);
					}
					if (has) {
						if (conv) ss.conv[j][lane] += add;
						else ss.direct[j][lane] += add;
					}
				}
				continue;
			}
			if (!is_radial(kind)) continue;
			const f32::Shape sh = f32::load_shape(P);
			const float fxc_hi = P.fxc_hi, fxc_lo = P.fxc_lo;
			const float dy = (yh - P.fyc_hi) + (yl - P.fyc_lo);
			const float inv_rscale = P.finv_rscale, frmax = P.frmax, fswitch = P.fswitch;
			const bool rough = P.rough != 0;
			const float fflux = P.fflux_scale;
			// the segment's tiles that the profile's culling box reaches
			const int jlo = max(0, (max(P.bbx0, col0) >> 5) - tc0);
			const int jhi = min(nt - 1, (min(P.bbx1, col1) >> 5) - tc0);
			unsigned long long *counts = dbg.counts ? dbg.counts + (size_t)pi * kLevelCounts : nullptr;
			// the pixels evaluated directly, tile by tile; the subsampled ones
			// marked, then walked tile by tile (no calls in the first loop, so
			// that its values stay in registers). Each pixel gets one addition
			// per profile, in profile order.
			unsigned int any_ss = 0;
			for (int j = jlo; j <= jhi; j++) {
				if (!((own >> j) & 1u)) continue;
				const unsigned int px = (unsigned int)(col0 + 32 * j + lane);
				const bool active = px < m.draw_w;
				const bool in_mask = active && evaluated(m, (int)px, row);  // the calculation mask
				const float cx = small_int_to_float(px) + 0.5f;
				const float xh = cx * m.fsx_hi;
				const float xl = fmaf(cx, m.fsx_lo, fmaf(cx, m.fsx_hi, -xh));
				const float dx = (xh - fxc_hi) + (xl - fxc_lo);
				const float xp = fmaf(dx, sh.cs, dy * sh.sn);
				const float yp = fmaf(dy, sh.cs, -(dx * sh.sn)) * sh.iq;
				const float rr = sqrtf(fmaf(xp, xp, yp * yp)) * inv_rscale;
				bool beyond = frmax > 0.f && rr > frmax;
				bool outside = rr > fswitch;
				const bool amb = (frmax > 0.f && fabsf(rr - frmax) <= kGuardRadius * frmax) ||
				                 fabsf(rr - fswitch) <= kGuardRadius * fswitch || !isfinite(rr);
				if (amb && in_mask) {
					const unsigned int d = radius_f64(P, m, px, (unsigned int)row);
					beyond = (d & 1u) != 0;
					outside = (d & 2u) != 0;
				}
				beyond |= !in_mask;  // masked pixels are not evaluated (src/radial.cpp:305-307)
				float pixel_val = 0.f;
				bool need_ss = false;
				if (beyond) {
				}
				else if (rough || outside) {
					pixel_val = f32::value<KINDS>(sh, xp, yp);
					if (!isfinite(pixel_val)) pixel_val = value_f64<KINDS>(P, dx, 0.f, 0.f, dy, 0.f, 0.f);
				}
				else {
					need_ss = true;
				}
				const unsigned int pending = __ballot_sync(0xffffffffu, need_ss && active);
				if (lane == 0) ss.pend[j] = pending;
				any_ss |= pending;
				if (counts) {
					const unsigned int nd = __popc(__ballot_sync(0xffffffffu, active && !beyond && !need_ss));
					if (lane == 0 && nd) atomicAdd(&counts[kCountDirectEvals], (unsigned long long)nd);
				}
				if (active && !need_ss) {
					if (dbg.depth) dbg.depth[P.depth_off + (size_t)row * m.draw_w + px] = (int8_t)(beyond ? -1 : 0);
					const float add = fflux * pixel_val;
					if (conv) ss.conv[j][lane] += add;
					else ss.direct[j][lane] += add;
				}
			}
			if (!any_ss) continue;
			__syncwarp();
			for (int j = jlo; j <= jhi; j++) {
				unsigned int pending = ss.pend[j];
				if (!((own >> j) & 1u) || !pending) continue;
				const bool mine = (pending >> lane) & 1u;
				const int tcol0 = col0 + 32 * j;
				// the pixel's split record and last split root, while trees are split
				int prec = -1, plast = -1;
				if constexpr (SPLIT) {
					prec = ss.prec[j][lane];
					plast = ss.plast[j][lane];
				}
				float pixel_val = 0.f;
				int depth = 0;
				bool split = false;
				while (pending) {
					const int src = __ffs(pending) - 1;
					pending &= pending - 1;
					const unsigned int spx = (unsigned int)tcol0 + src;
					unsigned int res = P.resolution, max_rec = P.max_recursions;
					if (P.center_boost) {  // src/sersic.cpp:331-347
						// the pixel's x offset from the centre, as the first loop formed it
						const float scx = small_int_to_float(spx) + 0.5f;
						const float sxh = scx * m.fsx_hi;
						const float sxl = fmaf(scx, m.fsx_lo, fmaf(scx, m.fsx_hi, -sxh));
						const float sdx = (sxh - fxc_hi) + (sxl - fxc_lo);
						bool center = fabsf(sdx) < m.fscale_x && fabsf(dy) < m.fscale_y;
						if (fabsf(fabsf(sdx) - m.fscale_x) <= 1e-5f * m.fscale_x ||
						    fabsf(fabsf(dy) - m.fscale_y) <= 1e-5f * m.fscale_y) {
							center = center_f64(P, m, spx, (unsigned int)row);
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
					corner_pair(small_int_to_float(spx), m.fsx_hi, m.fsx_lo, fxc_hi, fxc_lo, bxh, bxl);
					corner_pair(small_int_to_float((unsigned int)row), m.fsy_hi, m.fsy_lo, P.fyc_hi, P.fyc_lo, byh,
					            byl);
					int deepest = 0;
					float v = 0.f;
					if constexpr (SPLIT) {
						// the level-0 box; its failing sub-points' subtrees split off
						// to other warps, or walked here
						set_frame(ws, 0, bxh, bxl, byh, byl, m.fsx_hi, m.fsy_hi, lane);
						eval_frame_m<KINDS>(P, sh, ws, 0, res, __frcp_rn((float)res), max_rec, lane, counts);
						const long long didx =
						    dbg.depth ? P.depth_off + (long long)row * m.draw_w + (long long)spx : -1;
						if (split_root(pool, P, pi, m, ws, res, max_rec, lane, src,
						               (long long)m.draw_off + (long long)row * m.draw_w + spx, didx, prec, plast)) {
							if (lane == src) split = true;
							continue;
						}
						v = warp_walk_m<KINDS>(P, sh, ws, 0, res, max_rec, lane, counts, deepest);
					}
					else {
						v = warp_subsample_m<KINDS>(P, sh, ws, bxh, bxl, byh, byl, m.fsx_hi, m.fsy_hi, res, max_rec,
						                            lane, counts, deepest);
					}
					if (lane == src) {
						pixel_val = v;
						depth = deepest;
					}
				}
				if constexpr (SPLIT) {
					ss.prec[j][lane] = prec;
					ss.plast[j][lane] = plast;
				}
				// a split profile's value is added when its boxes finish
				if (mine && !split) {
					if (dbg.depth) dbg.depth[P.depth_off + (size_t)row * m.draw_w + tcol0 + lane] = (int8_t)depth;
					const float add = fflux * pixel_val;
					if (conv) ss.conv[j][lane] += add;
					else ss.direct[j][lane] += add;
				}
			}
			__syncwarp();
		}
	}
	for (int j = 0; j < nt; j++) {
		if (!((own >> j) & 1u)) continue;
		const unsigned int px = (unsigned int)(col0 + 32 * j + lane);
		if (px >= m.draw_w) continue;
		const size_t canvas_idx = (size_t)m.draw_off + (size_t)row * m.draw_w + px;
		const float c = ss.conv[j][lane], d = ss.direct[j][lane];
		if (SPLIT && ss.prec[j][lane] >= 0) {
			// the split profiles' values are still to come: the warp that
			// finishes the last of them writes the canvas
			const int prec = ss.prec[j][lane];
			pool.pix[prec].s_conv = c;
			pool.pix[prec].s_direct = d;
		}
		else {
			if (m.conv_required) conv_img[canvas_idx] = c;
			if (m.direct_required) direct_img[canvas_idx] = d;  // else all zero, and read as zero
		}
	}
	__syncwarp();
}

// Phase A item k (k < n_profiles * kRingRows * kRingCols): tile column
// k % kRingCols of a window of the profile's subsampling box around its
// centre, in the box's row ring(l), l = k /
// (n_profiles * kRingCols) -- the centre row, the one above, the one below,
// ... -- so that the rows nearest every profile's centre, where the
// subsampling trees are deep, come first. Returns the global tile number, or
// -1 if the item has none.
__device__ __forceinline__ long long ring_tile(const ModelDev *__restrict__ models,
                                               const ProfileDev *__restrict__ profs, unsigned int n_profiles,
                                               unsigned int k)
{
	const unsigned int per_ring = n_profiles * kRingCols;
	const unsigned int l = k / per_ring;
	const unsigned int rem = k - l * per_ring;
	const unsigned int p = rem / kRingCols;
	const int c = (int)(rem - p * kRingCols);
	const ProfileDev &P = profs[p];
	const ModelDev &m = models[P.model];
	int row, tcol;
	if (!ring_tile_of(P, m, (int)l, c, row, tcol)) return -1;
	return m.tile_base + (long long)row * m.tiles_per_row + tcol;
}

// Work items: phase A (ring_tile, n_ring_items of them, a multiple of 32),
// then phase B, every tile in order. Warps take phase-A items
// PF_EVAL_RING_CHUNK at a time from counter[0] (the costly centre tiles of one profile are not
// all left to one warp) and phase-B tiles 32 at a time from counter[1]; a
// tile is evaluated by the item that first sets its bit in `claims` (zeroed
// before the launch), so each tile exactly once.
template <unsigned int KINDS, bool SPLIT>
__global__ void __launch_bounds__(kWarps32 * 32, SPLIT ? PF_EVAL32_SPLIT_MIN_BLOCKS : PF_EVAL32_MIN_BLOCKS)
eval_tiles32_kernel(const ModelDev *__restrict__ models, int n_models, const ProfileDev *__restrict__ profs,
                    unsigned int n_profiles, const double *__restrict__ psf_pool, float *__restrict__ conv_img,
                    float *__restrict__ direct_img, unsigned int n_tiles, unsigned int n_ring_items,
                    unsigned int *counter, unsigned int *claims, DebugRec dbg, SplitPool pool)
{
	__shared__ WarpScratchM scratch[kWarps32];
	__shared__ SegScratch<SPLIT> segs[kWarps32];
	const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
	WarpScratchM &ws = scratch[warp];
	SegScratch<SPLIT> &ss = segs[warp];
	bool ring = n_ring_items > 0;
	int mi = 0;  // the model of the warp's last tile
	while (true) {
		unsigned int chunk = 0;
		if (lane == 0) {
			chunk = atomicAdd(&counter[ring ? 0 : 1],
			                  ring ? (unsigned int)PF_EVAL_RING_CHUNK : (unsigned int)PF_EVAL_TILE_CHUNK);
		}
		chunk = __shfl_sync(0xffffffffu, chunk, 0);
		if (ring && chunk >= n_ring_items) {
			ring = false;
			continue;
		}
		if (!ring && chunk >= n_tiles) break;
		long long tile = -1;
		unsigned int todo;
		if (!ring) {
			// phase B: PF_EVAL_TILE_CHUNK consecutive tiles, within one claim word
			const unsigned int t0 = chunk;
			const unsigned int left = n_tiles - t0;
			const unsigned int n = left < (unsigned int)PF_EVAL_TILE_CHUNK ? left : (unsigned int)PF_EVAL_TILE_CHUNK;
			const unsigned int sh = t0 & 31;
			const unsigned int bits = n >= 32 ? 0xffffffffu : ((1u << n) - 1u) << sh;
			unsigned int old = 0;
			if (lane == 0) old = atomicOr(&claims[t0 >> 5], bits);
			todo = (bits & ~__shfl_sync(0xffffffffu, old, 0)) >> sh;
			tile = (long long)t0 + lane;
		}
		else {
			tile = lane < PF_EVAL_RING_CHUNK ? ring_tile(models, profs, n_profiles, chunk + (unsigned int)lane) : -1;
			bool mine = false;
			if (tile >= 0) {
				const unsigned int bit = 1u << (tile & 31);
				mine = (atomicOr(&claims[tile >> 5], bit) & bit) == 0;
			}
			todo = __ballot_sync(0xffffffffu, mine);
		}
		while (todo) {
			const int src = __ffs(todo) - 1;
			const long long t = __shfl_sync(0xffffffffu, tile, src);
			mi = find_model_from(models, n_models, t, mi);
			const ModelDev &m = models[mi];
			const unsigned int local = (unsigned int)(t - m.tile_base);
			const int row = (int)(local / m.tiles_per_row);
			const int tc = (int)(local - (unsigned int)row * m.tiles_per_row);
			int nt = 1;
			unsigned int own = 1u;
			if (!ring) {
				// phase B: with it, the claim's next tiles of the same row (the
				// claim's tiles are consecutive), up to kSegTiles, those it owns
				const int span = min(min(kSegTiles, (int)m.tiles_per_row - tc), 32 - src);
				own = (todo >> src) & (span >= 32 ? 0xffffffffu : ((1u << span) - 1u));
				nt = 32 - __clz(own);
				todo &= ~(own << src);
			}
			else {
				// phase A: with it, the same item's next ring tiles (lanes 4g ..
				// 4g + 3 hold one profile's ring row, consecutive tile columns)
				const int span = min(kRingCols - src % kRingCols, kSegTiles);
				own = (todo >> src) & ((1u << span) - 1u);
				nt = 32 - __clz(own);
				todo &= ~(own << src);
			}
			eval_seg<KINDS, SPLIT>(models, mi, profs, psf_pool, conv_img, direct_img, row, tc, nt, own, ws, ss, lane,
			                       dbg, pool);
		}
	}
}

// Lane 0, box b of root r finished with value v (deepest level + 1 reached:
// deepest): its value stored; the warp that finishes the root's last box forms
// the pixel value in the walk's order (the level-0 box's accepted points, then
// the boxes in ascending sub-point order) and, if it finishes the pixel's last
// split profile, writes the pixel's canvas values.
__device__ void finish_split_box(const SplitPool &pool, unsigned int b, int r, float v, int deepest,
                                 float *__restrict__ conv_img, float *__restrict__ direct_img, const DebugRec &dbg)
{
	pool.box_val[b] = v;
	SplitRoot &R = pool.root[r];
	atomicMax(&R.depth, deepest);
	__threadfence();
	if (atomicSub(&R.pending, 1u) != 1u) return;
	__threadfence();
	const volatile float *vals = pool.box_val + R.first_box;
	float total = R.accepted;
	for (unsigned int j = 0; j < R.n_boxes; j++) total += vals[j];
	const float value = R.fflux * (total * __frcp_rn((float)(R.res * R.res)));
	*(volatile float *)&R.value = value;
	if (R.depth_idx >= 0) dbg.depth[R.depth_idx] = (int8_t)atomicAdd(&R.depth, 0);
	__threadfence();
	SplitPixel &X = pool.pix[R.pixel];
	if (atomicSub(&X.pending, 1u) != 1u) return;
	__threadfence();
	float c = X.s_conv, d = X.s_direct;
	for (int q = X.first_root; q >= 0; q = pool.root[q].next) {
		const float val = *(volatile const float *)&pool.root[q].value;
		if (pool.root[q].convolve) c += val;
		else d += val;
	}
	if (X.conv_required) conv_img[X.idx] = c;
	if (X.direct_required) direct_img[X.idx] = d;
}

// The split-off boxes (SplitPool), one per warp, each walked depth first
// below its level; taken one at a time from the pool's work counter.
template <unsigned int KINDS>
__global__ void __launch_bounds__(kWarps32 * 32, PF_EVAL32_SPLIT_MIN_BLOCKS)
split_boxes32_kernel(const ProfileDev *__restrict__ profs, float *__restrict__ conv_img,
                     float *__restrict__ direct_img, SplitPool pool, DebugRec dbg)
{
	__shared__ WarpScratchM scratch[kWarps32];
	const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
	WarpScratchM &ws = scratch[warp];
	// final: the evaluation kernel, launched before, allocated them
	const unsigned int n_boxes = min(*(volatile unsigned int *)&pool.cnt[0], pool.cap_box);
	while (true) {
		unsigned int b = 0;
		if (lane == 0) b = atomicAdd(&pool.cnt[3], 1u);
		b = __shfl_sync(0xffffffffu, b, 0);
		if (b >= n_boxes) break;
		const SplitBox bx = pool.box[b];
		const int pi = pool.root[bx.root].profile;
		const ProfileDev &P = profs[pi];
		const f32::Shape sh = f32::load_shape(P);
		const unsigned int res = bx.meta & 0xffu, level = (bx.meta >> 8) & 0xffu, max_rec = bx.meta >> 16;
		unsigned long long *counts = dbg.counts ? dbg.counts + (size_t)pi * kLevelCounts : nullptr;
		set_frame(ws, (int)level, bx.xhi, bx.xlo, bx.yhi, bx.ylo, bx.bx, bx.by, lane);
		eval_frame_m<KINDS>(P, sh, ws, (int)level, res, __frcp_rn((float)res), max_rec, lane, counts);
		int deepest = 0;
		const float v = warp_walk_m<KINDS>(P, sh, ws, (int)level, res, max_rec, lane, counts, deepest);
		if (lane == 0) finish_split_box(pool, b, bx.root, v, deepest, conv_img, direct_img, dbg);
		__syncwarp();
	}
}

__global__ void psf_to_float_kernel(const double *in, float *out, long long n)
{
	for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
		out[i] = (float)in[i];
}

}  // namespace

void launch_eval32(const ModelDev *models, int n_models, const ProfileDev *profs, int n_profiles,
                   const double *psf_pool, float *conv_img, float *direct_img, long long n_tiles,
                   unsigned int *counter, unsigned int *claims, DebugRec dbg, const SplitPool &pool, bool sersic_only,
                   int n_sm, cudaStream_t stream)
{
	const unsigned int n_ring = (unsigned int)n_profiles * kRingRows * kRingCols;
	// persistent kernels: as many blocks as fit at once
	const int blocks = n_sm * (pool.box ? PF_EVAL32_SPLIT_MIN_BLOCKS : PF_EVAL32_MIN_BLOCKS);
	// kernels without the split path where the batch does not split: it costs
	// the walk registers (measured 2.79 against 3.10 ms for the 1024-model step)
	if (sersic_only) {
		if (pool.box) {
			eval_tiles32_kernel<f32::kSersicOnly, true><<<blocks, kWarps32 * 32, 0, stream>>>(
			    models, n_models, profs, (unsigned int)n_profiles, psf_pool, conv_img, direct_img,
			    (unsigned int)n_tiles, n_ring, counter, claims, dbg, pool);
			split_boxes32_kernel<f32::kSersicOnly><<<blocks, kWarps32 * 32, 0, stream>>>(profs, conv_img, direct_img,
			                                                                             pool, dbg);
		}
		else {
			eval_tiles32_kernel<f32::kSersicOnly, false><<<blocks, kWarps32 * 32, 0, stream>>>(
			    models, n_models, profs, (unsigned int)n_profiles, psf_pool, conv_img, direct_img,
			    (unsigned int)n_tiles, n_ring, counter, claims, dbg, pool);
		}
	}
	else {
		if (pool.box) {
			eval_tiles32_kernel<f32::kAllKinds, true><<<blocks, kWarps32 * 32, 0, stream>>>(
			    models, n_models, profs, (unsigned int)n_profiles, psf_pool, conv_img, direct_img,
			    (unsigned int)n_tiles, n_ring, counter, claims, dbg, pool);
			split_boxes32_kernel<f32::kAllKinds><<<blocks, kWarps32 * 32, 0, stream>>>(profs, conv_img, direct_img,
			                                                                          pool, dbg);
		}
		else {
			eval_tiles32_kernel<f32::kAllKinds, false><<<blocks, kWarps32 * 32, 0, stream>>>(
			    models, n_models, profs, (unsigned int)n_profiles, psf_pool, conv_img, direct_img,
			    (unsigned int)n_tiles, n_ring, counter, claims, dbg, pool);
		}
	}
}

long long eval32_items(long long n_profiles, long long n_tiles)
{
	return n_profiles * kRingRows * kRingCols + n_tiles;
}

void launch_psf_to_float(const double *in, float *out, long long n, cudaStream_t stream)
{
	if (n <= 0) return;
	psf_to_float_kernel<<<(int)((n + 255) / 256 < 4096 ? (n + 255) / 256 : 4096), 256, 0, stream>>>(in, out, n);
}

}  // namespace pf
