// Plain FP64 path: the reference's arithmetic on the GPU.
//
// eval_tiles64 renders every profile of every model of a batch into the
// drawing areas: one warp per tile of 32 pixels of a row, profiles in model
// order, so each pixel accumulates exactly as Model::produce_image does
// (src/model.cpp:332-346; "image[i] += flux_scale * pixel_val" per profile,
// src/radial.cpp:341). Pixels that RadialProfile::evaluate_cpu would
// subsample (src/radial.cpp:323-339) are integrated by the whole warp: the
// res x res sub-points of a box are spread over the lanes, every sub-point
// gets its value and accuracy test as in subsample_pixel
// (src/radial.cpp:55-135), failing sub-points are visited depth-first in the
// reference's order, and each box's total is formed by one lane in the
// reference's summation order. The recursion tree is recomputed on the device
// instead of being shipped through the host level by level as the OpenCL
// path does (src/radial.cpp:567-673).
//
// finish64 produces the output image: model_image + (to_convolve convolved
// with the PSF) (src/model.cpp:344-356), the convolution done directly with
// the associative brute-force summation order (row dot products,
// src/convolve.cpp:158-231) but only for the pixels that survive the crop of
// the PSF padding (src/model.cpp:288-306), then Image::downsample(SUM)
// (src/image.cpp:250-262) when the model is finesampled and not returned so.
//
// Compiled with -fmad=false (no contraction, like the reference's x86-64 build).
#include <cstdint>

#include "pf_device.cuh"
#include "profiles_f64.cuh"
#include "psf_profile.cuh"

namespace pf {

namespace {

constexpr int kWarps64 = 4;

struct Frame64 {
	double x0, x1, y0, y1;
	double hx, hy;
	double total;
	unsigned int mask[kMaskWords];
};

struct WarpScratch64 {
	Frame64 fr[kMaxLevels];
	double vals[kMaxRes * kMaxRes];
};

// Coordinate of sub-point i of a box starting at x0 with half bin h: the
// reference advances x by h twice per sub-point and uses it after the first
// advance (src/radial.cpp:83-108), i.e. 2i+1 successive additions.
__device__ __forceinline__ double sub_coord(double x0, double h, unsigned int i)
{
	double x = x0;
	for (unsigned int t = 0; t < 2 * i + 1; t++) {
		x += h;
	}
	return x;
}

// Evaluates all sub-points of box fr[L]; leaves the non-failing total and the
// failing-point mask in fr[L].
__device__ void eval_frame64(const ProfileDev &P, WarpScratch64 &ws, int L, unsigned int res,
                             unsigned int max_rec, int lane, unsigned long long *counts)
{
	Frame64 &f = ws.fr[L];
	const double x0 = f.x0, x1 = f.x1, y0 = f.y0, y1 = f.y1;
	const double xbin = (x1 - x0) / res;
	const double ybin = (y1 - y0) / res;
	const double hx = xbin / 2.;
	const double hy = ybin / 2.;
	const bool recurse = res > 1 && (unsigned int)L < max_rec;
	const unsigned int n = res * res;
	if (counts && lane == 0 && L < kLevelCounts) {
		atomicAdd(&counts[L], 1ull);
		atomicAdd(&counts[kCountSubEvals], (unsigned long long)(recurse ? 2 * n : n));
	}
	for (unsigned int base = 0; base < n; base += 32) {
		const unsigned int idx = base + lane;
		bool fail = false;
		if (idx < n) {
			const unsigned int i = idx / res, j = idx % res;
			const double x = sub_coord(x0, hx, i);
			const double y = sub_coord(y0, hy, j);
			double xp, yp;
			f64::to_profile(P, x, y, xp, yp);
			const double subval = f64::evaluate_at(P, xp, yp);
			if (recurse) {
				const double dyp = (-xbin * P.sin_ang + ybin * P.cos_ang) / P.par[PF_P_AXRAT];
				const double testval = f64::evaluate_at(P, fabs(xp), fabs(yp) + fabs(dyp));
				fail = fabs(testval / subval - 1.0) > P.acc;
			}
			ws.vals[idx] = subval;
		}
		const unsigned int word = __ballot_sync(0xffffffffu, fail);
		if (lane == 0) {
			f.mask[base >> 5] = word;
		}
	}
	__syncwarp();
	if (lane == 0) {
		double total = 0;
		for (unsigned int idx = 0; idx < n; idx++) {
			if (!((f.mask[idx >> 5] >> (idx & 31)) & 1u)) {
				total += ws.vals[idx];
			}
		}
		f.total = total;
		f.hx = hx;
		f.hy = hy;
	}
	__syncwarp();
}

// subsample_pixel(x0, x1, y0, y1, L0, max_rec, res) computed by the whole
// warp (L0 = 0: a drawing pixel's box); deepest: the deepest level + 1.
__device__ double warp_subsample64(const ProfileDev &P, WarpScratch64 &ws, double x0, double x1, double y0,
                                   double y1, unsigned int res, unsigned int max_rec, int lane,
                                   unsigned long long *counts, int &deepest, int L0 = 0)
{
	if (lane == 0) {
		ws.fr[L0].x0 = x0;
		ws.fr[L0].x1 = x1;
		ws.fr[L0].y0 = y0;
		ws.fr[L0].y1 = y1;
	}
	__syncwarp();
	int L = L0;
	deepest = L0 + 1;
	eval_frame64(P, ws, L0, res, max_rec, lane, counts);
	const unsigned int nwords = (res * res + 31) / 32;
	while (true) {
		Frame64 &f = ws.fr[L];
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
			const unsigned int i = (unsigned int)k / res, j = (unsigned int)k % res;
			const double x = sub_coord(f.x0, f.hx, i);
			const double y = sub_coord(f.y0, f.hy, j);
			if (lane == 0) {
				f.mask[k >> 5] &= ~(1u << (k & 31));
				Frame64 &c = ws.fr[L + 1];
				c.x0 = x - f.hx;
				c.x1 = x + f.hx;
				c.y0 = y - f.hy;
				c.y1 = y + f.hy;
			}
			__syncwarp();
			L++;
			if (L + 1 > deepest) deepest = L + 1;
			eval_frame64(P, ws, L, res, max_rec, lane, counts);
		}
		else {
			const double v = f.total / (res * res);
			if (L == L0) {
				return v;
			}
			L--;
			if (lane == 0) {
				ws.fr[L].total += v;
			}
			__syncwarp();
		}
	}
}

// A subsampled drawing pixel's level-0 box exported to the level pool (lane
// by lane, no warp cooperation): the box, its LevelRoot64, and on the pixel's
// first export its LevelPixel64; the pixel's earlier subsampled profile (plast)
// chained to it. False, with nothing to do for the caller but to walk the
// tree itself, when the pool has no room.
__device__ bool export_root64(const LevelPool64 &pool, const ProfileDev &P, int pi, const ModelDev &m, double x0,
                              double x1, double y0, double y1, unsigned int res, unsigned int max_rec,
                              long long canvas_idx, long long depth_idx, int &prec, int &plast, unsigned int &nroots)
{
	const unsigned int n = res * res;
	const unsigned int b = atomicAdd(&pool.cnt[LC_BOX], 1u);
	if (b >= pool.cap_box) {
		atomicAdd(&pool.cnt[LC_REFUSED], 1u);
		return false;
	}
	bool ok = true;
	const unsigned long long vo = atomicAdd((unsigned long long *)&pool.cnt[LC_VAL], (unsigned long long)n);
	if (vo + n > pool.cap_val) ok = false;
	int r = -1, p = prec;
	if (ok) {
		const unsigned int q = atomicAdd(&pool.cnt[LC_ROOT], 1u);
		if (q < pool.cap_root) r = (int)q;
		else ok = false;
	}
	if (ok && p < 0) {
		const unsigned int q = atomicAdd(&pool.cnt[LC_PIX], 1u);
		if (q < pool.cap_pix) p = (int)q;
		else ok = false;
	}
	LevelBox64 &B = pool.box[b];
	if (!ok) {
		B.meta = kDeadBox;
		atomicAdd(&pool.cnt[LC_REFUSED], 1u);
		return false;
	}
	B.x0 = x0;
	B.x1 = x1;
	B.y0 = y0;
	B.y1 = y1;
	B.accepted = 0.;
	B.value = 0.;
	B.profile = pi;
	B.parent = -1;
	B.rank = 0;
	B.meta = res | (max_rec << 16);
	B.pending = (n + kChunk64 - 1) / kChunk64;
	B.first_child = 0;
	B.n_children = 0;
	B.root = r;
	B.val_off = vo;
	for (int w = 0; w < kMaskWords; w++) B.mask[w] = 0;
	LevelRoot64 &R = pool.root[r];
	R.flux_scale = P.flux_scale;
	R.value = 0.;
	R.pixel = p;
	R.next = -1;
	R.convolve = P.convolve;
	R.deepest = 1;
	R.depth_idx = depth_idx;
	if (prec < 0) {
		LevelPixel64 &X = pool.pix[p];
		X.idx = canvas_idx;
		X.s_conv = X.s_direct = 0.;
		X.first_root = r;
		X.pending = 0;
		X.conv_required = m.conv_required;
	}
	else {
		pool.root[plast].next = r;
	}
	prec = p;
	plast = r;
	nroots++;
	return true;
}

// The end of a block of the tile kernel (k = 0) or of the level-(k-1)
// kernel: the grid's last block to get here records where the boxes it
// allocated end (bound[k + 1]). No block waits for another.
__device__ void level_block_done(const LevelPool64 &pool, int k)
{
	__syncthreads();
	if (threadIdx.x == 0) {
		__threadfence();
		if (atomicAdd(&pool.cnt[LC_DONE + k], 1u) == gridDim.x - 1) {
			__threadfence();
			pool.cnt[LC_BOUND + k + 1] = min(atomicAdd(&pool.cnt[LC_BOX], 0u), pool.cap_box);
		}
	}
}

template <bool SPLIT>
__global__ void __launch_bounds__(kWarps64 * 32)
eval_tiles64_kernel(const ModelDev *__restrict__ models, int n_models, const ProfileDev *__restrict__ profs,
                    const double *__restrict__ psf_pool, double *__restrict__ conv_img,
                    double *__restrict__ direct_img, long long n_tiles, unsigned int *tile_counter,
                    DebugRec dbg, LevelPool64 pool)
{
	__shared__ WarpScratch64 scratch[kWarps64];
	const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
	WarpScratch64 &ws = scratch[warp];
	while (true) {
		unsigned int t = 0;
		if (lane == 0) {
			t = atomicAdd(tile_counter, 1u);
		}
		const long long tile = (long long)__shfl_sync(0xffffffffu, t, 0);
		if (tile >= n_tiles) {
			break;
		}
		const int mi = find_model(models, n_models, tile);
		const ModelDev &m = models[mi];
		const long long local = tile - m.tile_base;
		const unsigned int row = (unsigned int)(local / m.tiles_per_row);
		const int col0 = (int)(local % m.tiles_per_row) * 32;
		const int col1 = min(col0 + 31, (int)m.draw_w - 1);
		const unsigned int px = (unsigned int)col0 + lane;
		const bool active = px < m.draw_w;
		const bool in_mask = active && evaluated(m, (int)px, (int)row);  // the calculation mask (radial, sky)
		const double sx = m.sx, sy = m.sy;
		const double half_xbin = sx / 2.;
		const double half_ybin = sy / 2.;
		const double *psf = m.psf_off >= 0 ? psf_pool + m.psf_off : nullptr;
		const long long canvas_idx = (long long)m.draw_off + (long long)row * m.draw_w + px;
		double acc_conv = 0, acc_direct = 0;
		int prec = -1, plast = -1;  // this pixel's LevelPixel64 and last LevelRoot64
		unsigned int nroots = 0;

		for (int q0 = 0; q0 < m.n_profiles; q0 += 32) {
			// 32 profiles' culling boxes tested at once, one per lane; the ones
			// that reach this tile drawn one by one, in profile order
			const bool reaches = profile_reaches(profs, m, q0 + lane, (int)row, col0, col1);
			unsigned int todo = __ballot_sync(0xffffffffu, reaches);
			while (todo) {
				const int q = q0 + __ffs(todo) - 1;
				todo &= todo - 1;
				const int pi = m.first_profile + q;
				const ProfileDev &P = profs[pi];
				double add = 0;
				bool has = false;
				if (P.kind == PF_SKY) {
					add = P.bg;
					has = in_mask;  // src/sky.cpp:42-45
				}
				else if (P.kind == PF_PSF) {
					if (active && psf) {
						has = psf_pixel64(P, m, psf, px, row, add);
					}
				}
				else if (is_radial(P.kind)) {
					const double y = half_ybin + row * sy;
					const double x = half_xbin + px * sx;
					double xp, yp;
					f64::to_profile(P, x, y, xp, yp);
					const double r_prof = sqrt(xp * xp + yp * yp);
					double pixel_val = 0;
					int depth = 0;
					bool need_ss = false, split = false;
					if (!in_mask || (P.rscale_max > 0 && r_prof / P.rscale > P.rscale_max)) {
						// masked out (src/radial.cpp:305-307) or beyond rscale_max
						pixel_val = 0.;
						depth = -1;
					}
					else if (P.rough || r_prof / P.rscale > P.rscale_switch) {
						pixel_val = f64::evaluate_at(P, xp, yp);
					}
					else {
						need_ss = true;
					}
					unsigned long long *counts = dbg.counts ? dbg.counts + (size_t)pi * kLevelCounts : nullptr;
					if (counts) {
						const unsigned int nd = __popc(__ballot_sync(0xffffffffu, active && depth == 0 && !need_ss));
						if (lane == 0 && nd) atomicAdd(&counts[kCountDirectEvals], (unsigned long long)nd);
					}
					// the pixel's subsampling parameters (src/sersic.cpp:331-347 for the central pixel)
					unsigned int res = P.resolution, max_rec = P.max_recursions;
					if (P.kind == PF_SERSIC) {
						const bool center_pixel = fabs(x - P.xc) < m.scale_x && fabs(y - P.yc) < m.scale_y;
						if (P.adjust && center_pixel && P.par[7] > 1) {
							res = 8;
							max_rec = 10;
						}
					}
					if (res > (unsigned int)kMaxRes) res = kMaxRes;
					if (max_rec > (unsigned int)kMaxLevels - 1) max_rec = kMaxLevels - 1;
					if constexpr (SPLIT) {
						// the tree goes to the level kernels; walked here only when the pool is full
						if (need_ss && active &&
						    export_root64(pool, P, pi, m, x - half_xbin, x + half_xbin, y - half_ybin, y + half_ybin,
						                  res, max_rec, canvas_idx,
						                  dbg.depth ? P.depth_off + (long long)row * m.draw_w + px : -1, prec, plast,
						                  nroots)) {
							need_ss = false;
							split = true;
						}
					}
					unsigned int pending = __ballot_sync(0xffffffffu, need_ss && active);
					while (pending) {
						const int s = __ffs(pending) - 1;
						pending &= pending - 1;
						const double xs = __shfl_sync(0xffffffffu, x, s);
						const double ys = __shfl_sync(0xffffffffu, y, s);
						const unsigned int sres = __shfl_sync(0xffffffffu, res, s);
						const unsigned int smax = __shfl_sync(0xffffffffu, max_rec, s);
						int deepest = 0;
						const double v = warp_subsample64(P, ws, xs - half_xbin, xs + half_xbin, ys - half_ybin,
						                                  ys + half_ybin, sres, smax, lane, counts, deepest);
						if (lane == s) {
							pixel_val = v;
							depth = deepest;
						}
					}
					if (dbg.depth && active && !split) {
						dbg.depth[P.depth_off + (size_t)row * m.draw_w + px] = (int8_t)depth;
					}
					add = P.flux_scale * pixel_val;
					has = active && !split;  // a subsampled profile's value is added when its tree completes
				}
				if (has) {
					if (P.convolve) acc_conv += add;
					else acc_direct += add;
				}
			}
		}
		if (active) {
			if (SPLIT && prec >= 0) {
				// the pixel's subsampled profiles still to come: the warp that
				// completes the last of them writes the canvas
				LevelPixel64 &X = pool.pix[prec];
				X.s_conv = acc_conv;
				X.s_direct = acc_direct;
				X.pending = nroots;
			}
			else {
				if (m.conv_required) conv_img[canvas_idx] = acc_conv;
				direct_img[canvas_idx] = acc_direct;
			}
		}
	}
	if constexpr (SPLIT) level_block_done(pool, 0);
}

// Lane 0: box b complete with value v. Its value stored; the warp that
// completes a box's last child forms that box's value as the depth-first walk
// does (accepted sum, then the children's values in ascending order, over
// res^2), up to the level-0 box, whose profile value (flux_scale x the pixel
// value, src/radial.cpp:341) goes to its LevelRoot64; the warp that completes
// a pixel's last subsampled profile writes the pixel's canvas values: the
// tile's sums of its other profiles, then the subsampled ones in profile
// order.
__device__ void complete_box64(const LevelPool64 &pool, unsigned int b, double v, double *__restrict__ conv_img,
                               double *__restrict__ direct_img, const DebugRec &dbg)
{
	while (true) {
		LevelBox64 &B = pool.box[b];
		const int p = B.parent;
		if (p < 0) break;
		B.value = v;
		__threadfence();
		LevelBox64 &Q = pool.box[p];
		if (atomicSub(&Q.pending, 1u) != 1u) return;
		__threadfence();
		const unsigned int res = Q.meta & 0xffu;
		const unsigned int c0 = __ldcg(&Q.first_child), nc = __ldcg(&Q.n_children);
		double total = __ldcg(&Q.accepted);
		for (unsigned int r = 0; r < nc; r++) total += __ldcg(&pool.box[c0 + r].value);
		v = total / (res * res);
		b = (unsigned int)p;
	}
	LevelRoot64 &R = pool.root[pool.box[b].root];
	R.value = R.flux_scale * v;
	if (R.depth_idx >= 0) dbg.depth[R.depth_idx] = (int8_t)atomicAdd(&R.deepest, 0);
	__threadfence();
	LevelPixel64 &X = pool.pix[R.pixel];
	if (atomicSub(&X.pending, 1u) != 1u) return;
	__threadfence();
	double c = __ldcg(&X.s_conv), d = __ldcg(&X.s_direct);
	for (int q = __ldcg(&X.first_root); q >= 0; q = __ldcg(&pool.root[q].next)) {
		const double val = __ldcg(&pool.root[q].value);
		if (__ldcg(&pool.root[q].convolve)) c += val;
		else d += val;
	}
	if (X.conv_required) conv_img[X.idx] = c;
	direct_img[X.idx] = d;
}

// The warp that evaluated the last sub-points of level-L box b: the accepted
// values summed in index order; the failing sub-points' boxes allocated at
// level L + 1 in ascending order (or, without room, walked here in that order
// and added); a box with none complete.
__device__ void reduce_box64(const LevelPool64 &pool, const ProfileDev &P, unsigned int b, int level,
                             WarpScratch64 &ws, int lane, double *__restrict__ conv_img,
                             double *__restrict__ direct_img, const DebugRec &dbg)
{
	LevelBox64 &B = pool.box[b];
	const unsigned int res = B.meta & 0xffu, max_rec = B.meta >> 16, n = res * res;
	const unsigned int nwords = (n + 31) / 32;
	const unsigned long long vo = B.val_off;
	for (unsigned int k = lane; k < n; k += 32) ws.vals[k] = __ldcg(&pool.val[vo + k]);
	unsigned int nf = 0;
	for (unsigned int w = 0; w < nwords; w++) {
		ws.fr[0].mask[w] = __ldcg(&B.mask[w]);
		nf += __popc(ws.fr[0].mask[w]);
	}
	__syncwarp();
	unsigned long long *counts = dbg.counts ? dbg.counts + (size_t)B.profile * kLevelCounts : nullptr;
	const bool recurse = res > 1 && (unsigned int)level < max_rec;
	double total = 0;
	if (lane == 0) {
		for (unsigned int k = 0; k < n; k++) {
			if (!((ws.fr[0].mask[k >> 5] >> (k & 31)) & 1u)) total += ws.vals[k];
		}
		if (counts && level < kLevelCounts) {
			atomicAdd(&counts[level], 1ull);
			atomicAdd(&counts[kCountSubEvals], (unsigned long long)(recurse ? 2 * n : n));
		}
		if (dbg.depth) atomicMax(&pool.root[B.root].deepest, level + 1);
	}
	if (nf == 0) {
		if (lane == 0) complete_box64(pool, b, total / (res * res), conv_img, direct_img, dbg);
		return;
	}
	unsigned int b0 = 0, ok = 0;
	unsigned long long c_vo = 0;
	if (lane == 0) {
		b0 = atomicAdd(&pool.cnt[LC_BOX], nf);
		ok = b0 < pool.cap_box && pool.cap_box - b0 >= nf;
		if (ok) {
			c_vo = atomicAdd((unsigned long long *)&pool.cnt[LC_VAL], (unsigned long long)nf * n);
			ok = c_vo + (unsigned long long)nf * n <= pool.cap_val;
		}
		if (!ok) atomicAdd(&pool.cnt[LC_REFUSED], 1u);
	}
	ok = __shfl_sync(0xffffffffu, ok, 0);
	b0 = __shfl_sync(0xffffffffu, b0, 0);
	c_vo = __shfl_sync(0xffffffffu, c_vo, 0);
	const double x0 = B.x0, x1 = B.x1, y0 = B.y0, y1 = B.y1;
	const double hx = (x1 - x0) / res / 2., hy = (y1 - y0) / res / 2.;
	if (!ok) {
		// no room: the allocated part marked dead, the subtrees walked here
		for (unsigned int d = b0 + lane; d < b0 + nf && d < pool.cap_box; d += 32) pool.box[d].meta = kDeadBox;
		int deepest_all = level + 1;
		for (unsigned int w = 0; w < nwords; w++) {
			unsigned int bits = ws.fr[0].mask[w];
			while (bits) {
				const unsigned int k = w * 32 + __ffs(bits) - 1;
				bits &= bits - 1;
				const unsigned int i = k / res, j = k % res;
				const double x = sub_coord(x0, hx, i), y = sub_coord(y0, hy, j);
				int deepest = 0;
				const double v = warp_subsample64(P, ws, x - hx, x + hx, y - hy, y + hy, res, max_rec, lane, counts,
				                                  deepest, level + 1);
				if (deepest > deepest_all) deepest_all = deepest;
				total += v;
			}
		}
		if (lane == 0) {
			if (dbg.depth) atomicMax(&pool.root[B.root].deepest, deepest_all);
			complete_box64(pool, b, total / (res * res), conv_img, direct_img, dbg);
		}
		return;
	}
	if (lane == 0) {
		B.accepted = total;
		B.first_child = b0;
		B.n_children = nf;
		B.pending = nf;
	}
	const uint32_t meta = res | ((unsigned int)(level + 1) << 8) | (max_rec << 16);
	unsigned int rank = 0;
	for (unsigned int w = 0; w < nwords; w++) {
		const unsigned int bits = ws.fr[0].mask[w];
		if ((bits >> lane) & 1u) {
			const unsigned int k = w * 32 + (unsigned int)lane;
			const unsigned int rk = rank + __popc(bits & ((1u << lane) - 1u));
			const unsigned int i = k / res, j = k % res;
			const double x = sub_coord(x0, hx, i), y = sub_coord(y0, hy, j);
			LevelBox64 &C = pool.box[b0 + rk];
			C.x0 = x - hx;
			C.x1 = x + hx;
			C.y0 = y - hy;
			C.y1 = y + hy;
			C.accepted = 0.;
			C.value = 0.;
			C.profile = B.profile;
			C.parent = (int)b;
			C.rank = rk;
			C.meta = meta;
			C.pending = (n + kChunk64 - 1) / kChunk64;
			C.first_child = 0;
			C.n_children = 0;
			C.root = B.root;
			C.val_off = c_vo + (unsigned long long)rk * n;
			for (int q = 0; q < kMaskWords; q++) C.mask[q] = 0;
		}
		rank += __popc(bits);
	}
}

// Recursion level `level` of every exported tree: item (box, chunk) of the
// boxes allocated for this level, kMaxRes^2 / kChunk64 chunk slots per box;
// lane pair 2s, 2s + 1 of a chunk's warp evaluates sub-point 16 c + s and its
// accuracy test (src/radial.cpp:83-121).
__global__ void __launch_bounds__(kWarps64 * 32)
level64_kernel(const ProfileDev *__restrict__ profs, double *__restrict__ conv_img, double *__restrict__ direct_img,
               LevelPool64 pool, int level, DebugRec dbg)
{
	constexpr int kSlots = kMaxRes * kMaxRes / kChunk64;
	__shared__ WarpScratch64 scratch[kWarps64];
	const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
	WarpScratch64 &ws = scratch[warp];
	const unsigned int lo = *(volatile unsigned int *)&pool.cnt[LC_BOUND + level];
	const unsigned int hi = *(volatile unsigned int *)&pool.cnt[LC_BOUND + level + 1];
	if (hi <= lo) {
		// no box at this level, so none deeper: the next level's (empty)
		// range recorded without the blocks' completion count
		if (blockIdx.x == 0 && threadIdx.x == 0) pool.cnt[LC_BOUND + level + 2] = hi;
		return;
	}
	// chunk-major items (every box's chunk 0, then every box's chunk 1, ...):
	// the real chunks (res^2 / 16 of a box's kSlots) come first and fill the
	// grid's warps in one pass
	const unsigned int nb = hi - lo;
	const long long n_items = (long long)nb * kSlots;
	for (long long item = (long long)blockIdx.x * kWarps64 + warp; item < n_items;
	     item += (long long)gridDim.x * kWarps64) {
		const unsigned int b = lo + (unsigned int)(item % nb);
		const unsigned int c = (unsigned int)(item / nb);
		LevelBox64 &B = pool.box[b];
		const uint32_t meta = B.meta;
		if (meta == kDeadBox) continue;
		const unsigned int res = meta & 0xffu, max_rec = meta >> 16, n = res * res;
		if (c * kChunk64 >= n) continue;
		const ProfileDev &P = profs[B.profile];
		const double x0 = B.x0, x1 = B.x1, y0 = B.y0, y1 = B.y1;
		const double xbin = (x1 - x0) / res;
		const double ybin = (y1 - y0) / res;
		const double hx = xbin / 2.;
		const double hy = ybin / 2.;
		const bool recurse = res > 1 && (unsigned int)level < max_rec;
		const unsigned int s = (unsigned int)lane >> 1, e = (unsigned int)lane & 1u;
		const unsigned int k = c * kChunk64 + s;
		double val = 0.;
		if (k < n && (e == 0 || recurse)) {
			const unsigned int i = k / res, j = k % res;
			const double x = sub_coord(x0, hx, i);
			const double y = sub_coord(y0, hy, j);
			double xp, yp;
			f64::to_profile(P, x, y, xp, yp);
			if (e) {  // the test point, displaced by one sub-bin along the profile's minor axis
				const double dyp = (-xbin * P.sin_ang + ybin * P.cos_ang) / P.par[PF_P_AXRAT];
				xp = fabs(xp);
				yp = fabs(yp) + fabs(dyp);
			}
			val = f64::evaluate_at(P, xp, yp);
		}
		const double testval = __shfl_down_sync(0xffffffffu, val, 1);
		const bool fail = e == 0 && k < n && recurse && fabs(testval / val - 1.0) > P.acc;
		if (e == 0 && k < n) pool.val[B.val_off + k] = val;
		const unsigned int bits = __reduce_or_sync(0xffffffffu, fail ? 1u << s : 0u);
		if (lane == 0 && bits) atomicOr(&B.mask[(c * kChunk64) >> 5], bits << ((c * kChunk64) & 31));
		__threadfence();
		__syncwarp();
		unsigned int last = 0;
		if (lane == 0) last = atomicSub(&B.pending, 1u) == 1u;
		if (!__shfl_sync(0xffffffffu, last, 0)) continue;
		__threadfence();
		reduce_box64(pool, P, b, level, ws, lane, conv_img, direct_img, dbg);
		__syncwarp();
	}
	level_block_done(pool, level + 1);
}

__device__ __forceinline__ int find_model_out(const ModelDev *models, int n_models, long long g)
{
	int lo = 0, hi = n_models - 1;
	while (lo < hi) {
		int mid = (lo + hi + 1) >> 1;
		if (models[mid].out_off <= g) lo = mid; else hi = mid - 1;
	}
	return lo;
}

// Associative brute-force convolution of one pixel (src/convolve.cpp:158-231):
// row dot products of the source against the reversed kernel, zero outside.
__device__ __forceinline__ double conv_pixel64(const double *src, unsigned int src_width, unsigned int src_height,
                                               const double *krn, unsigned int krn_width, unsigned int krn_height,
                                               unsigned int dx, unsigned int dy)
{
	const unsigned int krn_half_width = krn_width / 2, krn_half_height = krn_height / 2;
	unsigned int l_min = 0, l_max = krn_height, k_min = 0, k_max = krn_width;
	if (dy < krn_half_height) l_min = krn_half_height - dy;
	else if ((dy + krn_half_height) >= src_height) l_max = src_height + krn_half_height - dy;
	if (dx < krn_half_width) k_min = krn_half_width - dx;
	else if ((dx + krn_half_width) >= src_width) k_max = src_width + krn_half_width - dx;
	const long long kn = (long long)krn_width * krn_height;
	double pixel = 0;
	for (unsigned int l = l_min; l < l_max; l++) {
		// row l of the reversed kernel against the matching source row
		const long long srow = (long long)(dy + l - krn_half_height) * src_width + (long long)dx - krn_half_width;
		const long long krow = kn - 1 - (long long)l * krn_width;
		double dot = 0;
		for (unsigned int k = k_min; k < k_max; k++) {
			dot += src[srow + k] * krn[krow - k];
		}
		pixel += dot;
	}
	return pixel;
}

// One drawing pixel of the final model image: model_image + convolved
// to_convolve, the convolution zero where the calculation mask is
// (Convolver::convolve with a mask, src/convolve.cpp:55-99).
__device__ __forceinline__ double drawn_pixel64(const ModelDev &m, const double *psf, const double *conv_img,
                                                const double *direct_img, unsigned int dx, unsigned int dy)
{
	double v = direct_img[m.draw_off + (size_t)dy * m.draw_w + dx];
	if (m.conv_required && evaluated(m, (int)dx, (int)dy)) {
		v += conv_pixel64(conv_img + m.draw_off, m.draw_w, m.draw_h, psf, m.psf_w, m.psf_h, dx, dy);
	}
	return v;
}

__global__ void convolve64_kernel(const double *__restrict__ src, unsigned int w, unsigned int h,
                                  const double *__restrict__ krn, unsigned int kw, unsigned int kh,
                                  const uint8_t *__restrict__ mask, double *__restrict__ out)
{
	const long long n = (long long)w * h;
	for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < n; g += (long long)gridDim.x * blockDim.x) {
		if (mask && !mask[g]) {
			out[g] = 0;
			continue;
		}
		out[g] = conv_pixel64(src, w, h, krn, kw, kh, (unsigned int)(g % w), (unsigned int)(g / w));
	}
}

// fft_fine 0: every model on the direct convolution (the FFT's last pass
// writes the others); 1: the SUM-downsampled FFT models, whose fine pixels
// that pass left in conv_img at their drawing positions.
__global__ void finish64_kernel(const ModelDev *__restrict__ models, int n_models, const double *__restrict__ psf_pool,
                                const double *__restrict__ conv_img, const double *__restrict__ direct_img,
                                double *__restrict__ out, long long total_out, int fft_fine)
{
	for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < total_out;
	     g += (long long)gridDim.x * blockDim.x) {
		const int mi = find_model_out(models, n_models, g);
		const ModelDev &m = models[mi];
		const bool downsample = m.fs > 1 && !m.return_fs;
		if (fft_fine ? !(m.use_fft && downsample) : (bool)m.use_fft) continue;
		const long long local = g - m.out_off;
		const unsigned int ox = (unsigned int)(local % m.out_w), oy = (unsigned int)(local / m.out_w);
		const double *psf = m.psf_off >= 0 ? psf_pool + m.psf_off : nullptr;
		double v;
		if (downsample) {
			v = 0;
			for (unsigned int r = oy * m.fs; r < min((oy + 1) * m.fs, m.crop_h); r++) {
				for (unsigned int c = ox * m.fs; c < min((ox + 1) * m.fs, m.crop_w); c++) {
					v += fft_fine ? conv_img[m.draw_off + (size_t)(r + m.pad_y) * m.draw_w + c + m.pad_x]
					              : drawn_pixel64(m, psf, conv_img, direct_img, c + m.pad_x, r + m.pad_y);
				}
			}
		}
		else {
			v = drawn_pixel64(m, psf, conv_img, direct_img, ox + m.pad_x, oy + m.pad_y);
		}
		out[g] = kept(m, (int)ox, (int)oy) ? v : 0.;  // image &= mask (src/model.cpp:313-317)
	}
}

}  // namespace

void launch_eval64(const ModelDev *models, int n_models, const ProfileDev *profs, const double *psf_pool,
                   double *conv_img, double *direct_img, long long n_tiles, unsigned int *tile_counter,
                   DebugRec dbg, const LevelPool64 &pool, int n_levels, int n_sm, cudaStream_t stream)
{
	int blocks = n_sm * 8;
	long long need = (n_tiles + kWarps64 - 1) / kWarps64;
	if (need < blocks) blocks = (int)(need > 0 ? need : 1);
	if (pool.box) {
		eval_tiles64_kernel<true><<<blocks, kWarps64 * 32, 0, stream>>>(models, n_models, profs, psf_pool, conv_img,
		                                                                direct_img, n_tiles, tile_counter, dbg, pool);
		// one launch per recursion level a tree of the batch can reach; a level
		// without boxes ends at once
		for (int level = 0; level < n_levels; level++) {
			level64_kernel<<<n_sm * 8, kWarps64 * 32, 0, stream>>>(profs, conv_img, direct_img, pool, level, dbg);
		}
	}
	else {
		eval_tiles64_kernel<false><<<blocks, kWarps64 * 32, 0, stream>>>(models, n_models, profs, psf_pool, conv_img,
		                                                                 direct_img, n_tiles, tile_counter, dbg, pool);
	}
}

void launch_convolve64(const double *src, unsigned int w, unsigned int h, const double *krn, unsigned int kw,
                       unsigned int kh, const uint8_t *mask, double *out, int n_sm, cudaStream_t stream)
{
	const long long n = (long long)w * h;
	long long need = (n + 255) / 256;
	int blocks = (int)(need < (long long)n_sm * 16 ? need : (long long)n_sm * 16);
	if (blocks < 1) blocks = 1;
	convolve64_kernel<<<blocks, 256, 0, stream>>>(src, w, h, krn, kw, kh, mask, out);
}

void launch_finish64(const ModelDev *models, int n_models, const double *psf_pool, const double *conv_img,
                     const double *direct_img, double *out, long long total_out, int fft_fine, int n_sm,
                     cudaStream_t stream)
{
	int threads = 256;
	long long need = (total_out + threads - 1) / threads;
	int blocks = (int)(need < (long long)n_sm * 16 ? need : (long long)n_sm * 16);
	if (blocks < 1) blocks = 1;
	finish64_kernel<<<blocks, threads, 0, stream>>>(models, n_models, psf_pool, conv_img, direct_img, out, total_out,
	                                                fft_fine);
}

}  // namespace pf
