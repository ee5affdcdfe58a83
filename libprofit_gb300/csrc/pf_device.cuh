// Device-side data layout shared by the kernels of the GB300 backend.
//
// A batch is a set of models (pf_model_desc) and their profiles
// (pf_profile_desc). For each model the device holds, back to back in HBM:
//   * its drawing area (width*fs + 2*pad_x) x (height*fs + 2*pad_y), the
//     padded canvas Model::produce_image draws into (src/model.cpp:322-360),
//     twice: "conv" (profiles with convolve = 1, the to_convolve image) and
//     "direct" (the rest, the model_image), both row-major;
//   * its output image (cropped, optionally downsampled), row-major, in the
//     caller's buffer.
// Work is dispatched in tiles of 32 consecutive drawing pixels of one row,
// a warp per tile or per row segment of tiles, tiles of all models numbered
// consecutively.
#pragma once

#include <climits>
#include <cstdint>

#include "../../include/pf_cuda.h"
#include "user_profile.cuh"

namespace pf {

constexpr int kMaxLevels = 16;   // subsample_pixel recursion levels held per warp
constexpr int kMaxRes = 16;      // largest sub-pixel resolution (res*res <= 256)
constexpr int kMaskWords = (kMaxRes * kMaxRes + 31) / 32;
constexpr int kLevelCounts = 32;       // per profile: subsample_pixel calls per level in [0, 16), then
constexpr int kCountDirectEvals = 30;  // evaluate_at calls made directly on pixel centres
constexpr int kCountSubEvals = 31;     // evaluate_at calls made inside subsample_pixel

// sersic r_factor specialisations (src/sersic.cpp:79-159)
enum RFactor : int { RF_GENERAL = 0, RF_POINTFIVE, RF_ONE, RF_TWO, RF_THREE, RF_FOUR, RF_EIGHT, RF_SIXTEEN };

enum DevError : unsigned int {
	ERR_NONE = 0,
	ERR_LEVELS = 1u << 0,    // max_recursions beyond kMaxLevels - 1
	ERR_RES = 1u << 1,       // resolution beyond kMaxRes
	ERR_NONFINITE = 1u << 2, // (informational) a non-finite constant was produced
};

struct ModelDev {
	uint32_t width, height, fs, return_fs;
	uint32_t draw_w, draw_h, pad_x, pad_y;
	uint32_t crop_w, crop_h, out_w, out_h;
	double scale_x, scale_y;   // image pixel scale (Model::scale)
	double sx, sy;             // drawing pixel scale (scale / finesampling)
	double magzero;
	int32_t first_profile, n_profiles;
	int32_t conv_required, convolver;
	int64_t psf_off;           // offset of the normalised PSF in the device PSF pool, -1 none
	uint32_t psf_w, psf_h;
	double psf_scale_x, psf_scale_y;
	int64_t draw_off;          // pixel offset of the drawing area in the conv / direct scratch
	int64_t out_off;           // pixel offset of the output image
	int64_t tile_base;         // first tile number of this model
	uint32_t tiles_per_row;
	uint32_t pad0;
	float fsx_hi, fsx_lo, fsy_hi, fsy_lo;  // drawing pixel scale as unevaluated float sums
	float fscale_x, fscale_y;              // image pixel scale (sersic central pixel test)
	// FFT convolution (fft.cu): transform sizes and complex-element offsets of
	// this model's work area (draw_h rows of fft_mx/2+1 bins) and PSF spectrum
	// (fft_my rows of fft_mx/2+1 bins)
	int32_t use_fft;
	uint32_t fft_mx, fft_my;
	int32_t pad2;
	int64_t fft_work_off, fft_spec_off;
	// calculation mask (Model::evaluate, src/model.cpp:152-317): the drawing
	// pixels the profiles and the convolution are evaluated at (null: all),
	// and the mask the output is multiplied by at the end (null: none), of
	// mask_final_w columns, output pixel (x, y) taking (x / div, y / div)
	const uint8_t *mask_eval;
	const uint8_t *mask_final;
	uint32_t mask_final_w, mask_final_div;
	// crop = false with the FFT convolver (double precision): output pixel
	// (c, r) takes the linear convolution (source * PSF) at (c + ufx0, r + ufy0)
	// and the direct image at drawing pixel (c + udx0, r + udy0), each zero
	// outside its area (Model::evaluate, src/model.cpp:288-306, on the
	// FFTConvolver's uncropped frame, src/convolve.cpp:263-312)
	int32_t uncropped;
	int32_t ufx0, ufy0, udx0, udy0;
	// some profile draws unconvolved: the direct image has content; without
	// one the single-precision evaluation leaves it unwritten and its readers
	// take zeros
	int32_t direct_required;
};

// The radial profile kinds: the six of the reference and a user-defined one
// compiled in (user_profile.cuh)
__host__ __device__ constexpr bool is_radial(int kind)
{
	return (kind >= PF_SERSIC && kind <= PF_BROKENEXP) || (kind == PF_USER && user::available);
}

// The reference's parameter validation of the radial profiles, in its order:
// RadialProfile::validate (src/radial.cpp:204-214), then each kind's own
// (src/sersic.cpp:207-218, src/coresersic.cpp:61-82, src/moffat.cpp:60-71,
// src/ferrer.cpp:62-76, src/king.cpp:61-74, src/brokenexponential.cpp:96-109).
// Returns the first rule the parameters break (param_rule_message gives the
// reference's text), 0 if none. Comparisons as the reference's: a NaN passes.
enum ParamRule : int {
	PR_OK = 0, PR_AXRAT_LE0, PR_AXRAT_GT1, PR_BOX, PR_RE, PR_NSER, PR_RB, PR_CORE_A, PR_CORE_B, PR_FWHM, PR_CON,
	PR_ROUT, PR_FERRER_A, PR_FERRER_B, PR_RC, PR_RT, PR_KING_A, PR_H1, PR_H2, PR_EXP_RB, PR_COUNT
};
// a user profile's validate() result k >= 1 is rule PR_COUNT - 1 + k (rules fit
// in 5 bits: at most 11 user messages)
static_assert(PR_COUNT + 11 <= 32, "rule numbers fit in 5 bits");

__host__ __device__ inline int param_rule(int kind, const double *v)
{
	if (is_radial(kind)) {
		if (v[PF_P_AXRAT] <= 0) return PR_AXRAT_LE0;
		if (v[PF_P_AXRAT] > 1) return PR_AXRAT_GT1;
		if (v[PF_P_BOX] <= -2) return PR_BOX;
	}
	switch (kind) {
	case PF_SERSIC:
		if (v[6] <= 0) return PR_RE;
		if (v[7] <= 0) return PR_NSER;
		break;
	case PF_CORESERSIC:
		if (v[6] <= 0) return PR_RE;
		if (v[8] <= 0) return PR_RB;
		if (v[7] <= 0) return PR_NSER;
		if (v[9] <= 0) return PR_CORE_A;
		if (v[10] > 1.999) return PR_CORE_B;
		break;
	case PF_MOFFAT:
		if (v[6] <= 0) return PR_FWHM;
		if (v[7] < 0) return PR_CON;
		break;
	case PF_FERRER:
		if (v[6] <= 0) return PR_ROUT;
		if (v[7] < 0) return PR_FERRER_A;
		if (v[8] > 2) return PR_FERRER_B;
		break;
	case PF_KING:
		if (v[6] <= 0) return PR_RC;
		if (v[7] <= 0) return PR_RT;
		if (v[8] < 0) return PR_KING_A;
		break;
	case PF_BROKENEXP:
		if (v[6] <= 0) return PR_H1;
		if (v[7] <= 0) return PR_H2;
		if (v[8] <= 0) return PR_EXP_RB;
		break;
	case PF_USER: {
		const int k = user::validate(v);
		if (k > 0 && k <= 11) return PR_COUNT - 1 + k;
		break;
	}
	default:
		break;
	}
	return PR_OK;
}

// the reference's invalid_parameter message of each rule
inline const char *param_rule_message(int rule)
{
	static const char *const msg[PR_COUNT] = {
	    "",
	    "axrat <= 0, must have axrat > 0",
	    "axrat > 1, must have axrat <= 1",
	    "box <= -2, must have box > -2",
	    "re <= 0, must have re > 0",
	    "nser <= 0, must have nser > 0",
	    "rb <= 0, must have rb > 0",
	    "a <= 0, must have a > 0",
	    "b > 1.999, must have b < 1.999",
	    "fwhm <= 0, must have fwhm > 0",
	    "con < 0, must have con >= 0",
	    "rout <= 0, must have rout >= 0",
	    "a < 0, must have a >= 0",
	    "b > 2, must have b <= 2",
	    "rc <= 0, must have rc > 0",
	    "rt <= 0, must have rt > 0",
	    "a < 0, must have a >=0",
	    "h1 <= 0, must have h1 > 0",
	    "h2 <= 0, must have h2 > 0",
	    "rb <= 0, must have rb > 0",
	};
	if (rule >= PR_COUNT && user::available) return user::message(rule - PR_COUNT);
	return rule > 0 && rule < PR_COUNT ? msg[rule] : "";
}

// whether drawing pixel (x, y) of model m is evaluated (not masked out)
__device__ __forceinline__ bool evaluated(const ModelDev &m, int x, int y)
{
	return !m.mask_eval || m.mask_eval[(size_t)y * m.draw_w + x] != 0;
}

// whether output pixel (x, y) of model m survives the final masking
__device__ __forceinline__ bool kept(const ModelDev &m, int x, int y)
{
	return !m.mask_final || m.mask_final[(size_t)(y / m.mask_final_div) * m.mask_final_w + x / m.mask_final_div] != 0;
}

struct ProfileDev {
	// from the descriptor (never modified on the device)
	int32_t kind, convolve, rough, adjust, rescale_flux;
	uint32_t resolution_in, max_recursions;
	int32_t model;
	double acc_in, rscale_switch_in, rscale_max_in;
	double par[PF_NPAR];
	// working copies after RadialProfile::initial_calculations' adjustments
	uint32_t resolution;
	int32_t pad1;
	double acc, rscale_switch, rscale_max;
	// computed by the setup kernel (RadialProfile::initial_calculations and evaluate)
	int32_t rf_boxy, rf_t;
	double rscale, ie, bn, lumtot, rescale_factor;
	double cos_ang, sin_ang, xc, yc;
	double flux_scale;
	double bg;                 // sky: bg / fs^2
	double psf_mag_scale;      // psf: 10^(-0.4 (mag - magzero))
	int32_t bbx0, bbx1, bby0, bby1;   // drawing pixels outside are exactly zero
	int32_t sbx0, sbx1, sby0, sby1;   // drawing pixels outside are never subsampled (empty: x1 < x0)
	int64_t depth_off;         // offset of this profile's depth map (debug recording)
	// single-precision copies for the FP32 path (setup kernel); 16-byte
	// aligned and contiguous up to fpar[11], read as float4 vectors
	alignas(16) float fxc_hi;
	float fxc_lo, fyc_hi, fyc_lo;          // centre as an unevaluated float sum
	float fcos, fsin, finv_axrat, finv_rscale;
	float fswitch, frmax, facc, fflux_scale;
	float fbg;
	int32_t fboxy;
	float fpar[12];            // per-kind folded constants, FP_* slots
	// adjoint: d bn / d nser and d ln(flux_scale) / d par[k] (setup kernel)
	double dbn;
	double dlnfs[PF_NPAR];
	int32_t grad_ok;           // the adjoint supports this profile
	int32_t center_boost;      // sersic, adjust and nser > 1: the central pixel uses res 8, 10 levels
	float fbn, fdbn, fnser, fre;
};

// Gradient accumulators of one profile in the adjoint: the pixel value (for
// the flux-scale derivatives) and the shape derivatives d ln f / d par.
enum GradSlot : int {
	G_V = 0, G_XCEN, G_YCEN, G_ANG, G_AXRAT, G_BOX, G_X0, G_X1, kGradSlots
};

// Slots of ProfileDev::fpar (folded by the setup kernel)
enum FParSlot : int {
	FP_B = 0, FP_INVB = 1,                         // box + 2 and its inverse
	FP_S_INV_RE2 = 2, FP_S_HALF_INV_N = 3, FP_S_INV_RE = 4, FP_S_INV_NB = 5, FP_S_K = 6,
	FP_C_A = 2, FP_C_B_OVER_A = 3, FP_C_INV_RB = 4, FP_C_RB_A = 5, FP_C_INV_RE_A = 6, FP_C_K = 7, FP_C_INV_NA = 8,
	FP_M_INV_RS2 = 2, FP_M_INV_RS = 3, FP_M_CON = 4,
	FP_F_INV_ROUT = 2, FP_F_A = 3, FP_F_2MB = 4,
	FP_K_RT = 2, FP_K_INV_RC = 3, FP_K_A = 4, FP_K_INV_A = 5, FP_K_TEMP = 6,
	FP_E_RB = 2, FP_E_A = 3, FP_E_INV_A = 4, FP_E_INV_H1 = 5, FP_E_EXPO = 6,
};

// Sub-pixel boxes split off the subsampling trees (FP32 path). A subsampled
// pixel whose level-0 box (subsample_pixel's first call, src/radial.cpp:55-135)
// fails the accuracy test at some sub-points does not walk their subtrees in
// the warp that meets it: it exports them as level-1 boxes, which a later
// kernel takes one per warp. The pixel's value is then formed as the
// depth-first walk forms it -- the level-0 box's accepted points, then each
// failing sub-point's subtree in ascending order -- by whichever warp
// finishes the pixel's last box, and the pixel's canvas value (the tile's sum
// of its other profiles, then the split profiles in profile order) by the
// warp that finishes its last split profile. Counters, never waits.
struct SplitBox {
	float xhi, xlo, yhi, ylo;  // corner relative to the profile centre (unevaluated sums)
	float bx, by;              // size
	int32_t root;              // the SplitRoot it belongs to
	uint32_t meta;             // res | level << 8 | max_rec << 16
};

struct SplitRoot {
	float accepted;            // the level-0 box's accepted sub-points (warp sum)
	uint32_t first_box, n_boxes;
	uint32_t pending;          // boxes not finished
	int32_t profile;
	int32_t pixel;             // the SplitPixel of its drawing pixel
	int32_t next;              // the pixel's next split profile (profile order), -1 none
	int32_t depth;             // deepest level + 1 (depth map)
	uint32_t res;
	float fflux;               // the profile's flux scale
	int32_t convolve;
	float value;               // fflux x the pixel value, once complete
	int64_t depth_idx;         // index into the depth maps, -1 when not recording
};

struct SplitPixel {
	int64_t idx;               // canvas index (the model's draw_off + row x draw_w + column)
	float s_conv, s_direct;    // the tile's sums of the profiles not split
	int32_t first_root;        // split profiles, in profile order
	uint32_t pending;          // split profiles not complete
	int32_t conv_required;
	int32_t direct_required;
};

// The device pool (sized at batch creation; box == nullptr: no splitting).
// cnt: [0] boxes, [1] roots, [2] pixels allocated, [3] the box kernel's work
// counter, [4] splits refused for lack of room (the tree then walked in place);
// reset by the setup kernel.
struct SplitPool {
	SplitBox *box;
	float *box_val;
	SplitRoot *root;
	SplitPixel *pix;
	unsigned int *cnt;
	unsigned int cap_box, cap_root, cap_pix;
	unsigned int min_fail;     // failing level-0 sub-points for a split
};
// The FP64 path's subsampling trees, one recursion level at a time
// (eval_f64.cu). A subsampled drawing pixel of a profile becomes a level-0
// box (subsample_pixel's first call, src/radial.cpp:55-135); the level-L
// kernel evaluates every level-L box's res x res sub-points, 16 per warp, and
// the warp that evaluates a box's last sub-points sums its accepted values in
// index order and allocates its failing sub-points' boxes at level L + 1 in
// ascending order. A box whose children are all complete forms its value as
// the depth-first walk does (the accepted sum, then the children's values in
// ascending order, over res^2) in the warp that completed its last child, up
// to the pixel. Counters, never waits.
struct LevelBox64 {
	double x0, x1, y0, y1;     // subsample_pixel's box
	double accepted;           // the accepted sub-points' values, summed in index order
	double value;              // (accepted + the children's values) / res^2, once complete
	int32_t profile;
	int32_t parent;            // -1: a drawing pixel's level-0 box
	uint32_t rank;             // the parent's failing sub-point it refines (in ascending order)
	uint32_t meta;             // res | level << 8 | max_rec << 16; kDeadBox: allocated without room
	uint32_t pending;          // chunks not evaluated, then children not complete
	uint32_t first_child, n_children;
	int32_t root;              // its LevelRoot64
	unsigned long long val_off;  // its res^2 sub-point values in LevelPool64::val
	uint32_t mask[kMaskWords]; // the failing sub-points
};
constexpr uint32_t kDeadBox = 0xffffffffu;
constexpr int kChunk64 = 16;  // sub-points per warp (a lane pair each: value, test)

struct LevelRoot64 {
	double flux_scale;
	double value;              // flux_scale x the pixel value, once complete
	int32_t pixel;             // its LevelPixel64
	int32_t next;              // the pixel's next subsampled profile (profile order), -1 none
	int32_t convolve;
	int32_t deepest;           // deepest level + 1 (depth map)
	int64_t depth_idx;         // index into the depth maps, -1 when not recording
};

struct LevelPixel64 {
	int64_t idx;               // canvas index
	double s_conv, s_direct;   // the tile's sums of the profiles not subsampled
	int32_t first_root;
	uint32_t pending;          // subsampled profiles not complete
	int32_t conv_required;
	int32_t pad;
};

// cnt: the LevelCnt words, reset by the setup kernel. bound[L] .. bound[L+1]
// are the level-L boxes (bound[L+1] written by the last block of the kernel
// that allocated them); done[k] counts the finished blocks of the tile kernel
// (k = 0) and of the level-(k-1) kernel.
enum LevelCnt : int {
	LC_BOX = 0, LC_ROOT = 1, LC_VAL = 2 /* and 3: 64 bits */, LC_PIX = 4, LC_REFUSED = 5,
	LC_BOUND = 8, LC_DONE = LC_BOUND + kMaxLevels + 2, LC_END = LC_DONE + kMaxLevels + 1,
};

struct LevelPool64 {
	LevelBox64 *box;           // nullptr: no level pool (the tile warps walk the trees)
	double *val;
	LevelRoot64 *root;
	LevelPixel64 *pix;
	unsigned int *cnt;
	unsigned int cap_box, cap_root, cap_pix;
	unsigned long long cap_val;
};

constexpr int kSplitCounters = LC_END;  // the FP32 pool's 5 counters or the FP64 pool's LevelCnt words

struct DebugRec {
	int8_t *depth;             // per profile drawing-area depth maps, or nullptr
	unsigned long long *counts;// n_profiles * kLevelCounts, or nullptr
};

// floor(idx / res) for idx < 256, res <= 16, by a 16-bit fixed-point
// reciprocal (error < 256 / 65536 < 1 / res): no integer division
__device__ __forceinline__ unsigned int div_res(unsigned int idx, unsigned int magic) { return (idx * magic) >> 16; }
__host__ __device__ __forceinline__ unsigned int res_magic(unsigned int res) { return (65536u + res - 1) / res; }

// (float)i for 0 <= i < 2^23 without a conversion instruction
__device__ __forceinline__ float small_int_to_float(unsigned int i)
{
	return __int_as_float(0x4B000000 | (int)i) - 8388608.f;
}

// Whether profile q of model m contributes to the 32-pixel row tile
// [col0, col1] of drawing row `row`: a radial profile only within its culling
// box, the sky and psf profiles everywhere, null profiles nowhere. The eval
// kernels test 32 profiles at once, one per lane, and draw the ones that
// reach the tile in profile order.
__device__ __forceinline__ bool profile_reaches(const ProfileDev *__restrict__ profs, const ModelDev &m, int q,
                                                int row, int col0, int col1)
{
	if (q >= m.n_profiles) return false;
	const ProfileDev &P = profs[m.first_profile + q];
	if (!is_radial(P.kind)) return P.kind == PF_SKY || P.kind == PF_PSF;
	return !(row < P.bby0 || row > P.bby1 || col1 < P.bbx0 || col0 > P.bbx1);
}

// Costly tiles first (FP32 eval and backward). A profile's ring tiles lie in
// its subsampling box: rows by distance from the row of its centre (ring
// index l = 0: that row, 1: the row above, 2: the row below, ...; l <
// kRingRows) and a window of kRingCols tile columns around the centre.
constexpr int kRingRows = 64;
constexpr int kRingCols = 4;

__device__ __forceinline__ int ring_centre_row(const ProfileDev &P, const ModelDev &m)
{
	const int centre = (int)floorf(__fdividef(P.fyc_hi, m.fsy_hi));
	return min(max(centre, P.sby0), P.sby1);
}

__device__ __forceinline__ int ring_first_col(const ProfileDev &P, const ModelDev &m)
{
	const int ctile = (int)floorf(__fdividef(P.fxc_hi, m.fsx_hi)) / 32;
	return max(P.sbx0 / 32, ctile - (kRingCols - 1) / 2);
}

// The ring tile (l, c) of profile P: false if its box has none there.
__device__ __forceinline__ bool ring_tile_of(const ProfileDev &P, const ModelDev &m, int l, int c, int &row,
                                             int &tcol)
{
	if (P.sby1 < P.sby0 || P.sbx1 < P.sbx0) return false;
	const int centre = ring_centre_row(P, m);
	const int half = (l + 1) >> 1;
	row = (l & 1) ? centre - half : centre + half;
	if (row < P.sby0 || row > P.sby1) return false;
	tcol = ring_first_col(P, m) + c;
	return tcol <= P.sbx1 / 32;
}

// The tile columns [first, last] of drawing row `row` that are ring tiles of
// P (last < first if none).
__device__ __forceinline__ void ring_cols_of_row(const ProfileDev &P, const ModelDev &m, int row, int &first,
                                                 int &last)
{
	first = 0;
	last = -1;
	if (P.sby1 < P.sby0 || P.sbx1 < P.sbx0 || row < P.sby0 || row > P.sby1) return;
	const int centre = ring_centre_row(P, m);
	const int l = row >= centre ? 2 * (row - centre) : 2 * (centre - row) - 1;
	if (l >= kRingRows) return;
	first = ring_first_col(P, m);
	last = min(first + kRingCols - 1, P.sbx1 / 32);
}

__device__ __forceinline__ int find_model(const ModelDev *models, int n_models, long long tile)
{
	int lo = 0, hi = n_models - 1;
	while (lo < hi) {
		int mid = (lo + hi + 1) >> 1;
		if (models[mid].tile_base <= tile) lo = mid; else hi = mid - 1;
	}
	return lo;
}

// find_model, tried first at the model `hint` and the one after it
__device__ __forceinline__ int find_model_from(const ModelDev *models, int n_models, long long tile, int hint)
{
	const long long b0 = models[hint].tile_base;
	const long long b1 = hint + 1 < n_models ? models[hint + 1].tile_base : LLONG_MAX;
	const long long b2 = hint + 2 < n_models ? models[hint + 2].tile_base : LLONG_MAX;
	if (b0 <= tile && tile < b1) return hint;
	if (b1 <= tile && tile < b2) return hint + 1;
	return find_model(models, n_models, tile);
}

}  // namespace pf
