// Host side of the C ABI declared in include/pf_cuda.h.
//
// Validation follows Model::analyze_inputs (src/model.cpp:186-219) and the
// profiles' validate() methods with the reference's messages; the drawing
// geometry follows Model::analyze_expansion_requirements
// (src/model.cpp:152-184) for models without a calculation mask. Every
// device buffer of a batch is sized once, at pf_batch_create; pf_forward only
// enqueues kernels.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <new>
#include <string>
#include <vector>

#include "../../include/pf_cuda.h"
#include "pf_device.cuh"

namespace pf {
void launch_setup(const ModelDev *models, ProfileDev *profs, int n_profiles, int n_models,
                  unsigned int *tile_counter, unsigned int *err, const double *psf_raw, double *psf_norm,
                  bool have_psf, double *solves, int want_grad, cudaStream_t stream);
void launch_eval64(const ModelDev *models, int n_models, const ProfileDev *profs, const double *psf_pool,
                   double *conv_img, double *direct_img, long long n_tiles, unsigned int *tile_counter,
                   DebugRec dbg, const LevelPool64 &pool, int n_levels, int n_sm, cudaStream_t stream);
void launch_finish64(const ModelDev *models, int n_models, const double *psf_pool, const double *conv_img,
                     const double *direct_img, double *out, long long total_out, int fft_fine, int n_sm,
                     cudaStream_t stream);
void launch_convolve64(const double *src, unsigned int w, unsigned int h, const double *krn, unsigned int kw,
                       unsigned int kh, const uint8_t *mask, double *out, int n_sm, cudaStream_t stream);
void launch_flux_sum(const ModelDev *models, int n_models, const void *images, int is_double, double *flux,
                     cudaStream_t stream);
void launch_set_params(ProfileDev *profs, int n_profiles, const double *params, cudaStream_t stream);
void launch_eval32(const ModelDev *models, int n_models, const ProfileDev *profs, int n_profiles,
                   const double *psf_pool, float *conv_img, float *direct_img, long long n_tiles,
                   unsigned int *counter, unsigned int *claims, DebugRec dbg, const SplitPool &pool, bool sersic_only, int n_sm,
                   cudaStream_t stream);
long long eval32_items(long long n_profiles, long long n_tiles);
int fft32_rows_per_job(int n);
int fft32_cols_per_job(int n);
int fft32_size_at_least(int n);
int fft32_twiddle_len();
cudaError_t fft32_configure();
void launch_fft32_twiddles(void *tw, cudaStream_t stream);
void launch_fft32(int pass, int mode, int n, const void *jobs, int n_jobs, const ModelDev *models, const float *src,
                  const float *psf, void *work, void *spec, const float *direct, float *out, const void *tw,
                  cudaStream_t stream);
template <typename T>
int conv_num_shapes();
template <typename T>
void conv_tile_dims(int shape, int *bw, int *bh);
template <typename T>
long long conv_tiles(unsigned int w, unsigned int h, int shape);
template <typename T>
size_t conv_smem(unsigned int kw, unsigned int kh, int shape);
template <typename T>
cudaError_t conv_configure(size_t smem, int shape, int kwp);
template <typename T>
void launch_conv(int mode, int shape, int kwp, const ModelDev *models, int n_models, const T *psf, const T *in,
                 const T *direct, T *out, const long long *tile_base, long long n_tiles, size_t smem, int n_sm,
                 cudaStream_t stream);
bool conv_stride_fixed(int kwp);
void launch_psf_to_float(const double *in, float *out, long long n, cudaStream_t stream);
int fft_job_size();
template <typename T>
size_t fft_smem(int n, int count);
template <typename T>
cudaError_t fft_configure(size_t smem);
template <typename T>
void launch_twiddles(void *tw, int nmax, cudaStream_t stream);
template <typename T>
void launch_fft_pass(int pass, const ModelDev *models, const void *jobs, int n_jobs, const T *src, const T *psf,
                     void *work, void *spec, const T *direct, T *out, T *fine, const void *tw, int nmax, size_t smem,
                     cudaStream_t stream);
template <typename T>
void launch_chi2(const ModelDev *models, int n_models, const void *img, const void *data, const void *sigma,
                 const void *cot, void *gout, double *chi2, int parts, double *partial, unsigned int *done,
                 cudaStream_t stream);
template <typename T>
void launch_backward(const ModelDev *models, const ProfileDev *profs, int n_profiles, const void *gout,
                     const void *gsrc, const double *psf_pool, const long long *prow_base, unsigned int n_ring,
                     unsigned int *counter, double *partial, double *ring_partial, double *grad, bool sersic_only,
                     int n_sm, cudaStream_t stream);
long long backward_items(long long n_profiles, long long n_ring);
int backward_slots(bool sersic_only);
long long backward_ring_slots(bool sersic_only);
}  // namespace pf

namespace {

thread_local std::string g_last_error;

pf_status fail(pf_status s, const std::string &msg)
{
	g_last_error = msg;
	return s;
}

}  // namespace

namespace pf {
// the calling thread's pf_last_error message, for the host-only entry points
// of other translation units (fits.cu)
void set_last_error(const std::string &msg) { g_last_error = msg; }
}  // namespace pf

namespace {

#define PF_CUDA_TRY(call)                                                                              \
	do {                                                                                               \
		cudaError_t e_ = (call);                                                                       \
		if (e_ != cudaSuccess) {                                                                       \
			return fail(e_ == cudaErrorMemoryAllocation ? PF_ERR_NO_MEMORY : PF_ERR_CUDA,              \
			            std::string(#call) + ": " + cudaGetErrorString(e_));                           \
		}                                                                                              \
	} while (0)

using pf::is_radial;

// Profile::validate of every kind, with the reference's messages.
pf_status validate_profile(const pf_profile_desc &d, bool model_has_psf)
{
	const double *v = d.par;
	if (d.kind < PF_SERSIC || d.kind > PF_USER || (d.kind == PF_USER && !pf::user::available)) {
		return fail(PF_ERR_INVALID_PARAMETER, "Unknown profile kind " + std::to_string(d.kind));
	}
	const int rule = pf::param_rule(d.kind, v);  // src/radial.cpp:204-214 and each kind's validate()
	if (rule != pf::PR_OK) return fail(PF_ERR_INVALID_PARAMETER, pf::param_rule_message(rule));
	switch (d.kind) {
	case PF_PSF:  // src/psf.cpp:39-45
		if (!model_has_psf) {
			return fail(PF_ERR_INVALID_PARAMETER, "No psf present in the model, cannot produce a psf profile");
		}
		break;
	default:
		break;
	}
	if (is_radial(d.kind) && !d.rough) {
		// the device holds at most kMaxLevels nested sub-pixel boxes per warp
		unsigned int levels = d.max_recursions;
		if (d.kind == PF_SERSIC && d.adjust) levels = std::max(levels, 10u);
		if (levels + 1 > (unsigned int)pf::kMaxLevels) {
			return fail(PF_ERR_UNSUPPORTED, "max_recursions > " + std::to_string(pf::kMaxLevels - 1) +
			                                    " is not supported by the CUDA backend");
		}
		if (!d.adjust && d.resolution > (unsigned int)pf::kMaxRes) {
			return fail(PF_ERR_UNSUPPORTED, "resolution > " + std::to_string(pf::kMaxRes) +
			                                    " is not supported by the CUDA backend");
		}
	}
	return PF_OK;
}

struct Geometry {
	uint32_t pad_x, pad_y, draw_w, draw_h, crop_w, crop_h, out_w, out_h;
	bool conv;
	bool direct = false;  // some profile draws unconvolved
	// crop = false with the FFT convolver: the output window in the FFT's
	// uncropped frame (ModelDev::ufx0..udy0) and the offset Model::evaluate
	// reports (offset_out); 0 otherwise
	bool uncropped = false;
	int32_t ufx0 = 0, ufy0 = 0, udx0 = 0, udy0 = 0;
	uint32_t off_x = 0, off_y = 0;
	// calculation mask (adjustable): what Model::evaluate does with it
	bool mask_needs_convolution = false, mask_needs_psf_padding = false, mask_needs_adjustment = false;
};

// crop = false with the FFT convolver (Model::evaluate, src/model.cpp:288-317):
// the convolution returns its uncropped frame E = 2 max(D, K) (D the drawing
// dimensions, K the PSF's; the x component of max() for both sides,
// include/profit/image.h:204-207), the source at offset_after_convolution(D, K)
// in it (src/convolve.cpp:270-281), the linear convolution shifted by the
// kernel's start (D - K) / 2; the direct image is extended to E at that
// offset and added; then only the PSF padding is removed, by the difference
// between FFTConvolver::padding of D and of D - 2 x padding
// (src/convolve.cpp:263-268). Unsigned arithmetic as the reference's: the
// per-axis sum offset_diff + dim_diff is max(D, K).x - max(D - 2p, K).x.
pf_status uncropped_fft_geometry(const pf_model_desc &m, Geometry &g)
{
	if (m.finesampling > 1 && !m.return_finesampled) {
		return fail(PF_ERR_UNSUPPORTED, "crop = false with the FFT convolver and a SUM-downsampled image is not "
		                                "supported by the CUDA backend");
	}
	if (g.mask_needs_adjustment) {
		// the reference masks the larger uncropped image with the model's own
		// mask (src/model.cpp:312-314) and reads past the mask's end
		return fail(PF_ERR_UNSUPPORTED, "crop = false with the FFT convolver and an adjustable calculation mask "
		                                "is not supported by the CUDA backend (the reference's result is undefined)");
	}
	const int64_t dx = g.draw_w, dy = g.draw_h, kx = m.psf_w, ky = m.psf_h;
	if (dx < kx || dy < ky) {
		return fail(PF_ERR_UNSUPPORTED, "crop = false with the FFT convolver and a PSF larger than the drawing area "
		                                "is not supported by the CUDA backend");
	}
	auto off = [&](int64_t a, int64_t k) { return a / 2 - ((a % 2 == 0 || k % 2 == 0) ? 1 : 0); };
	const int64_t px = g.pad_x, py = g.pad_y;
	const int64_t mx = std::max(dx, kx), e = 2 * mx;
	// the reference transforms the flattened frame as one sequence: when the
	// linear convolution's rows (the kernel starting (dy - ky) / 2 down) pass
	// the frame's e rows, they wrap into its first rows
	if (dy + (dy - ky) / 2 + ky - 1 > e) {
		return fail(PF_ERR_UNSUPPORTED, "crop = false with the FFT convolver: the reference's frame wraps around "
		                                "for an image this much taller than wide");
	}
	const int64_t odx = off(dx, kx), ody = off(dy, ky);
	int64_t cox = 0, coy = 0, cw = e, ch = e, rx = odx, ry = ody;
	if (px > 0 && py > 0) {  // Dimensions' bool: both components (include/profit/image.h:92-94)
		const int64_t d2x = dx - 2 * px, d2y = dy - 2 * py;
		const int64_t o2x = off(d2x, kx), o2y = off(d2y, ky);
		const int64_t shrink = mx - std::max(d2x, kx);
		cw = e - 2 * px - shrink;
		ch = e - 2 * py - shrink;
		cox = px + (odx - o2x);
		coy = py + (ody - o2y);
		rx = o2x;
		ry = o2y;
	}
	if (odx < 0 || ody < 0 || rx < 0 || ry < 0 || cw <= 0 || ch <= 0) {
		return fail(PF_ERR_UNSUPPORTED, "crop = false with the FFT convolver: an image too small for its PSF");
	}
	g.uncropped = true;
	g.out_w = (uint32_t)cw;
	g.out_h = (uint32_t)ch;
	g.ufx0 = (int32_t)(cox - (dx - kx) / 2);
	g.ufy0 = (int32_t)(coy - (dy - ky) / 2);
	g.udx0 = (int32_t)(cox - odx);
	g.udy0 = (int32_t)(coy - ody);
	g.off_x = (uint32_t)rx;
	g.off_y = (uint32_t)ry;
	return PF_OK;
}

// Model::analyze_inputs + analyze_expansion_requirements (src/model.cpp:152-219);
// `mask` the model's calculation mask or null; `mask_declared`: a mask of the
// descriptor's mask_w x mask_h is set even if its bytes are not given (its
// dimension checks and, used as given, its padding rule need only those)
pf_status model_geometry(const pf_model_desc &m, const pf_profile_desc *profiles, Geometry &g,
                         const uint8_t *mask = nullptr, bool mask_declared = false)
{
	const bool has_mask = mask != nullptr || mask_declared;
	if (m.width == 0 || m.height == 0) return fail(PF_ERR_INVALID_PARAMETER, "Model's requested dimensions are 0");
	if (m.scale_x <= 0) return fail(PF_ERR_INVALID_PARAMETER, "Model's scale_x cannot be negative or zero");
	if (m.scale_y <= 0) return fail(PF_ERR_INVALID_PARAMETER, "Model's scale_y cannot be negative or zero");
	if (m.finesampling == 0) return fail(PF_ERR_INVALID_PARAMETER, "finesampling must be > 0");
	const bool has_psf = m.psf_offset >= 0 && m.psf_w > 0 && m.psf_h > 0;
	g.conv = false;
	g.direct = false;
	for (uint32_t i = 0; i < m.n_profiles; i++) {
		g.conv |= profiles[m.first_profile + i].convolve != 0;
		g.direct |= profiles[m.first_profile + i].convolve == 0;
	}
	if (g.conv && !has_psf) {
		return fail(PF_ERR_INVALID_PARAMETER, "No psf provided but profile(s) requested convolution");
	}
	for (uint32_t i = 0; i < m.n_profiles; i++) {
		pf_status s = validate_profile(profiles[m.first_profile + i], has_psf);
		if (s != PF_OK) return s;
	}
	// src/model.cpp:198-201
	if (has_mask && m.adjust_mask && (m.mask_w != m.width || m.mask_h != m.height)) {
		return fail(PF_ERR_INVALID_PARAMETER, "Mask dimensions != model dimensions");
	}
	// the PSF padding: with a mask used as given, when the mask is larger than
	// the model (times the finesampling) in both directions; with an
	// adjustable one, only when its bounding box (times the finesampling)
	// comes closer than half the PSF to an edge (src/model.cpp:152-184)
	bool padding = g.conv;
	if (has_mask && !m.adjust_mask) {
		padding = m.mask_w > m.width * m.finesampling && m.mask_h > m.height * m.finesampling;
	}
	else if (mask && g.conv) {
		uint32_t lbx = m.width, lby = m.height, ubx = 0, uby = 0;
		bool any = false;
		for (uint32_t j = 0; j < m.height; j++) {
			for (uint32_t i = 0; i < m.width; i++) {
				if (!mask[i + (size_t)j * m.width]) continue;
				lbx = std::min(lbx, i);
				lby = std::min(lby, j);
				ubx = std::max(ubx, i + 1);
				uby = std::max(uby, j + 1);
				any = true;
			}
		}
		if (!any) lbx = lby = ubx = uby = 0;
		const uint32_t fs = m.finesampling, nx = m.psf_w / 2, ny = m.psf_h / 2;
		const uint32_t lowx = lbx * fs, lowy = lby * fs, upx = (m.width - ubx) * fs, upy = (m.height - uby) * fs;
		padding = !(lowx >= nx && lowy >= ny) || !(upx >= nx && upy >= ny);
		g.mask_needs_convolution = true;
		g.mask_needs_psf_padding = padding;
	}
	g.mask_needs_adjustment = mask && m.adjust_mask &&
	                          (g.mask_needs_convolution || g.mask_needs_psf_padding || m.finesampling > 1);
	g.pad_x = padding && has_psf ? m.psf_w / 2 : 0;
	g.pad_y = padding && has_psf ? m.psf_h / 2 : 0;
	g.crop_w = m.width * m.finesampling;
	g.crop_h = m.height * m.finesampling;
	g.draw_w = g.crop_w + 2 * g.pad_x;
	g.draw_h = g.crop_h + 2 * g.pad_y;
	g.out_w = g.crop_w;
	g.out_h = g.crop_h;
	if (m.finesampling > 1 && !m.return_finesampled) {
		g.out_w = (g.crop_w + m.finesampling - 1) / m.finesampling;
		g.out_h = (g.crop_h + m.finesampling - 1) / m.finesampling;
	}
	// src/model.cpp:277-283
	if (has_mask && !m.adjust_mask && (m.mask_w != g.draw_w || m.mask_h != g.draw_h)) {
		return fail(PF_ERR_INVALID_PARAMETER, "Mask dimensions != drawing dimensions: [" + std::to_string(m.mask_w) +
		                                          ", " + std::to_string(m.mask_h) + "] != [" +
		                                          std::to_string(g.draw_w) + ", " + std::to_string(g.draw_h) + "]");
	}
	if (m.no_crop && g.conv && m.convolver == PF_CONV_FFT) return uncropped_fft_geometry(m, g);
	return PF_OK;
}

// The drawing-area mask the profiles and the convolution see (Model::adjust,
// src/model.cpp:230-246): the model's mask upsampled by the finesampling
// (Mask::upsample), extended by the PSF padding (Surface::extend) and, with
// convolution, expanded by half the PSF (Mask::expand_by, src/image.cpp:
// 112-160: a pixel is set if any mask pixel within half the PSF is; done here
// as a separable box dilation, rows then columns, with running counts).
void adjusted_mask(const pf_model_desc &m, const Geometry &g, const uint8_t *mask, std::vector<uint8_t> &out)
{
	const uint32_t fs = m.finesampling, dw = g.draw_w, dh = g.draw_h;
	out.assign((size_t)dw * dh, 0);
	for (uint32_t j = 0; j < g.crop_h; j++) {
		for (uint32_t i = 0; i < g.crop_w; i++) {
			out[(i + g.pad_x) + (size_t)(j + g.pad_y) * dw] = mask[i / fs + (size_t)(j / fs) * m.width] != 0;
		}
	}
	if (!g.mask_needs_convolution) return;
	const int px = (int)(m.psf_w / 2), py = (int)(m.psf_h / 2);
	std::vector<uint8_t> rows(out.size(), 0);
	std::vector<uint32_t> run(std::max(dw, dh) + 1);
	for (uint32_t j = 0; j < dh; j++) {
		run[0] = 0;
		for (uint32_t i = 0; i < dw; i++) run[i + 1] = run[i] + out[i + (size_t)j * dw];
		for (int i = 0; i < (int)dw; i++) {
			const int a = std::max(0, i - px), z = std::min((int)dw - 1, i + px);
			rows[i + (size_t)j * dw] = run[z + 1] - run[a] > 0;
		}
	}
	for (uint32_t i = 0; i < dw; i++) {
		run[0] = 0;
		for (uint32_t j = 0; j < dh; j++) run[j + 1] = run[j] + rows[i + (size_t)j * dw];
		for (int j = 0; j < (int)dh; j++) {
			const int a = std::max(0, j - py), z = std::min((int)dh - 1, j + py);
			out[i + (size_t)j * dw] = run[z + 1] - run[a] > 0;
		}
	}
}

}  // namespace

// One batch layout's autotuned decisions (-1 / empty: not decided yet).
struct TuneEntry {
	int fwd_shape = -1;         // forward direct-convolution block shape
	int split = -1;             // subsampling trees split off to other warps
	int adj_shape = -1;         // adjoint direct-convolution block shape
	std::vector<int8_t> fft;    // per model: the FFT (PF_CONV_AUTO models)
};

struct pf_env {
	int device = 0;
	uint32_t flags = 0;
	int n_sm = 1;
	cudaStream_t stream = nullptr;
	// the caller's handle plus one per live batch: the environment (its stream)
	// is released with the last of them, whatever order they are destroyed in
	std::atomic<int> refs{1};
	// Model::evaluate's state across calls (pf_model_evaluate*, pf_convolve):
	// the last model's batch, reused while only parameter values change, and
	// device buffers that only grow
	struct Cache {
		std::mutex mu;
		pf_batch *batch = nullptr;
		pf_model_desc model{};
		std::vector<pf_profile_desc> profiles;  // parameter values not part of the key
		std::vector<double> psf;
		std::vector<uint8_t> mask;
		bool has_mask = false;
		void *d_out = nullptr;
		size_t out_bytes = 0;
		std::vector<double> params;
		std::vector<float> host32;
		void *d_conv = nullptr;                 // pf_convolve: source, output, kernel, mask
		size_t conv_bytes = 0;
		// the last model's statistics (PF_ENV_PROFILE): stage times, per-level counts
		pf_stage_times last_times{};
		std::vector<unsigned long long> last_counts;
	} cache;
	// The autotuner's decisions (the analogue of FFTW's plans and wisdom), by
	// batch layout: kept for the environment's life and, with PF_AUTOTUNE_CACHE
	// naming a file at its creation, read from and appended to that file.
	struct Tune {
		std::mutex mu;
		std::map<uint64_t, TuneEntry> entries;
		std::string file;
		std::string gpu;                   // device name and SM count: part of every key
		uint64_t timed = 0, reused = 0;    // decisions timed, decisions taken from the cache
	} tune;
};

struct pf_batch {
	pf_env *env = nullptr;
	uint64_t tune_key = 0;              // its layout's key in env->tune (0: not tuned)
	bool dbl = true;
	std::vector<pf_model_desc> models;
	std::vector<pf_profile_desc> profiles;
	std::vector<pf::ModelDev> mdev;
	pf::ProfileDev *h_profiles = nullptr;   // pinned staging copy
	bool params_dirty = true;
	pf::ModelDev *d_models = nullptr;
	pf::ProfileDev *d_profiles = nullptr;
	double *d_psf_raw = nullptr;
	double *d_psf_norm = nullptr;
	uint8_t *d_mask_eval = nullptr;     // the models' drawing-area masks, back to back
	uint8_t *d_mask_final = nullptr;    // the models' own masks for the final masking
	size_t psf_len = 0;
	void *d_conv = nullptr;
	void *d_direct = nullptr;
	size_t draw_total = 0;
	unsigned int *d_counter = nullptr;
	unsigned int *d_claims = nullptr;   // FP32 eval: one bit per tile, set by the warp that evaluates it
	// FP32 eval: sub-pixel boxes split off to other warps (pf::SplitPool); no
	// pool (box == nullptr) for FP64 batches and PF_ENV_NO_SPLIT
	pf::SplitPool split{};
	// FP64 eval: the subsampling trees level by level (pf::LevelPool64), over
	// levels64 recursion levels; no pool for PF_ENV_NO_SPLIT
	pf::LevelPool64 level64{};
	int levels64 = 0;
	bool sersic_only = false;           // every radial profile is a sersic: the FP32 kernels drop the other kinds
	unsigned int *d_err = nullptr;
	double *d_solves = nullptr;  // per profile: the inverse-gamma solves of the setup
	long long n_tiles = 0;
	uint64_t total_out = 0;
	bool record = false;
	bool count_only = false;            // per-level counts recorded without the depth maps
	int8_t *d_depth = nullptr;
	size_t depth_total = 0;
	unsigned long long *d_counts = nullptr;
	// single-precision path
	float *d_psf32 = nullptr;
	long long *d_tile_base_out = nullptr;
	long long n_out_tiles = 0;
	size_t finish_smem = 0;
	int conv_kwp = 0;                   // PSF row stride compiled into the direct convolution (0: read per model)
	bool any_downsample = false;
	bool any_fft_downsample = false;    // FP64: an FFT model SUM-downsampled (one more finishing pass)
	int fwd_shape = 0, adj_shape = 0;  // convolution block shapes (conv.cu)
	// FFT convolution
	bool any_fft = false;
	int fft_nmax = 0;
	void *d_fft_work = nullptr;
	void *d_fft_spec = nullptr;
	void *d_fft_tw = nullptr;
	void *d_fft_jobs[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
	int fft_njobs[5] = {0, 0, 0, 0, 0};
	size_t fft_smem_bytes = 0;
	int64_t fft_work_elems = 0, fft_spec_elems = 0;
	// single precision (fft32.cu): job lists per [mode: forward, adjoint,
	// spectrum][pass: rows, columns, inverse rows], one per transform length
	struct Fft32Jobs {
		int n = 0, n_jobs = 0;
		void *d_jobs = nullptr;
	};
	std::vector<Fft32Jobs> f32_jobs[3][3];
	// adjoint
	bool adjoint = false;
	void *d_gout = nullptr;
	void *d_gsrc = nullptr;
	int chi2_parts = 1;                 // chi^2 blocks per model (large models split, ~64 k pixels each)
	double *d_chi2_partial = nullptr;   // chi2_parts FP64 per model
	unsigned int *d_chi2_done = nullptr;// per model: chi^2 blocks finished (the last one sums, resets)
	double *d_partial = nullptr;        // backward_slots() FP64 per (profile, drawing row)
	double *d_ring_partial = nullptr;   // backward_slots() FP64 per (profile, ring tile)
	long long *d_prow_base = nullptr;   // first partial row of each profile
	unsigned int *d_bwd_counter = nullptr;
	unsigned int n_ring = 0;            // row items per profile: twice the tallest drawing area
	long long *d_adj_tile_base = nullptr;
	long long n_adj_tiles = 0;
	size_t adj_smem = 0;
	// pf_step_graph: the captured step and the buffers, stream and recording
	// state it was captured with
	cudaGraphExec_t graph = nullptr;
	struct GraphKey {
		const void *params = nullptr, *images = nullptr, *data = nullptr, *sigma = nullptr;
		const void *chi2 = nullptr, *grad = nullptr;
		cudaStream_t stream = nullptr;
		bool record = false;
		bool operator==(const GraphKey &o) const
		{
			return params == o.params && images == o.images && data == o.data && sigma == o.sigma &&
			       chi2 == o.chi2 && grad == o.grad && stream == o.stream && record == o.record;
		}
	} graph_key;
	bool capturing = false;             // stage timing is off while a step is captured
	// stage timing (PF_ENV_PROFILE)
	struct EventPair {
		cudaEvent_t a, b;
		int stage;
	};
	std::vector<EventPair> ev_pool;
	size_t ev_used = 0;
	double stage_ms[6] = {0, 0, 0, 0, 0, 0};
	uint64_t forward_calls = 0, backward_calls = 0;
	uint64_t kernel_launches = 0, graph_kernels = 0;
};

namespace {

// Failing level-0 sub-points from which a subsampled pixel's subtrees are split
// off to other warps (FP32 evaluation)
#ifndef PF_SPLIT_MIN_FAIL
#define PF_SPLIT_MIN_FAIL 1
#endif
constexpr unsigned int kSplitMinFail = PF_SPLIT_MIN_FAIL;

enum Stage { ST_SETUP = 0, ST_EVAL, ST_FINISH, ST_CHI2, ST_ADJCONV, ST_BACKWARD };

// Drops one reference to an environment; the last frees it.
void env_release(pf_env *env)
{
	if (env->refs.fetch_sub(1) != 1) return;
	cudaSetDevice(env->device);
	if (env->stream) cudaStreamDestroy(env->stream);
	delete env;
}

// Entry points that check cudaGetLastError() after their launches first clear
// an error an earlier, unrelated runtime call of the process left there (a
// failed cudaMalloc, say), so that the check reports their own launches only.
// Sticky errors (a faulted context) are not cleared by this and still show.
void clear_stale_error() { (void)cudaGetLastError(); }

void fold_stage_times(pf_batch *b)
{
	for (size_t i = 0; i < b->ev_used; i++) {
		float ms = 0.f;
		if (cudaEventSynchronize(b->ev_pool[i].b) == cudaSuccess &&
		    cudaEventElapsedTime(&ms, b->ev_pool[i].a, b->ev_pool[i].b) == cudaSuccess) {
			b->stage_ms[b->ev_pool[i].stage] += ms;
		}
	}
	b->ev_used = 0;
}

// Records the start of a stage on `s`; returns the slot to close, or -1.
long stage_begin(pf_batch *b, int stage, cudaStream_t s)
{
	if (!(b->env->flags & PF_ENV_PROFILE) || b->capturing) return -1;
	if (b->ev_used >= 4096) fold_stage_times(b);
	if (b->ev_used == b->ev_pool.size()) {
		pf_batch::EventPair p{};
		if (cudaEventCreate(&p.a) != cudaSuccess || cudaEventCreate(&p.b) != cudaSuccess) return -1;
		b->ev_pool.push_back(p);
	}
	const size_t slot = b->ev_used++;
	b->ev_pool[slot].stage = stage;
	cudaEventRecord(b->ev_pool[slot].a, s);
	return (long)slot;
}

void stage_end(pf_batch *b, long slot, cudaStream_t s)
{
	if (slot >= 0) cudaEventRecord(b->ev_pool[(size_t)slot].b, s);
}

}  // namespace

namespace {

// Whether two model descriptions give the same batch layout (every field).
bool same_model(const pf_model_desc &a, const pf_model_desc &b)
{
	return a.width == b.width && a.height == b.height && a.scale_x == b.scale_x && a.scale_y == b.scale_y &&
	       a.magzero == b.magzero && a.finesampling == b.finesampling && a.return_finesampled == b.return_finesampled &&
	       a.first_profile == b.first_profile && a.n_profiles == b.n_profiles && a.psf_offset == b.psf_offset &&
	       a.psf_w == b.psf_w && a.psf_h == b.psf_h && a.psf_scale_x == b.psf_scale_x &&
	       a.psf_scale_y == b.psf_scale_y && a.convolver == b.convolver && a.mask_offset == b.mask_offset &&
	       a.adjust_mask == b.adjust_mask && a.no_crop == b.no_crop && a.mask_w == b.mask_w && a.mask_h == b.mask_h;
}

// Whether two profiles differ at most in their parameter values.
bool same_profile_layout(const pf_profile_desc &a, const pf_profile_desc &b)
{
	return a.kind == b.kind && a.convolve == b.convolve && a.rough == b.rough && a.adjust == b.adjust &&
	       a.rescale_flux == b.rescale_flux && a.resolution == b.resolution && a.max_recursions == b.max_recursions &&
	       a.acc == b.acc && a.rscale_switch == b.rscale_switch && a.rscale_max == b.rscale_max;
}

}  // namespace

// ---- the autotuner's decision cache

static uint64_t fnv1a(uint64_t h, const void *data, size_t n)
{
	const unsigned char *p = static_cast<const unsigned char *>(data);
	for (size_t i = 0; i < n; i++) {
		h ^= p[i];
		h *= 1099511628211ull;
	}
	return h;
}

// The key of a batch layout: the GPU, every model's geometry, PSF size,
// convolver, mask and crop settings, and every profile's kind and subsampling
// controls; not the parameter values. Never 0.
static uint64_t tune_key(const pf_env *env, const pf_model_desc *models, size_t n_models,
                         const pf_profile_desc *profiles, size_t n_profiles)
{
	uint64_t h = fnv1a(1469598103934665603ull, env->tune.gpu.data(), env->tune.gpu.size());
	h = fnv1a(h, &n_models, sizeof(n_models));
	for (size_t i = 0; i < n_models; i++) {
		const pf_model_desc &m = models[i];
		const uint32_t f[] = {m.width, m.height, m.finesampling, (uint32_t)m.return_finesampled, m.first_profile,
		                      m.n_profiles, (uint32_t)(m.psf_offset >= 0), m.psf_w, m.psf_h, (uint32_t)m.convolver,
		                      (uint32_t)(m.mask_offset >= 0), (uint32_t)m.adjust_mask, (uint32_t)m.no_crop,
		                      m.mask_w, m.mask_h};
		h = fnv1a(h, f, sizeof(f));
	}
	h = fnv1a(h, &n_profiles, sizeof(n_profiles));
	for (size_t i = 0; i < n_profiles; i++) {
		const pf_profile_desc &d = profiles[i];
		const int32_t f[] = {d.kind, d.convolve, d.rough, d.adjust, (int32_t)d.resolution, (int32_t)d.max_recursions};
		h = fnv1a(h, f, sizeof(f));
	}
	return h ? h : 1;
}

// One line per entry: "pfcuda-tune 1 <key> <fwd> <split> <adj> <fft: one digit per model, or ->";
// a later line for a key replaces an earlier one. Lines that do not parse are skipped.
static void tune_load(pf_env *e)
{
	std::FILE *f = std::fopen(e->tune.file.c_str(), "r");
	if (!f) return;
	std::string line;
	char buf[4096];
	while (std::fgets(buf, sizeof(buf), f)) {
		line += buf;
		if (line.empty() || line.back() != '\n') {
			if (!std::feof(f)) continue;
		}
		unsigned long long key = 0;
		int fwd = -1, split = -1, adj = -1, used = 0;
		if (std::sscanf(line.c_str(), "pfcuda-tune 1 %llx %d %d %d %n", &key, &fwd, &split, &adj, &used) == 4 &&
		    used > 0) {
			TuneEntry t;
			t.fwd_shape = fwd;
			t.split = split;
			t.adj_shape = adj;
			for (size_t i = (size_t)used; i < line.size() && (line[i] == '0' || line[i] == '1'); i++)
				t.fft.push_back((int8_t)(line[i] - '0'));
			e->tune.entries[key] = t;
		}
		line.clear();
	}
	std::fclose(f);
}

// the entry of `key` (a copy); false if none
static bool tune_lookup(pf_env *e, uint64_t key, TuneEntry *out)
{
	std::lock_guard<std::mutex> lock(e->tune.mu);
	auto it = e->tune.entries.find(key);
	if (it == e->tune.entries.end()) return false;
	*out = it->second;
	return true;
}

// entry `key` updated by `update` and, with a cache file, appended to it
template <typename F>
static void tune_store(pf_env *e, uint64_t key, F update)
{
	std::lock_guard<std::mutex> lock(e->tune.mu);
	TuneEntry &t = e->tune.entries[key];
	update(t);
	e->tune.timed++;
	if (e->tune.file.empty()) return;
	std::string line = "pfcuda-tune 1 ";
	char head[96];
	std::snprintf(head, sizeof(head), "%llx %d %d %d ", (unsigned long long)key, t.fwd_shape, t.split, t.adj_shape);
	line += head;
	if (t.fft.empty()) line += "-";
	for (int8_t v : t.fft) line += v ? '1' : '0';
	line += "\n";
	if (std::FILE *f = std::fopen(e->tune.file.c_str(), "a")) {
		std::fputs(line.c_str(), f);
		std::fclose(f);
	}
}

extern "C" {

const char *pf_last_error(void) { return g_last_error.c_str(); }

pf_status pf_user_profile_info(const char **name, const char *const **param_names, const double **param_defaults,
                               uint32_t *n_params)
{
	if (!pf::user::available) {
		return fail(PF_ERR_UNSUPPORTED, "this library was built without a user-defined profile");
	}
	if (name) *name = pf::user::name();
	if (param_names) *param_names = pf::user::param_names();
	if (param_defaults) *param_defaults = pf::user::param_defaults();
	if (n_params) *n_params = (uint32_t)pf::user::n_params;
	return PF_OK;
}

const char *pf_version(void) { return "0.1.0 (libprofit 1.9.3 image path, sm_103a)"; }

pf_status pf_env_autotune_counts(pf_env *env, uint64_t *timed, uint64_t *reused)
{
	if (!env) return fail(PF_ERR_INVALID_PARAMETER, "env is NULL");
	std::lock_guard<std::mutex> lock(env->tune.mu);
	if (timed) *timed = env->tune.timed;
	if (reused) *reused = env->tune.reused;
	return PF_OK;
}

pf_status pf_env_create(int device, uint32_t flags, pf_env **env)
{
	if (!env) return fail(PF_ERR_INVALID_PARAMETER, "env is NULL");
	*env = nullptr;
	int count = 0;
	PF_CUDA_TRY(cudaGetDeviceCount(&count));
	if (device < 0 || device >= count) {
		return fail(PF_ERR_INVALID_PARAMETER, "no CUDA device " + std::to_string(device));
	}
	PF_CUDA_TRY(cudaSetDevice(device));
	pf_env *e = new (std::nothrow) pf_env();
	if (!e) return fail(PF_ERR_NO_MEMORY, "out of host memory");
	e->device = device;
	e->flags = flags;
	cudaError_t err = cudaDeviceGetAttribute(&e->n_sm, cudaDevAttrMultiProcessorCount, device);
	if (err == cudaSuccess) err = cudaStreamCreateWithFlags(&e->stream, cudaStreamNonBlocking);
	cudaDeviceProp prop{};
	if (err == cudaSuccess) err = cudaGetDeviceProperties(&prop, device);
	if (err != cudaSuccess) {
		delete e;
		return fail(PF_ERR_CUDA, std::string("pf_env_create: ") + cudaGetErrorString(err));
	}
	e->tune.gpu = std::string(prop.name) + "/" + std::to_string(e->n_sm) + "/" + pf_version();
	if (const char *f = std::getenv("PF_AUTOTUNE_CACHE")) {
		e->tune.file = f;
		tune_load(e);
	}
	*env = e;
	return PF_OK;
}

void pf_env_destroy(pf_env *env)
{
	if (!env) return;
	{
		std::lock_guard<std::mutex> lock(env->cache.mu);
		cudaSetDevice(env->device);
		if (env->cache.batch) pf_batch_destroy(env->cache.batch);  // drops its reference
		env->cache.batch = nullptr;
		cudaFree(env->cache.d_out);
		cudaFree(env->cache.d_conv);
		env->cache.d_out = env->cache.d_conv = nullptr;
	}
	env_release(env);
}

pf_status pf_model_output_offset(const pf_model_desc *model, const pf_profile_desc *profiles, uint32_t *offset_x,
                                 uint32_t *offset_y)
{
	if (!model || (!profiles && model->n_profiles)) return fail(PF_ERR_INVALID_PARAMETER, "NULL model or profiles");
	pf_model_desc m = *model;
	m.first_profile = 0;
	Geometry g;
	pf_status s = model_geometry(m, profiles, g, nullptr, m.mask_offset >= 0 && m.mask_w > 0 && m.mask_h > 0);
	if (s != PF_OK) return s;
	if (offset_x) *offset_x = g.off_x;
	if (offset_y) *offset_y = g.off_y;
	return PF_OK;
}

pf_status pf_model_output_dims(const pf_model_desc *model, const pf_profile_desc *profiles, uint32_t *out_w,
                               uint32_t *out_h)
{
	if (!model || (!profiles && model->n_profiles)) return fail(PF_ERR_INVALID_PARAMETER, "NULL model or profiles");
	pf_model_desc m = *model;
	m.first_profile = 0;
	Geometry g;
	pf_status s = model_geometry(m, profiles, g, nullptr, m.mask_offset >= 0 && m.mask_w > 0 && m.mask_h > 0);
	if (s != PF_OK) return s;
	if (out_w) *out_w = g.out_w;
	if (out_h) *out_h = g.out_h;
	return PF_OK;
}

void pf_batch_destroy(pf_batch *b)
{
	if (!b) return;
	cudaSetDevice(b->env->device);
	if (b->graph) cudaGraphExecDestroy(b->graph);
	cudaFree(b->d_models);
	cudaFree(b->d_profiles);
	cudaFree(b->d_psf_raw);
	cudaFree(b->d_mask_eval);
	cudaFree(b->d_mask_final);
	cudaFree(b->d_psf_norm);
	cudaFree(b->d_conv);
	cudaFree(b->d_direct);
	cudaFree(b->d_counter);
	cudaFree(b->d_claims);
	cudaFree(b->split.box);
	cudaFree(b->split.box_val);
	cudaFree(b->split.root);
	cudaFree(b->split.pix);
	cudaFree(b->level64.box);
	cudaFree(b->level64.val);
	cudaFree(b->level64.root);
	cudaFree(b->level64.pix);
	cudaFree(b->d_err);
	cudaFree(b->d_solves);
	cudaFree(b->d_depth);
	cudaFree(b->d_counts);
	cudaFree(b->d_psf32);
	cudaFree(b->d_tile_base_out);
	cudaFree(b->d_fft_work);
	cudaFree(b->d_fft_spec);
	cudaFree(b->d_fft_tw);
	for (void *p : b->d_fft_jobs) cudaFree(p);
	for (auto &mode : b->f32_jobs)
		for (auto &pass : mode)
			for (auto &j : pass) cudaFree(j.d_jobs);
	cudaFree(b->d_gout);
	cudaFree(b->d_gsrc);
	cudaFree(b->d_partial);
	cudaFree(b->d_chi2_partial);
	cudaFree(b->d_chi2_done);
	cudaFree(b->d_ring_partial);
	cudaFree(b->d_prow_base);
	cudaFree(b->d_bwd_counter);
	cudaFree(b->d_adj_tile_base);
	for (auto &p : b->ev_pool) {
		cudaEventDestroy(p.a);
		cudaEventDestroy(p.b);
	}
	cudaFreeHost(b->h_profiles);
	pf_env *env = b->env;
	delete b;
	if (env) env_release(env);
}

}  // extern "C"

namespace {

struct HostFftJob {
	int model, first, count, pad;
};

// Choices made for a batch by the autotuner (pf_batch_create); defaults: the
// fixed cost model.
struct ConvPlan {
	int shape = -1;                         // direct convolution block shape; -1: least tile area
	const std::vector<int8_t> *auto_fft = nullptr;  // per model, PF_CONV_AUTO: 1 FFT, 0 direct
	bool split = true;                      // single precision: a split pool unless PF_ENV_NO_SPLIT
};

// PF_SPLIT: 1 splits the single-precision subsampling trees off to other
// warps, 0 walks them where met, instead of the timed choice, for exercising
// both (-1: not set)
static int forced_split()
{
	const char *v = std::getenv("PF_SPLIT");
	if (!v || !*v) return -1;
	return std::atoi(v) != 0 ? 1 : 0;
}

// The PSF row stride (4 ceil(kw / 4) floats) shared by every model that the
// single-precision direct convolution convolves, when kernels with that
// stride compiled in exist (conv_k*.cu), else 0: the kernels that read it per
// model. PF_CONV_STRIDE=0 always takes the latter, for exercising both.
static int shared_conv_stride(const pf_batch *b)
{
	if (b->dbl) return 0;
	if (const char *v = std::getenv("PF_CONV_STRIDE")) {
		if (*v && std::atoi(v) == 0) return 0;
	}
	int k = -1;
	for (const auto &d : b->mdev) {
		if (!d.conv_required || d.use_fft) continue;
		const int w = (int)((d.psf_w + 3) & ~3u);
		if (k >= 0 && w != k) return 0;
		k = w;
	}
	return k > 0 && pf::conv_stride_fixed(k) ? k : 0;
}

// PF_CONV_SHAPE: a single-precision direct-convolution block shape to use in
// both directions instead of the chosen one, for exercising every shape
// (-1: none)
static int forced_conv_shape()
{
	const char *v = std::getenv("PF_CONV_SHAPE");
	if (!v || !*v) return -1;
	const int s = std::atoi(v);
	return s >= 0 && s < pf::conv_num_shapes<float>() ? s : -1;
}

// The convolution block shape covering the given images with the least tile area.
template <typename T>
int best_conv_shape(const std::vector<std::pair<unsigned int, unsigned int>> &dims)
{
	int best = 0;
	double best_area = -1;
	for (int s = 0; s < pf::conv_num_shapes<T>(); s++) {
		double area = 0;
		int bw = 0, bh = 0;
		pf::conv_tile_dims<T>(s, &bw, &bh);
		for (const auto &d : dims) {
			area += (double)pf::conv_tiles<T>(d.first, d.second, s) * bw * bh;
		}
		if (best_area < 0 || area < best_area) {
			best_area = area;
			best = s;
		}
	}
	return best;
}

// Whether a single-precision direct convolution with a kw x kh PSF fits the
// shared memory of a block in some block shape, both directions.
static bool direct_fits(unsigned int kw, unsigned int kh)
{
	for (int sh = 0; sh < pf::conv_num_shapes<float>(); sh++)
		if (pf::conv_smem<float>(kw, kh, sh) <= 227 * 1024) return true;
	return false;
}

// PF_CONV_AUTO in single precision takes the FFT for a model only where it
// cuts the convolution's time at least fourfold (large PSFs): its FP32
// rounding is absolute (about 1e-7 x the image peak at every pixel) where the
// direct convolution's is relative, which faint pixels and the gradients
// they carry feel; PF_CONV_FFT takes it regardless. (The bench workload's
// 25 x 25 PSF: FFT 1.06 against 2.24 ms, kept direct.)
constexpr double kFftGain = 0.25;

unsigned int next_pow2(unsigned int v)
{
	unsigned int p = 2;
	while (p < v) p <<= 1;
	return p;
}

// Picks direct or FFT convolution per model and lays out the FFT buffers and
// job lists. An explicit PF_CONV_BRUTE / PF_CONV_FFT is obeyed; PF_CONV_AUTO
// keeps the plain FP64 path on the direct convolution (the reference's
// default BRUTE convolver and summation order) and, for the FP32 path, takes
// the FFT where it costs at most kFftGain of the direct convolution by a cost
// model of this GPU: direct = 2 P^2 flop per output pixel at 35 TFLOP/s;
// FFT = its HBM bytes at 3 TB/s plus 5 N log2 N flop per transform at
// 10 TFLOP/s (large batches: by the autotuner's timings instead).
pf_status plan_fft(pf_batch *b, std::vector<HostFftJob> jobs[5], const double *psf_pool,
                   std::map<int, std::vector<HostFftJob>> f32[3][3], const ConvPlan &plan)
{
	const int nmax = b->dbl ? 4096 : 8192;
	const int per_block = b->dbl ? 4096 : 8192;  // complex elements of one ping-pong half in shared memory
	int64_t work = 0, spec = 0;
	int used_nmax = 2;
	for (size_t i = 0; i < b->mdev.size(); i++) {
		pf::ModelDev &d = b->mdev[i];
		d.use_fft = 0;
		if (!d.conv_required) continue;
		// the cropped outputs need no wrap-around below crop + psf; the
		// uncropped frame takes the whole linear convolution, draw + psf - 1.
		// Double precision: powers of two; single precision: the smallest of
		// its lengths (2^a from 64 and 3, 5, 9 x 2^a), a larger zero padding
		// leaving the linear convolution unchanged (0: none long enough)
		const unsigned int need_x = (d.uncropped ? d.draw_w : d.crop_w) + d.psf_w;
		const unsigned int need_y = (d.uncropped ? d.draw_h : d.crop_h) + d.psf_h;
		unsigned int mx, my;
		if (b->dbl) {
			mx = next_pow2(need_x);
			my = next_pow2(need_y);
		}
		else {
			const int fx = pf::fft32_size_at_least((int)std::min<unsigned int>(need_x, 1u << 30));
			const int fy = pf::fft32_size_at_least((int)std::min<unsigned int>(need_y, 1u << 30));
			mx = fx > 0 ? (unsigned int)fx : next_pow2(need_x);
			my = fy > 0 ? (unsigned int)fy : next_pow2(need_y);
		}
		bool fft = false;
		if (d.convolver == PF_CONV_FFT) {
			if ((int)mx > nmax || (int)my > nmax) {
				// longer than this precision's transforms: the cropped image is the
				// linear convolution, which the direct convolution gives (exactly,
				// more slowly); the uncropped FFT frame has no such stand-in
				if (d.uncropped) {
					return fail(PF_ERR_UNSUPPORTED, "model " + std::to_string(i) + ": crop = false with an FFT "
					                                    "above " + std::to_string(nmax) + " points in this precision");
				}
				continue;
			}
			fft = true;
		}
		else if (d.convolver == PF_CONV_AUTO && !b->dbl && (int)mx <= nmax && (int)my <= nmax &&
		         !direct_fits(d.psf_w, d.psf_h)) {
			fft = true;  // a PSF too large for the shared-memory direct convolution
		}
		else if (d.convolver == PF_CONV_AUTO && !b->dbl && (int)mx <= nmax && (int)my <= nmax && plan.auto_fft) {
			fft = (*plan.auto_fft)[i] != 0;
		}
		else if (d.convolver == PF_CONV_AUTO && !b->dbl && (int)mx <= nmax && (int)my <= nmax) {
			const double nb = mx / 2 + 1;
			const double direct_s = 2.0 * d.crop_w * d.crop_h * d.psf_w * d.psf_h / 35e12;
			const double bytes = nb * 8 * (2.0 * d.draw_h + 2.0 * d.crop_h + my) +
			                     4.0 * ((double)d.draw_w * d.draw_h + 2.0 * d.crop_w * d.crop_h);
			const double flops = 5.0 * (d.draw_h * mx * std::log2((double)mx) + 2 * nb * my * std::log2((double)my) +
			                            d.crop_h * mx * std::log2((double)mx));
			fft = bytes / 3e12 + flops / 10e12 < kFftGain * direct_s;
		}
		if (!fft) continue;
		d.use_fft = 1;
		if (b->dbl && d.fs > 1 && !d.return_fs) b->any_fft_downsample = true;
		d.fft_mx = mx;
		d.fft_my = my;
		const int64_t nb = mx / 2 + 1;
		d.fft_work_off = work;
		// the source rows in, the output rows out (in place)
		const unsigned int rows_out = d.uncropped ? d.out_h : d.crop_h;
		work += (int64_t)std::max(d.draw_h, rows_out) * nb;
		used_nmax = std::max(used_nmax, (int)std::max(mx, my));
		if (!b->dbl) {
			// models with the same PSF values and transform sizes share one spectrum
			bool shared = false;
			for (size_t q = 0; q < i && !shared; q++) {
				const pf::ModelDev &e = b->mdev[q];
				if (e.use_fft && e.fft_mx == mx && e.fft_my == my && e.psf_w == d.psf_w && e.psf_h == d.psf_h &&
				    (e.psf_off == d.psf_off ||
				     std::memcmp(psf_pool + e.psf_off, psf_pool + d.psf_off, sizeof(double) * d.psf_w * d.psf_h) == 0)) {
					d.fft_spec_off = e.fft_spec_off;
					shared = true;
				}
			}
			const int rpj_x = pf::fft32_rows_per_job((int)mx), cpj_y = pf::fft32_cols_per_job((int)my);
			if (rpj_x <= 0 || cpj_y <= 0) {
				return fail(PF_ERR_UNSUPPORTED, "model " + std::to_string(i) + ": no single-precision FFT of " +
				                                    std::to_string(mx) + " x " + std::to_string(my) + " points");
			}
			auto add = [&](int mode, int pass, int n, int count, int per) {
				for (int r = 0; r < count; r += per) f32[mode][pass][n].push_back({(int)i, r, std::min(per, count - r), 0});
			};
			if (!shared) {
				d.fft_spec_off = spec;
				spec += (int64_t)my * nb;
				add(2, 0, (int)mx, (int)d.psf_h, rpj_x);
				add(2, 1, (int)my, (int)nb, cpj_y);
			}
			add(0, 0, (int)mx, (int)d.draw_h, rpj_x);
			add(0, 1, (int)my, (int)nb, cpj_y);
			add(0, 2, (int)mx, (int)d.crop_h, rpj_x);
			add(1, 0, (int)mx, (int)d.crop_h, rpj_x);
			add(1, 1, (int)my, (int)nb, cpj_y);
			add(1, 2, (int)mx, (int)d.draw_h, rpj_x);
			b->any_fft = true;
			continue;
		}
		d.fft_spec_off = spec;
		spec += (int64_t)my * nb;
		const int cr = std::max(1, std::min(16, per_block / (int)mx));
		const int cc = std::max(1, std::min(16, per_block / (int)my));
		for (unsigned int r = 0; r < d.draw_h; r += cr) jobs[0].push_back({(int)i, (int)r, (int)std::min<unsigned int>(cr, d.draw_h - r), 0});
		for (int c = 0; c < nb; c += cc) jobs[1].push_back({(int)i, c, (int)std::min<int64_t>(cc, nb - c), 0});
		for (unsigned int r = 0; r < rows_out; r += cr) jobs[2].push_back({(int)i, (int)r, (int)std::min<unsigned int>(cr, rows_out - r), 0});
		for (unsigned int r = 0; r < d.psf_h; r += cr) jobs[3].push_back({(int)i, (int)r, (int)std::min<unsigned int>(cr, d.psf_h - r), 0});
		for (int c = 0; c < nb; c += cc) jobs[4].push_back({(int)i, c, (int)std::min<int64_t>(cc, nb - c), 0});
		b->any_fft = true;
	}
	b->fft_nmax = used_nmax;
	b->fft_work_elems = work;
	b->fft_spec_elems = spec;
	// the shared memory of the largest job: two halves of count x n complex values
	size_t smem = 0;
	for (int p = 0; p < 5; p++) {
		for (const auto &j : jobs[p]) {
			const pf::ModelDev &d = b->mdev[j.model];
			const int n = (p == 1 || p == 4) ? (int)d.fft_my : (int)d.fft_mx;
			smem = std::max(smem, b->dbl ? pf::fft_smem<double>(n, j.count) : pf::fft_smem<float>(n, j.count));
		}
	}
	b->fft_smem_bytes = smem;
	return PF_OK;
}

}  // namespace

extern "C" {

static pf_status batch_create_impl(pf_env *env, const pf_model_desc *models, size_t n_models,
                                   const pf_profile_desc *profiles, size_t n_profiles, const double *psf_pool,
                                   size_t psf_pool_len, const uint8_t *mask_pool, size_t mask_pool_len, pf_batch *b,
                                   const ConvPlan &plan)
{
	std::vector<uint8_t> mask_eval, mask_final;
	std::vector<int64_t> eval_off(n_models, -1), final_off(n_models, -1);
	b->env = env;
	b->dbl = (env->flags & PF_ENV_DOUBLE) != 0;
	b->models.assign(models, models + n_models);
	b->profiles.assign(profiles, profiles + n_profiles);
	b->mdev.resize(n_models);
	std::vector<int32_t> owner(n_profiles, -1);
	int64_t draw_off = 0, out_off = 0, tile_base = 0;
	bool any_psf = false;
	for (size_t i = 0; i < n_models; i++) {
		const pf_model_desc &m = models[i];
		if ((uint64_t)m.first_profile + m.n_profiles > n_profiles) {
			return fail(PF_ERR_INVALID_PARAMETER, "model " + std::to_string(i) + ": profile range out of bounds");
		}
		if (m.psf_offset >= 0 && (uint64_t)m.psf_offset + (uint64_t)m.psf_w * m.psf_h > psf_pool_len) {
			return fail(PF_ERR_INVALID_PARAMETER, "model " + std::to_string(i) + ": PSF outside the PSF pool");
		}
		const uint8_t *mask = nullptr;
		if (mask_pool && m.mask_offset >= 0) {
			mask = mask_pool + m.mask_offset;
			if ((uint64_t)m.mask_offset + (uint64_t)m.mask_w * m.mask_h > mask_pool_len) {
				return fail(PF_ERR_INVALID_PARAMETER, "model " + std::to_string(i) + ": mask outside the mask pool");
			}
		}
		Geometry g;
		pf_status s = model_geometry(m, profiles, g, mask);
		if (s != PF_OK) {
			g_last_error = "model " + std::to_string(i) + ": " + g_last_error;
			return s;
		}
		if (mask) {
			// the evaluation mask (drawing dimensions) and, after an adjustment,
			// the model's own mask for the output (src/model.cpp:269-317)
			eval_off[i] = (int64_t)mask_eval.size();
			if (m.adjust_mask && g.mask_needs_adjustment) {
				std::vector<uint8_t> adj;
				adjusted_mask(m, g, mask, adj);
				mask_eval.insert(mask_eval.end(), adj.begin(), adj.end());
				final_off[i] = (int64_t)mask_final.size();
				mask_final.insert(mask_final.end(), mask, mask + (size_t)m.width * m.height);
			}
			else {
				// used as given: the model's dimensions without padding or
				// finesampling (adjustable), else the drawing dimensions
				const size_t n = (size_t)g.draw_w * g.draw_h;
				if ((uint64_t)m.mask_offset + n > mask_pool_len) {
					return fail(PF_ERR_INVALID_PARAMETER, "model " + std::to_string(i) + ": mask outside the mask pool");
				}
				mask_eval.insert(mask_eval.end(), mask, mask + n);
			}
		}
		for (uint32_t q = 0; q < m.n_profiles; q++) {
			if (owner[m.first_profile + q] != -1) {
				return fail(PF_ERR_INVALID_PARAMETER, "profile " + std::to_string(m.first_profile + q) +
				                                          " belongs to two models");
			}
			owner[m.first_profile + q] = (int32_t)i;
		}
		pf::ModelDev &d = b->mdev[i];
		std::memset(&d, 0, sizeof(d));
		d.width = m.width;
		d.height = m.height;
		d.fs = m.finesampling;
		d.return_fs = m.return_finesampled != 0;
		d.draw_w = g.draw_w;
		d.draw_h = g.draw_h;
		d.pad_x = g.pad_x;
		d.pad_y = g.pad_y;
		d.crop_w = g.crop_w;
		d.crop_h = g.crop_h;
		d.out_w = g.out_w;
		d.out_h = g.out_h;
		if (g.uncropped) {
			if (!b->dbl) {
				return fail(PF_ERR_UNSUPPORTED, "crop = false with the FFT convolver is supported in the double "
				                                "precision environment only");
			}
			d.uncropped = 1;
			d.ufx0 = g.ufx0;
			d.ufy0 = g.ufy0;
			d.udx0 = g.udx0;
			d.udy0 = g.udy0;
		}
		d.scale_x = m.scale_x;
		d.scale_y = m.scale_y;
		d.sx = m.scale_x / m.finesampling;
		d.sy = m.scale_y / m.finesampling;
		d.fsx_hi = (float)d.sx;
		d.fsx_lo = (float)(d.sx - (double)d.fsx_hi);
		d.fsy_hi = (float)d.sy;
		d.fsy_lo = (float)(d.sy - (double)d.fsy_hi);
		d.fscale_x = (float)m.scale_x;
		d.fscale_y = (float)m.scale_y;
		d.magzero = m.magzero;
		d.first_profile = (int32_t)m.first_profile;
		d.n_profiles = (int32_t)m.n_profiles;
		d.conv_required = g.conv;
		d.direct_required = g.direct;
		d.convolver = m.convolver;
		const bool has_psf = m.psf_offset >= 0 && m.psf_w > 0 && m.psf_h > 0;
		d.psf_off = has_psf ? m.psf_offset : -1;
		any_psf |= has_psf;
		d.psf_w = m.psf_w;
		d.psf_h = m.psf_h;
		d.psf_scale_x = m.psf_scale_x;
		d.psf_scale_y = m.psf_scale_y;
		d.draw_off = draw_off;
		d.out_off = out_off;
		d.tile_base = tile_base;
		d.tiles_per_row = (g.draw_w + 31) / 32;
		draw_off += (int64_t)g.draw_w * g.draw_h;
		out_off += (int64_t)g.out_w * g.out_h;
		tile_base += (int64_t)d.tiles_per_row * g.draw_h;
	}
	b->draw_total = (size_t)draw_off;
	b->total_out = (uint64_t)out_off;
	b->n_tiles = tile_base;
	if (b->n_tiles >= (1ll << 32)) {
		return fail(PF_ERR_UNSUPPORTED, "batch too large: more than 2^32 tiles of 32 pixels");
	}
	std::vector<HostFftJob> fft_jobs[5];
	std::map<int, std::vector<HostFftJob>> f32_jobs[3][3];
	pf_status fs = plan_fft(b, fft_jobs, psf_pool, f32_jobs, plan);
	if (fs != PF_OK) return fs;
	std::vector<long long> tile_base_out(std::max<size_t>(1, n_models), 0);
	if (!b->dbl) {
		unsigned int max_kw = 1, max_kh = 1;
		std::vector<std::pair<unsigned int, unsigned int>> conv_dims;
		for (size_t i = 0; i < n_models; i++) {
			const pf::ModelDev &d = b->mdev[i];
			if (!d.use_fft) conv_dims.push_back({d.crop_w, d.crop_h});
		}
		b->fwd_shape = plan.shape >= 0 ? plan.shape : best_conv_shape<float>(conv_dims);
		if (forced_conv_shape() >= 0) b->fwd_shape = forced_conv_shape();
		for (size_t i = 0; i < n_models; i++) {
			const pf::ModelDev &d = b->mdev[i];
			if (!d.use_fft && d.conv_required) {
				max_kw = std::max(max_kw, d.psf_w);
				max_kh = std::max(max_kh, d.psf_h);
			}
		}
		if (pf::conv_smem<float>(max_kw, max_kh, b->fwd_shape) > 227 * 1024 && forced_conv_shape() < 0) {
			// the chosen block shape's patch too large for this PSF: the first one that fits
			for (int sh = 0; sh < pf::conv_num_shapes<float>(); sh++) {
				if (pf::conv_smem<float>(max_kw, max_kh, sh) <= 227 * 1024) {
					b->fwd_shape = sh;
					break;
				}
			}
		}
		long long t = 0;
		for (size_t i = 0; i < n_models; i++) {
			const pf::ModelDev &d = b->mdev[i];
			tile_base_out[i] = t;
			if (!d.use_fft) t += pf::conv_tiles<float>(d.crop_w, d.crop_h, b->fwd_shape);  // FFT models: their last pass
			b->any_downsample |= d.fs > 1 && !d.return_fs;
		}
		b->n_out_tiles = t;
		b->finish_smem = pf::conv_smem<float>(max_kw, max_kh, b->fwd_shape);
		b->conv_kwp = shared_conv_stride(b);
		if (b->finish_smem > 227 * 1024) {
			return fail(PF_ERR_UNSUPPORTED, "PSF too large for the single-precision direct convolution's shared "
			                                "memory: request the FFT convolver or double precision");
		}
	}

	PF_CUDA_TRY(cudaMallocHost(&b->h_profiles, sizeof(pf::ProfileDev) * std::max<size_t>(1, n_profiles)));
	std::memset(b->h_profiles, 0, sizeof(pf::ProfileDev) * std::max<size_t>(1, n_profiles));
	int64_t depth_off = 0;
	for (size_t i = 0; i < n_profiles; i++) {
		const pf_profile_desc &s = profiles[i];
		pf::ProfileDev &p = b->h_profiles[i];
		p.kind = s.kind;
		p.convolve = s.convolve != 0;
		p.rough = s.rough != 0;
		p.adjust = s.adjust != 0;
		p.rescale_flux = s.rescale_flux != 0;
		p.resolution_in = s.resolution;
		p.max_recursions = s.max_recursions;
		p.acc_in = s.acc;
		p.rscale_switch_in = s.rscale_switch;
		p.rscale_max_in = s.rscale_max;
		std::memcpy(p.par, s.par, sizeof(p.par));
		p.model = owner[i] < 0 ? 0 : owner[i];
		p.depth_off = depth_off;
		if (owner[i] >= 0) {
			const pf::ModelDev &m = b->mdev[owner[i]];
			depth_off += (int64_t)m.draw_w * m.draw_h;
		}
		if (owner[i] < 0) {
			p.kind = PF_NULL;  // not referenced by any model
		}
	}
	b->depth_total = (size_t)depth_off;

	PF_CUDA_TRY(cudaMalloc(&b->d_models, sizeof(pf::ModelDev) * std::max<size_t>(1, n_models)));
	PF_CUDA_TRY(cudaMalloc(&b->d_profiles, sizeof(pf::ProfileDev) * std::max<size_t>(1, n_profiles)));
	// the eval kernels' two work counters, then the split pool's (reset by the setup kernel)
	PF_CUDA_TRY(cudaMalloc(&b->d_counter, (2 + pf::kSplitCounters) * sizeof(unsigned int)));
	PF_CUDA_TRY(cudaMemset(b->d_counter, 0, (2 + pf::kSplitCounters) * sizeof(unsigned int)));
	b->sersic_only = true;
	for (size_t i = 0; i < n_profiles; i++) {
		const int k = b->h_profiles[i].kind;
		if (k == PF_USER && !b->dbl) {
			return fail(PF_ERR_UNSUPPORTED, "profile " + std::to_string(i) + ": the user-defined profile " +
			                                    pf::user::name() + " is evaluated in double precision only");
		}
		if (is_radial(k) && k != PF_SERSIC) b->sersic_only = false;
	}
	if (!b->dbl) {
		if (pf::eval32_items((long long)n_profiles, b->n_tiles) >= (1ll << 31)) {
			return fail(PF_ERR_UNSUPPORTED, "batch too large for one single-precision evaluation pass");
		}
		PF_CUDA_TRY(cudaMalloc(&b->d_claims, sizeof(unsigned int) * (size_t)std::max<long long>(1, (b->n_tiles + 31) / 32)));
		if (!(env->flags & PF_ENV_NO_SPLIT) && plan.split) {
			// room for a split record per drawing pixel up to 2^21 and 16 boxes per
			// record up to 2^23 (about 470 MB at most); a split that finds no room
			// is walked by the warp that meets it instead
			pf::SplitPool &sp = b->split;
			sp.cap_pix = (unsigned int)std::min<size_t>(std::max<size_t>(1, b->draw_total), 1u << 21);
			sp.cap_root = sp.cap_pix;
			sp.cap_box = (unsigned int)std::min<size_t>(std::max<size_t>(16 * (size_t)sp.cap_root, 1u << 16), 1u << 23);
			sp.min_fail = kSplitMinFail;
			PF_CUDA_TRY(cudaMalloc(&sp.box, sizeof(pf::SplitBox) * sp.cap_box));
			PF_CUDA_TRY(cudaMalloc(&sp.box_val, sizeof(float) * sp.cap_box));
			PF_CUDA_TRY(cudaMalloc(&sp.root, sizeof(pf::SplitRoot) * sp.cap_root));
			PF_CUDA_TRY(cudaMalloc(&sp.pix, sizeof(pf::SplitPixel) * sp.cap_pix));
			sp.cnt = b->d_counter + 2;
		}
	}
	if (b->dbl && !(env->flags & PF_ENV_NO_SPLIT)) {
		// the recursion levels a tree can reach: max_recursions, 10 for a
		// sersic's central pixel (src/sersic.cpp:339-345), at most kMaxLevels - 1
		int top = -1;
		for (size_t i = 0; i < n_profiles; i++) {
			const pf::ProfileDev &d = b->h_profiles[i];
			if (!is_radial(d.kind) || d.rough) continue;
			unsigned int rec = d.max_recursions;
			if (d.kind == PF_SERSIC && d.adjust) rec = std::max(rec, 10u);
			top = std::max(top, (int)std::min<unsigned int>(rec, pf::kMaxLevels - 1));
		}
		if (top >= 0) {
			// room for a subsampled profile per drawing pixel up to 2^21, twice
			// as many boxes within [2^15, 2^20] and 64 sub-point values per box
			// (about 640 MB at most); a tree that finds no room is walked by the
			// warp that meets it instead
			pf::LevelPool64 &lp = b->level64;
			lp.cap_pix = (unsigned int)std::min<size_t>(std::max<size_t>(1, b->draw_total), 1u << 21);
			lp.cap_root = lp.cap_pix;
			lp.cap_box = (unsigned int)std::min<size_t>(std::max<size_t>(2 * (size_t)lp.cap_root, 1u << 15), 1u << 20);
			if (const char *cap = std::getenv("PF_LEVEL_POOL_BOXES")) {
				// a smaller pool, for exercising the walks that a full pool falls back to
				lp.cap_box = (unsigned int)std::max(1l, std::min(std::atol(cap), (long)lp.cap_box));
			}
			lp.cap_val = 64ull * lp.cap_box;
			PF_CUDA_TRY(cudaMalloc(&lp.box, sizeof(pf::LevelBox64) * lp.cap_box));
			PF_CUDA_TRY(cudaMalloc(&lp.val, sizeof(double) * lp.cap_val));
			PF_CUDA_TRY(cudaMalloc(&lp.root, sizeof(pf::LevelRoot64) * lp.cap_root));
			PF_CUDA_TRY(cudaMalloc(&lp.pix, sizeof(pf::LevelPixel64) * lp.cap_pix));
			lp.cnt = b->d_counter + 2;
			b->levels64 = top + 1;
		}
	}
	// [0] device-limit flags, [1] the last pass's first invalid profile (index << 5 | rule)
	PF_CUDA_TRY(cudaMalloc(&b->d_err, 2 * sizeof(unsigned int)));
	// per profile the three solves, then the nser each was made for (NaN: none yet)
	PF_CUDA_TRY(cudaMalloc(&b->d_solves, sizeof(double) * 6 * std::max<size_t>(1, n_profiles)));
	PF_CUDA_TRY(cudaMemset(b->d_solves, 0xff, sizeof(double) * 6 * std::max<size_t>(1, n_profiles)));
	PF_CUDA_TRY(cudaMemset(b->d_err, 0, sizeof(unsigned int)));
	PF_CUDA_TRY(cudaMemset(b->d_err + 1, 0xff, sizeof(unsigned int)));
	const size_t elem = b->dbl ? sizeof(double) : sizeof(float);
	PF_CUDA_TRY(cudaMalloc(&b->d_conv, elem * std::max<size_t>(1, b->draw_total)));
	PF_CUDA_TRY(cudaMalloc(&b->d_direct, elem * std::max<size_t>(1, b->draw_total)));
	b->psf_len = psf_pool_len;
	if (psf_pool_len) {
		PF_CUDA_TRY(cudaMalloc(&b->d_psf_raw, sizeof(double) * psf_pool_len));
		PF_CUDA_TRY(cudaMalloc(&b->d_psf_norm, sizeof(double) * psf_pool_len));
		PF_CUDA_TRY(cudaMemcpy(b->d_psf_raw, psf_pool, sizeof(double) * psf_pool_len, cudaMemcpyHostToDevice));
	}
	if (!mask_eval.empty()) {
		PF_CUDA_TRY(cudaMalloc(&b->d_mask_eval, mask_eval.size()));
		PF_CUDA_TRY(cudaMemcpy(b->d_mask_eval, mask_eval.data(), mask_eval.size(), cudaMemcpyHostToDevice));
	}
	if (!mask_final.empty()) {
		PF_CUDA_TRY(cudaMalloc(&b->d_mask_final, mask_final.size()));
		PF_CUDA_TRY(cudaMemcpy(b->d_mask_final, mask_final.data(), mask_final.size(), cudaMemcpyHostToDevice));
	}
	for (size_t i = 0; i < n_models; i++) {
		pf::ModelDev &d = b->mdev[i];
		d.mask_eval = eval_off[i] >= 0 ? b->d_mask_eval + eval_off[i] : nullptr;
		d.mask_final = final_off[i] >= 0 ? b->d_mask_final + final_off[i] : nullptr;
		d.mask_final_w = models[i].width;
		d.mask_final_div = models[i].finesampling > 1 && models[i].return_finesampled ? models[i].finesampling : 1;
	}
	if (n_models) {
		PF_CUDA_TRY(cudaMemcpy(b->d_models, b->mdev.data(), sizeof(pf::ModelDev) * n_models, cudaMemcpyHostToDevice));
	}
	if (any_psf) {
		// PSF normalisation (Model::set_psf), once per batch
		pf::launch_setup(b->d_models, b->d_profiles, 0, (int)n_models, b->d_counter, b->d_err, b->d_psf_raw,
		                 b->d_psf_norm, true, b->d_solves, 0, env->stream);
		if (!b->dbl) {
			PF_CUDA_TRY(cudaMalloc(&b->d_psf32, sizeof(float) * psf_pool_len));
			pf::launch_psf_to_float(b->d_psf_norm, b->d_psf32, (long long)psf_pool_len, env->stream);
		}
		PF_CUDA_TRY(cudaGetLastError());
		PF_CUDA_TRY(cudaStreamSynchronize(env->stream));
	}
	if (!b->dbl) {
		PF_CUDA_TRY(cudaMalloc(&b->d_tile_base_out, sizeof(long long) * tile_base_out.size()));
		PF_CUDA_TRY(cudaMemcpy(b->d_tile_base_out, tile_base_out.data(), sizeof(long long) * tile_base_out.size(),
		                       cudaMemcpyHostToDevice));
		PF_CUDA_TRY(pf::conv_configure<float>(b->finish_smem, b->fwd_shape, b->conv_kwp));
	}
	if (b->any_fft) {
		// FFT buffers, twiddles and, once per batch, the PSF spectra
		if ((size_t)pf::fft_job_size() != sizeof(HostFftJob)) return fail(PF_ERR_INTERNAL, "FFT job layout");
		const size_t celem = b->dbl ? 2 * sizeof(double) : 2 * sizeof(float);
		PF_CUDA_TRY(cudaMalloc(&b->d_fft_work, celem * std::max<int64_t>(1, b->fft_work_elems)));
		PF_CUDA_TRY(cudaMalloc(&b->d_fft_spec, celem * std::max<int64_t>(1, b->fft_spec_elems)));
		PF_CUDA_TRY(cudaMalloc(&b->d_fft_tw, b->dbl ? celem * (b->fft_nmax / 2)
		                                            : sizeof(float) * 2 * (size_t)pf::fft32_twiddle_len()));
		for (int p = 0; p < 5; p++) {
			b->fft_njobs[p] = (int)fft_jobs[p].size();
			PF_CUDA_TRY(cudaMalloc(&b->d_fft_jobs[p], sizeof(HostFftJob) * std::max<size_t>(1, fft_jobs[p].size())));
			if (!fft_jobs[p].empty()) {
				PF_CUDA_TRY(cudaMemcpy(b->d_fft_jobs[p], fft_jobs[p].data(), sizeof(HostFftJob) * fft_jobs[p].size(),
				                       cudaMemcpyHostToDevice));
			}
		}
		if (b->dbl && b->fft_smem_bytes > 227 * 1024) return fail(PF_ERR_UNSUPPORTED, "FFT too large for shared memory");
		if (b->dbl) {
			PF_CUDA_TRY(pf::fft_configure<double>(b->fft_smem_bytes));
			pf::launch_twiddles<double>(b->d_fft_tw, b->fft_nmax, env->stream);
			for (int p = 3; p <= 4; p++) {
				pf::launch_fft_pass<double>(p, b->d_models, b->d_fft_jobs[p], b->fft_njobs[p], nullptr, b->d_psf_norm,
				                            b->d_fft_work, b->d_fft_spec, nullptr, nullptr, nullptr, b->d_fft_tw,
				                            b->fft_nmax, b->fft_smem_bytes, env->stream);
			}
		}
		else {
			for (int mode = 0; mode < 3; mode++) {
				for (int pass = 0; pass < 3; pass++) {
					for (const auto &kv : f32_jobs[mode][pass]) {
						pf_batch::Fft32Jobs j;
						j.n = kv.first;
						j.n_jobs = (int)kv.second.size();
						PF_CUDA_TRY(cudaMalloc(&j.d_jobs, sizeof(HostFftJob) * kv.second.size()));
						b->f32_jobs[mode][pass].push_back(j);
						PF_CUDA_TRY(cudaMemcpy(j.d_jobs, kv.second.data(), sizeof(HostFftJob) * kv.second.size(),
						                       cudaMemcpyHostToDevice));
					}
				}
			}
			PF_CUDA_TRY(pf::fft32_configure());
			pf::launch_fft32_twiddles(b->d_fft_tw, env->stream);
			for (int pass = 0; pass < 2; pass++) {
				for (const auto &j : b->f32_jobs[2][pass]) {
					pf::launch_fft32(pass, 2, j.n, j.d_jobs, j.n_jobs, b->d_models, nullptr, b->d_psf32, b->d_fft_work,
					                 b->d_fft_spec, nullptr, nullptr, b->d_fft_tw, env->stream);
				}
			}
		}
		PF_CUDA_TRY(cudaGetLastError());
		PF_CUDA_TRY(cudaStreamSynchronize(env->stream));
	}
	b->params_dirty = true;
	return PF_OK;
}

static pf_status create_planned(pf_env *env, const pf_model_desc *models, size_t n_models,
                                const pf_profile_desc *profiles, size_t n_profiles, const double *psf_pool,
                                size_t psf_pool_len, const uint8_t *mask_pool, size_t mask_pool_len,
                                const ConvPlan &plan, pf_batch **batch)
{
	*batch = nullptr;
	pf_batch *b = new (std::nothrow) pf_batch();
	if (!b) return fail(PF_ERR_NO_MEMORY, "out of host memory");
	b->env = env;
	env->refs.fetch_add(1);
	clear_stale_error();
	pf_status s = batch_create_impl(env, models, n_models, profiles, n_profiles, psf_pool, psf_pool_len, mask_pool,
	                                mask_pool_len, b, plan);
	if (s != PF_OK) {
		pf_batch_destroy(b);
		return s;
	}
	*batch = b;
	return PF_OK;
}

// Autotuner timings (ms, best of three after one warm-up launch) of the
// forward convolution of a batch: its direct convolution with block shape
// `shape` over every model it convolves directly, or its FFT passes.
static double time_forward_conv(pf_batch *b, int shape, bool fft, float *out)
{
	cudaStream_t st = b->env->stream;
	const int n_models = (int)b->mdev.size();
	std::vector<long long> base(std::max<size_t>(1, b->mdev.size()), 0);
	long long t = 0;
	unsigned int max_kw = 1, max_kh = 1;
	for (size_t i = 0; i < b->mdev.size(); i++) {
		const pf::ModelDev &d = b->mdev[i];
		base[i] = t;
		if (d.use_fft) continue;
		t += pf::conv_tiles<float>(d.crop_w, d.crop_h, shape);
		if (d.conv_required) {
			max_kw = std::max(max_kw, d.psf_w);
			max_kh = std::max(max_kh, d.psf_h);
		}
	}
	const size_t smem = pf::conv_smem<float>(max_kw, max_kh, shape);
	const int kwp = shared_conv_stride(b);
	long long *d_base = nullptr;
	if (!fft && (smem > 227 * 1024 || cudaMalloc(&d_base, sizeof(long long) * base.size()) != cudaSuccess)) return -1;
	if (!fft) {
		cudaMemcpy(d_base, base.data(), sizeof(long long) * base.size(), cudaMemcpyHostToDevice);
		pf::conv_configure<float>(smem, shape, kwp);
	}
	cudaEvent_t e0, e1;
	cudaEventCreate(&e0);
	cudaEventCreate(&e1);
	double best = -1;
	for (int rep = 0; rep < 4; rep++) {
		cudaEventRecord(e0, st);
		if (fft) {
			for (int pass = 0; pass < 3; pass++) {
				for (const auto &j : b->f32_jobs[0][pass]) {
					pf::launch_fft32(pass, 0, j.n, j.d_jobs, j.n_jobs, b->d_models, (const float *)b->d_conv, nullptr,
					                 b->d_fft_work, b->d_fft_spec, (const float *)b->d_direct, out, b->d_fft_tw, st);
				}
			}
		}
		else if (t > 0) {
			pf::launch_conv<float>(0, shape, kwp, b->d_models, n_models, b->d_psf32, (const float *)b->d_conv,
			                       (const float *)b->d_direct, out, d_base, t, smem, b->env->n_sm, st);
		}
		cudaEventRecord(e1, st);
		cudaEventSynchronize(e1);
		float ms = 0;
		cudaEventElapsedTime(&ms, e0, e1);
		if (rep > 0 && (best < 0 || ms < best)) best = ms;
	}
	cudaEventDestroy(e0);
	cudaEventDestroy(e1);
	cudaFree(d_base);
	if (!fft) pf::conv_configure<float>(b->finish_smem, b->fwd_shape, b->conv_kwp);
	return cudaGetLastError() == cudaSuccess ? best : -1;
}

// Autotuner timing (ms, best of three after a warm-up) of a single-precision
// batch's setup and evaluation passes, with its subsampling trees split off
// to other warps (split) or walked where met.
static double time_eval(pf_batch *b, bool split);

// The batch's split pool given back: its trees walked where met from now on.
static void release_split_pool(pf_batch *b)
{
	cudaFree(b->split.box);
	cudaFree(b->split.box_val);
	cudaFree(b->split.root);
	cudaFree(b->split.pix);
	b->split = pf::SplitPool{};
}

static double time_eval(pf_batch *b, bool split)
{
	cudaStream_t st = b->env->stream;
	const int n_models = (int)b->mdev.size(), n_profiles = (int)b->profiles.size();
	if (b->params_dirty) {
		if (cudaMemcpyAsync(b->d_profiles, b->h_profiles, sizeof(pf::ProfileDev) * std::max(1, n_profiles),
		                    cudaMemcpyHostToDevice, st) != cudaSuccess) return -1;
		b->params_dirty = false;
	}
	const pf::SplitPool pool = split ? b->split : pf::SplitPool{};
	cudaEvent_t e0, e1;
	cudaEventCreate(&e0);
	cudaEventCreate(&e1);
	double best = -1;
	for (int rep = 0; rep < 4; rep++) {
		cudaEventRecord(e0, st);
		pf::launch_setup(b->d_models, b->d_profiles, n_profiles, n_models, b->d_counter, b->d_err, nullptr, nullptr,
		                 false, b->d_solves, b->adjoint ? 1 : 0, st);
		cudaMemsetAsync(b->d_claims, 0, sizeof(unsigned int) * (size_t)std::max<long long>(1, (b->n_tiles + 31) / 32),
		                st);
		pf::launch_eval32(b->d_models, n_models, b->d_profiles, n_profiles, b->d_psf_norm, (float *)b->d_conv,
		                  (float *)b->d_direct, b->n_tiles, b->d_counter, b->d_claims, pf::DebugRec{nullptr, nullptr},
		                  pool, b->sersic_only, b->env->n_sm, st);
		cudaEventRecord(e1, st);
		cudaEventSynchronize(e1);
		float ms = 0;
		cudaEventElapsedTime(&ms, e0, e1);
		if (rep > 0 && (best < 0 || ms < best)) best = ms;
	}
	cudaEventDestroy(e0);
	cudaEventDestroy(e1);
	return cudaGetLastError() == cudaSuccess ? best : -1;
}

// Autotuner timing (ms, best of three after a warm-up) of the adjoint direct
// convolution of a batch with block shape `shape`, into its drawing-area
// cotangent buffer.
static double time_adjoint_conv(pf_batch *b, int shape)
{
	cudaStream_t st = b->env->stream;
	const int n_models = (int)b->mdev.size();
	std::vector<long long> base(std::max<size_t>(1, b->mdev.size()), 0);
	long long t = 0;
	unsigned int max_kw = 1, max_kh = 1;
	for (size_t i = 0; i < b->mdev.size(); i++) {
		const pf::ModelDev &m = b->mdev[i];
		base[i] = t;
		if (!m.conv_required || m.use_fft) continue;
		t += pf::conv_tiles<float>(m.draw_w, m.draw_h, shape);
		max_kw = std::max(max_kw, m.psf_w);
		max_kh = std::max(max_kh, m.psf_h);
	}
	const size_t smem = pf::conv_smem<float>(max_kw, max_kh, shape);
	long long *d_base = nullptr;
	if (t == 0 || smem > 227 * 1024 || cudaMalloc(&d_base, sizeof(long long) * base.size()) != cudaSuccess) return -1;
	cudaMemcpy(d_base, base.data(), sizeof(long long) * base.size(), cudaMemcpyHostToDevice);
	const int kwp = shared_conv_stride(b);
	pf::conv_configure<float>(smem, shape, kwp);
	cudaEvent_t e0, e1;
	cudaEventCreate(&e0);
	cudaEventCreate(&e1);
	double best = -1;
	for (int rep = 0; rep < 4; rep++) {
		cudaEventRecord(e0, st);
		pf::launch_conv<float>(1, shape, kwp, b->d_models, n_models, b->d_psf32, (const float *)b->d_gout, nullptr,
		                       (float *)b->d_gsrc, d_base, t, smem, b->env->n_sm, st);
		cudaEventRecord(e1, st);
		cudaEventSynchronize(e1);
		float ms = 0;
		cudaEventElapsedTime(&ms, e0, e1);
		if (rep > 0 && (best < 0 || ms < best)) best = ms;
	}
	cudaEventDestroy(e0);
	cudaEventDestroy(e1);
	cudaFree(d_base);
	return cudaGetLastError() == cudaSuccess ? best : -1;
}

pf_status pf_batch_create(pf_env *env, const pf_model_desc *models, size_t n_models, const pf_profile_desc *profiles,
                          size_t n_profiles, const double *psf_pool, size_t psf_pool_len, pf_batch **batch)
{
	return pf_batch_create_masked(env, models, n_models, profiles, n_profiles, psf_pool, psf_pool_len, nullptr, 0,
	                              batch);
}

pf_status pf_batch_create_masked(pf_env *env, const pf_model_desc *models, size_t n_models,
                                 const pf_profile_desc *profiles, size_t n_profiles, const double *psf_pool,
                                 size_t psf_pool_len, const uint8_t *mask_pool, size_t mask_pool_len,
                                 pf_batch **batch)
{
	if (!env || !batch || (!models && n_models) || (!profiles && n_profiles) || (!psf_pool && psf_pool_len) ||
	    (!mask_pool && mask_pool_len)) {
		return fail(PF_ERR_INVALID_PARAMETER, "pf_batch_create: NULL argument");
	}
	*batch = nullptr;
	PF_CUDA_TRY(cudaSetDevice(env->device));
	ConvPlan fixed;
	const int fsplit = forced_split();
	if (fsplit == 0) fixed.split = false;
	bool tune = !(env->flags & (PF_ENV_DOUBLE | PF_ENV_NO_AUTOTUNE));
	uint64_t out_pixels = 0;
	bool any_auto = false;
	for (size_t i = 0; i < n_models && tune; i++) {
		out_pixels += (uint64_t)models[i].width * models[i].height;
		any_auto |= models[i].convolver == PF_CONV_AUTO && models[i].psf_offset >= 0 && models[i].psf_w > 0;
	}
	// the split of the subsampling trees is timed for every single-precision
	// batch (it loses on some small ones, e.g. one 1000 x 1000 model); the
	// convolution methods and shapes only from 2^22 output pixels up
	const bool tune_split = tune && fsplit < 0;
	const uint64_t key = tune ? tune_key(env, models, n_models, profiles, n_profiles) : 0;
	tune = tune && out_pixels >= (1ull << 22) && any_auto;
	TuneEntry known;
	const bool have = key && tune_lookup(env, key, &known);
	if (!tune) {
		pf_status s = create_planned(env, models, n_models, profiles, n_profiles, psf_pool, psf_pool_len, mask_pool,
		                             mask_pool_len, fixed, batch);
		if (s == PF_OK && key) (*batch)->tune_key = key;
		if (s == PF_OK && tune_split && (*batch)->split.box) {
			// the evaluation timed with and without its subsampling trees split
			// off (below), or the decision taken from the cache
			bool walk;
			if (have && known.split >= 0) {
				walk = known.split == 0;
				std::lock_guard<std::mutex> lock(env->tune.mu);
				env->tune.reused++;
			}
			else {
				const double t_split = time_eval(*batch, true), t_walk = time_eval(*batch, false);
				walk = t_walk > 0 && t_split > 0 && t_walk < t_split;
				tune_store(env, key, [&](TuneEntry &t) { t.split = walk ? 0 : 1; });
			}
			if (walk) release_split_pool(*batch);
		}
		return s;
	}
	if (have && known.fwd_shape >= 0 && known.split >= 0 && known.fft.size() == n_models) {
		// this layout's decisions, taken before (in this environment or from its cache file)
		ConvPlan fin;
		fin.shape = known.fwd_shape;
		fin.auto_fft = &known.fft;
		fin.split = fsplit >= 0 ? fsplit == 1 : known.split == 1;
		pf_status s = create_planned(env, models, n_models, profiles, n_profiles, psf_pool, psf_pool_len, mask_pool,
		                             mask_pool_len, fin, batch);
		if (s == PF_OK) {
			(*batch)->tune_key = key;
			std::lock_guard<std::mutex> lock(env->tune.mu);
			env->tune.reused++;
		}
		return s;
	}

	// The autotuner (single precision, PF_CONV_AUTO, large batches): the batch
	// built with every automatic model on the direct convolution, each block
	// shape timed; built again with them on the FFT, timed; per model, the
	// method whose fitted cost is lower (cost = seconds per unit of work,
	// crop area x PSF area for the direct convolution, M_x M_y log2(M_x M_y)
	// for the FFT, fitted to the two timings); the fastest shape; the
	// evaluation's subsampling trees split off to other warps or not, whichever
	// was faster.
	std::vector<int8_t> none(n_models, 0), all(n_models, 1);
	ConvPlan pd, pfft;
	pd.auto_fft = &none;
	pfft.auto_fft = &all;
	pfft.split = false;  // only its FFT passes are timed
	pf_batch *bd = nullptr, *bf = nullptr;
	pf_status s = create_planned(env, models, n_models, profiles, n_profiles, psf_pool, psf_pool_len, mask_pool,
	                             mask_pool_len, pd, &bd);
	if (s != PF_OK) return s;
	float *out = nullptr;
	if (cudaMalloc(&out, sizeof(float) * std::max<uint64_t>(1, bd->total_out)) != cudaSuccess) {
		pf_batch_destroy(bd);
		return fail(PF_ERR_NO_MEMORY, "pf_batch_create: autotuner output buffer");
	}
	cudaMemsetAsync(bd->d_conv, 0, sizeof(float) * std::max<size_t>(1, bd->draw_total), env->stream);
	cudaMemsetAsync(bd->d_direct, 0, sizeof(float) * std::max<size_t>(1, bd->draw_total), env->stream);
	// splitting the subsampling trees off to other warps pays where a few
	// pixels' trees would set the pass's end, and costs a little where the
	// work is spread already: the evaluation timed both ways
	bool split = bd->split.box != nullptr;
	if (fsplit >= 0) split = split && fsplit == 1;
	else if (split) {
		const double t_split = time_eval(bd, true), t_walk = time_eval(bd, false);
		split = !(t_walk > 0 && t_split > 0 && t_walk < t_split);
	}
	// every shape timed in each of two rounds, the best time of each kept:
	// a clock ramp or a slow launch early on does not decide the choice
	double t_direct = -1;
	int best_shape = bd->fwd_shape;
	std::vector<double> t_shape(pf::conv_num_shapes<float>(), -1.);
	for (int round = 0; round < 2; round++) {
		for (int sh = 0; sh < pf::conv_num_shapes<float>(); sh++) {
			const double ms = time_forward_conv(bd, sh, false, out);
			if (ms >= 0 && (t_shape[sh] < 0 || ms < t_shape[sh])) t_shape[sh] = ms;
		}
	}
	for (int sh = 0; sh < pf::conv_num_shapes<float>(); sh++) {
		if (t_shape[sh] >= 0 && (t_direct < 0 || t_shape[sh] < t_direct)) {
			t_direct = t_shape[sh];
			best_shape = sh;
		}
	}
	double work_d = 0;
	for (const auto &d : bd->mdev) {
		work_d += (double)d.crop_w * d.crop_h * (d.conv_required ? (double)d.psf_w * d.psf_h : 1.0);
	}
	std::vector<int8_t> choice(n_models, 0);
	s = create_planned(env, models, n_models, profiles, n_profiles, psf_pool, psf_pool_len, mask_pool, mask_pool_len,
	                   pfft, &bf);
	if (s == PF_OK && bf->any_fft) {
		cudaMemsetAsync(bf->d_conv, 0, sizeof(float) * std::max<size_t>(1, bf->draw_total), env->stream);
		cudaMemsetAsync(bf->d_direct, 0, sizeof(float) * std::max<size_t>(1, bf->draw_total), env->stream);
		const double t_fft = time_forward_conv(bf, 0, true, out);
		double work_f = 0;
		for (const auto &d : bf->mdev) {
			if (d.use_fft) work_f += (double)d.fft_mx * d.fft_my * std::log2((double)d.fft_mx * d.fft_my);
		}
		if (t_fft > 0 && t_direct > 0 && work_f > 0 && work_d > 0) {
			const double cf = t_fft / work_f, cd = t_direct / work_d;
			for (size_t i = 0; i < n_models; i++) {
				const pf::ModelDev &d = bf->mdev[i];
				if (!d.use_fft) continue;
				choice[i] = cf * d.fft_mx * d.fft_my * std::log2((double)d.fft_mx * d.fft_my) <
				            kFftGain * cd * (double)d.crop_w * d.crop_h * d.psf_w * d.psf_h;
			}
		}
	}
	if (bf) pf_batch_destroy(bf);
	cudaFree(out);
	pf_batch_destroy(bd);
	ConvPlan fin;
	fin.shape = best_shape;
	fin.auto_fft = &choice;
	fin.split = split;
	if (fsplit < 0) {
		tune_store(env, key, [&](TuneEntry &t) {
			t.fwd_shape = best_shape;
			t.split = split ? 1 : 0;
			t.fft = choice;
		});
	}
	s = create_planned(env, models, n_models, profiles, n_profiles, psf_pool, psf_pool_len, mask_pool, mask_pool_len,
	                   fin, batch);
	if (s == PF_OK) (*batch)->tune_key = key;
	return s;
}

pf_status pf_batch_layout(const pf_batch *b, uint64_t *offsets, uint32_t *dims, uint64_t *total_pixels)
{
	if (!b) return fail(PF_ERR_INVALID_PARAMETER, "batch is NULL");
	for (size_t i = 0; i < b->mdev.size(); i++) {
		if (offsets) offsets[i] = (uint64_t)b->mdev[i].out_off;
		if (dims) {
			dims[2 * i] = b->mdev[i].out_w;
			dims[2 * i + 1] = b->mdev[i].out_h;
		}
	}
	if (offsets) offsets[b->mdev.size()] = b->total_out;
	if (total_pixels) *total_pixels = b->total_out;
	return PF_OK;
}

pf_status pf_batch_set_params(pf_batch *b, const double *params)
{
	if (!b || !params) return fail(PF_ERR_INVALID_PARAMETER, "pf_batch_set_params: NULL argument");
	for (size_t i = 0; i < b->profiles.size(); i++) {
		pf_profile_desc d = b->profiles[i];
		std::memcpy(d.par, params + i * PF_NPAR, sizeof(d.par));
		const pf::ModelDev &m = b->mdev[b->h_profiles[i].model];
		pf_status s = validate_profile(d, m.psf_off >= 0);
		if (s != PF_OK) {
			g_last_error = "profile " + std::to_string(i) + ": " + g_last_error;
			return s;
		}
	}
	for (size_t i = 0; i < b->profiles.size(); i++) {
		std::memcpy(b->profiles[i].par, params + i * PF_NPAR, sizeof(double) * PF_NPAR);
		std::memcpy(b->h_profiles[i].par, params + i * PF_NPAR, sizeof(double) * PF_NPAR);
	}
	b->params_dirty = true;
	return PF_OK;
}

pf_status pf_batch_set_params_dev(pf_batch *b, const double *params_dev, void *stream_ptr)
{
	if (!b || !params_dev) return fail(PF_ERR_INVALID_PARAMETER, "pf_batch_set_params_dev: NULL argument");
	cudaStream_t stream = stream_ptr ? (cudaStream_t)stream_ptr : b->env->stream;
	PF_CUDA_TRY(cudaSetDevice(b->env->device));
	clear_stale_error();
	if (b->params_dirty) {
		// descriptors first, so that the device copy is complete before the scatter
		PF_CUDA_TRY(cudaMemcpyAsync(b->d_profiles, b->h_profiles,
		                            sizeof(pf::ProfileDev) * std::max<size_t>(1, b->profiles.size()),
		                            cudaMemcpyHostToDevice, stream));
		b->params_dirty = false;
	}
	pf::launch_set_params(b->d_profiles, (int)b->profiles.size(), params_dev, stream);
	b->kernel_launches++;
	PF_CUDA_TRY(cudaGetLastError());
	return PF_OK;
}

pf_status pf_batch_record_depth(pf_batch *b, int enable)
{
	if (!b) return fail(PF_ERR_INVALID_PARAMETER, "batch is NULL");
	PF_CUDA_TRY(cudaSetDevice(b->env->device));
	b->record = enable != 0;
	if (b->record && !b->d_depth) {
		PF_CUDA_TRY(cudaMalloc(&b->d_depth, std::max<size_t>(1, b->depth_total)));
		PF_CUDA_TRY(cudaMalloc(&b->d_counts, sizeof(unsigned long long) * pf::kLevelCounts *
		                                         std::max<size_t>(1, b->profiles.size())));
	}
	return PF_OK;
}

pf_status pf_forward(pf_batch *b, void *images_dev, double *flux_dev, void *stream_ptr)
{
	if (!b || (!images_dev && b->total_out)) return fail(PF_ERR_INVALID_PARAMETER, "pf_forward: NULL argument");
	cudaStream_t stream = stream_ptr ? (cudaStream_t)stream_ptr : b->env->stream;
	PF_CUDA_TRY(cudaSetDevice(b->env->device));
	clear_stale_error();
	const int n_models = (int)b->mdev.size();
	const int n_profiles = (int)b->profiles.size();
	if (n_models == 0) return PF_OK;
	if (b->params_dirty) {
		PF_CUDA_TRY(cudaMemcpyAsync(b->d_profiles, b->h_profiles, sizeof(pf::ProfileDev) * std::max(1, n_profiles),
		                            cudaMemcpyHostToDevice, stream));
		b->params_dirty = false;
	}
	pf::DebugRec dbg{nullptr, nullptr};
	if (b->count_only && !b->record) {
		PF_CUDA_TRY(cudaMemsetAsync(b->d_counts, 0, sizeof(unsigned long long) * pf::kLevelCounts *
		                                               std::max(1, n_profiles), stream));
		dbg.counts = b->d_counts;
	}
	if (b->record) {
		PF_CUDA_TRY(cudaMemsetAsync(b->d_depth, 0xff, std::max<size_t>(1, b->depth_total), stream));
		PF_CUDA_TRY(cudaMemsetAsync(b->d_counts, 0, sizeof(unsigned long long) * pf::kLevelCounts *
		                                               std::max(1, n_profiles), stream));
		dbg.depth = b->d_depth;
		dbg.counts = b->d_counts;
	}
	long t = stage_begin(b, ST_SETUP, stream);
	pf::launch_setup(b->d_models, b->d_profiles, n_profiles, n_models, b->d_counter, b->d_err, nullptr, nullptr,
	                 false, b->d_solves, b->adjoint ? 1 : 0, stream);
	stage_end(b, t, stream);
	if (b->dbl) {
		t = stage_begin(b, ST_EVAL, stream);
		pf::launch_eval64(b->d_models, n_models, b->d_profiles, b->d_psf_norm, (double *)b->d_conv,
		                  (double *)b->d_direct, b->n_tiles, b->d_counter, dbg, b->level64, b->levels64,
		                  b->env->n_sm, stream);
		stage_end(b, t, stream);
		t = stage_begin(b, ST_FINISH, stream);
		pf::launch_finish64(b->d_models, n_models, b->d_psf_norm, (const double *)b->d_conv,
		                    (const double *)b->d_direct, (double *)images_dev, (long long)b->total_out, 0,
		                    b->env->n_sm, stream);
		for (int p = 0; b->any_fft && p <= 2; p++) {
			pf::launch_fft_pass<double>(p, b->d_models, b->d_fft_jobs[p], b->fft_njobs[p], (const double *)b->d_conv,
			                            nullptr, b->d_fft_work, b->d_fft_spec, (const double *)b->d_direct,
			                            (double *)images_dev, (double *)b->d_conv, b->d_fft_tw, b->fft_nmax,
			                            b->fft_smem_bytes, stream);
		}
		if (b->any_fft_downsample) {
			// the SUM downsampling of the FFT models' fine pixels, in the reference's order
			pf::launch_finish64(b->d_models, n_models, b->d_psf_norm, (const double *)b->d_conv,
			                    (const double *)b->d_direct, (double *)images_dev, (long long)b->total_out, 1,
			                    b->env->n_sm, stream);
		}
		stage_end(b, t, stream);
	}
	else {
		t = stage_begin(b, ST_EVAL, stream);
		PF_CUDA_TRY(cudaMemsetAsync(b->d_claims, 0, sizeof(unsigned int) * (size_t)std::max<long long>(1, (b->n_tiles + 31) / 32),
		                            stream));
		pf::launch_eval32(b->d_models, n_models, b->d_profiles, n_profiles, b->d_psf_norm, (float *)b->d_conv,
		                  (float *)b->d_direct, b->n_tiles, b->d_counter, b->d_claims, dbg, b->split, b->sersic_only,
		                  b->env->n_sm, stream);
		stage_end(b, t, stream);
		t = stage_begin(b, ST_FINISH, stream);
		if (b->any_downsample) {
			PF_CUDA_TRY(cudaMemsetAsync(images_dev, 0, sizeof(float) * b->total_out, stream));
		}
		pf::launch_conv<float>(0, b->fwd_shape, b->conv_kwp, b->d_models, n_models, b->d_psf32,
		                       (const float *)b->d_conv, (const float *)b->d_direct, (float *)images_dev,
		                       b->d_tile_base_out, b->n_out_tiles, b->finish_smem, b->env->n_sm, stream);
		for (int pass = 0; b->any_fft && pass < 3; pass++) {
			for (const auto &j : b->f32_jobs[0][pass]) {
				pf::launch_fft32(pass, 0, j.n, j.d_jobs, j.n_jobs, b->d_models, (const float *)b->d_conv, nullptr,
				                 b->d_fft_work, b->d_fft_spec, (const float *)b->d_direct, (float *)images_dev,
				                 b->d_fft_tw, stream);
			}
		}
		stage_end(b, t, stream);
	}
	b->forward_calls++;
	{
		uint64_t k = (n_profiles > 0 ? 2 : 1) + 1;  // setup (solves, profiles), evaluation
		if (b->dbl) {
			k += 1 + (b->any_fft ? 3 : 0) + (b->any_fft_downsample ? 1 : 0);  // finish, FFT passes
			k += b->level64.box ? b->levels64 : 0;  // the recursion levels
		}
		else {
			k += b->split.box ? 1 : 0;  // the split boxes
			k += b->n_out_tiles > 0 ? 1 : 0;
			for (int pass = 0; b->any_fft && pass < 3; pass++) k += b->f32_jobs[0][pass].size();
		}
		b->kernel_launches += k;
	}
	if (flux_dev) {
		pf::launch_flux_sum(b->d_models, n_models, images_dev, b->dbl ? 1 : 0, flux_dev, stream);
		b->kernel_launches++;
	}
	PF_CUDA_TRY(cudaGetLastError());
	return PF_OK;
}

pf_status pf_batch_check(pf_batch *b, void *stream_ptr)
{
	if (!b) return fail(PF_ERR_INVALID_PARAMETER, "batch is NULL");
	cudaStream_t stream = stream_ptr ? (cudaStream_t)stream_ptr : b->env->stream;
	PF_CUDA_TRY(cudaSetDevice(b->env->device));
	PF_CUDA_TRY(cudaStreamSynchronize(stream));
	unsigned int errs[2] = {0, 0xffffffffu};
	PF_CUDA_TRY(cudaMemcpy(errs, b->d_err, sizeof(errs), cudaMemcpyDeviceToHost));
	const unsigned int err = errs[0];
	if (errs[1] != 0xffffffffu) {
		// parameters written on the device that the reference's validate()
		// refuses (its message); the profile drew nothing in that pass
		return fail(PF_ERR_INVALID_PARAMETER, std::string(pf::param_rule_message((int)(errs[1] & 31u))) +
		                                          " (profile " + std::to_string(errs[1] >> 5) + " of the batch)");
	}
	if (err & (pf::ERR_LEVELS | pf::ERR_RES)) {
		return fail(PF_ERR_DEVICE_LIMIT, "a profile needed more sub-pixel levels or a finer resolution than the "
		                                 "device supports; its pixels were clamped");
	}
	return PF_OK;
}

pf_status pf_batch_depth(pf_batch *b, int8_t *depth, size_t depth_len, int64_t *level_counts)
{
	if (!b) return fail(PF_ERR_INVALID_PARAMETER, "batch is NULL");
	if (!b->record) return fail(PF_ERR_INVALID_PARAMETER, "depth recording is not enabled");
	PF_CUDA_TRY(cudaSetDevice(b->env->device));
	PF_CUDA_TRY(cudaStreamSynchronize(b->env->stream));
	PF_CUDA_TRY(cudaDeviceSynchronize());
	if (depth) {
		PF_CUDA_TRY(cudaMemcpy(depth, b->d_depth, std::min(depth_len, b->depth_total), cudaMemcpyDeviceToHost));
	}
	if (level_counts) {
		std::vector<unsigned long long> tmp(pf::kLevelCounts * b->profiles.size());
		if (!tmp.empty()) {
			PF_CUDA_TRY(cudaMemcpy(tmp.data(), b->d_counts, sizeof(unsigned long long) * tmp.size(),
			                       cudaMemcpyDeviceToHost));
		}
		for (size_t i = 0; i < tmp.size(); i++) level_counts[i] = (int64_t)tmp[i];
	}
	return PF_OK;
}

pf_status pf_batch_drawing_dims(pf_batch *b, uint32_t *dims)
{
	if (!b || !dims) return fail(PF_ERR_INVALID_PARAMETER, "pf_batch_drawing_dims: NULL argument");
	for (size_t i = 0; i < b->mdev.size(); i++) {
		dims[2 * i] = b->mdev[i].draw_w;
		dims[2 * i + 1] = b->mdev[i].draw_h;
	}
	return PF_OK;
}

pf_status pf_batch_conv_info(const pf_batch *b, int32_t *forward_shape, int32_t *adjoint_shape,
                             uint32_t *fft_models)
{
	if (!b) return fail(PF_ERR_INVALID_PARAMETER, "batch is NULL");
	if (forward_shape) *forward_shape = b->fwd_shape;
	if (adjoint_shape) *adjoint_shape = b->adjoint ? b->adj_shape : -1;
	if (fft_models) {
		uint32_t n = 0;
		for (const auto &m : b->mdev) n += m.use_fft ? 1u : 0u;
		*fft_models = n;
	}
	return PF_OK;
}

pf_status pf_batch_split_info(pf_batch *b, void *stream_ptr, uint32_t *boxes, uint32_t *roots, uint32_t *pixels,
                              uint32_t *refused)
{
	if (!b) return fail(PF_ERR_INVALID_PARAMETER, "batch is NULL");
	uint32_t c[pf::kSplitCounters] = {};
	if (b->split.box) {
		cudaStream_t stream = stream_ptr ? (cudaStream_t)stream_ptr : b->env->stream;
		PF_CUDA_TRY(cudaSetDevice(b->env->device));
		PF_CUDA_TRY(cudaStreamSynchronize(stream));
		PF_CUDA_TRY(cudaMemcpy(c, b->split.cnt, sizeof(c), cudaMemcpyDeviceToHost));
		c[1] = std::min(c[1], b->split.cap_root);  // failed allocations counted past the capacity
		c[2] = std::min(c[2], b->split.cap_pix);
	}
	else if (b->level64.box) {
		cudaStream_t stream = stream_ptr ? (cudaStream_t)stream_ptr : b->env->stream;
		PF_CUDA_TRY(cudaSetDevice(b->env->device));
		PF_CUDA_TRY(cudaStreamSynchronize(stream));
		uint32_t l[pf::kSplitCounters] = {};
		PF_CUDA_TRY(cudaMemcpy(l, b->level64.cnt, sizeof(l), cudaMemcpyDeviceToHost));
		c[0] = std::min(l[pf::LC_BOX], b->level64.cap_box);
		c[1] = std::min(l[pf::LC_ROOT], b->level64.cap_root);
		c[2] = std::min(l[pf::LC_PIX], b->level64.cap_pix);
		c[4] = l[pf::LC_REFUSED];
	}
	if (boxes) *boxes = c[0];
	if (roots) *roots = c[1];
	if (pixels) *pixels = c[2];
	if (refused) *refused = c[4];
	return PF_OK;
}

pf_status pf_batch_enable_adjoint(pf_batch *b)
{
	if (!b) return fail(PF_ERR_INVALID_PARAMETER, "batch is NULL");
	if (b->adjoint) return PF_OK;
	for (size_t i = 0; i < b->profiles.size(); i++) {
		const pf_profile_desc &d = b->profiles[i];
		const bool ok = (d.kind >= PF_SERSIC && d.kind <= PF_BROKENEXP) || d.kind == PF_SKY || d.kind == PF_PSF ||
		                d.kind == PF_NULL;
		if (!ok) {
			return fail(PF_ERR_UNSUPPORTED, "profile " + std::to_string(i) + ": no adjoint for this profile kind");
		}
	}
	for (size_t i = 0; i < b->mdev.size(); i++) {
		if (b->mdev[i].uncropped) {
			return fail(PF_ERR_UNSUPPORTED, "model " + std::to_string(i) + ": no adjoint of the FFT convolver's "
			                                "uncropped image (crop = false)");
		}
	}
	PF_CUDA_TRY(cudaSetDevice(b->env->device));
	const size_t elem = b->dbl ? sizeof(double) : sizeof(float);
	const size_t n_models = b->mdev.size();
	std::vector<long long> adj_tile_base(std::max<size_t>(1, n_models));
	std::vector<long long> prow_base(std::max<size_t>(1, b->profiles.size()), 0);
	long long rows = 0, tiles = 0;
	unsigned int max_h = 1;
	unsigned int max_kw = 1, max_kh = 1;
	std::vector<std::pair<unsigned int, unsigned int>> conv_dims;
	for (const auto &m : b->mdev) {
		if (m.conv_required && (b->dbl || !m.use_fft)) conv_dims.push_back({m.draw_w, m.draw_h});
	}
	b->adj_shape = b->dbl ? best_conv_shape<double>(conv_dims) : best_conv_shape<float>(conv_dims);
	if (!b->dbl && forced_conv_shape() >= 0) b->adj_shape = forced_conv_shape();
	for (const auto &m : b->mdev) {
		if (m.conv_required && (b->dbl || !m.use_fft)) {
			max_kw = std::max(max_kw, m.psf_w);
			max_kh = std::max(max_kh, m.psf_h);
		}
	}
	if (!b->dbl && pf::conv_smem<float>(max_kw, max_kh, b->adj_shape) > 227 * 1024 && forced_conv_shape() < 0) {
		// the chosen block shape's patch too large for this PSF: the first one that fits
		for (int sh = 0; sh < pf::conv_num_shapes<float>(); sh++) {
			if (pf::conv_smem<float>(max_kw, max_kh, sh) <= 227 * 1024) {
				b->adj_shape = sh;
				break;
			}
		}
	}
	for (size_t i = 0; i < n_models; i++) {
		const pf::ModelDev &m = b->mdev[i];
		for (int q = 0; q < m.n_profiles; q++) {
			prow_base[m.first_profile + q] = rows;
			rows += m.draw_h;
		}
		max_h = std::max(max_h, m.draw_h);
		adj_tile_base[i] = tiles;
		if (m.conv_required && (b->dbl || !m.use_fft)) {
			tiles += b->dbl ? pf::conv_tiles<double>(m.draw_w, m.draw_h, b->adj_shape)
			                : pf::conv_tiles<float>(m.draw_w, m.draw_h, b->adj_shape);
		}
	}
	if (pf::backward_items((long long)std::max<size_t>(1, b->profiles.size()), 2ll * max_h) >= (1ll << 31)) {
		return fail(PF_ERR_UNSUPPORTED, "too many profile rows for the adjoint's work counter");
	}
	b->n_ring = 2 * max_h;
	b->n_adj_tiles = tiles;
	b->adj_smem = b->dbl ? pf::conv_smem<double>(max_kw, max_kh, b->adj_shape)
	                     : pf::conv_smem<float>(max_kw, max_kh, b->adj_shape);
	if (b->adj_smem > 227 * 1024) return fail(PF_ERR_UNSUPPORTED, "PSF too large for the adjoint convolution");
	PF_CUDA_TRY(cudaMalloc(&b->d_gout, elem * std::max<uint64_t>(1, b->total_out)));
	uint64_t max_out = 1;
	for (const auto &m : b->mdev) max_out = std::max<uint64_t>(max_out, (uint64_t)m.out_w * m.out_h);
	b->chi2_parts = (int)std::min<uint64_t>(128, (max_out + 65535) / 65536);
	PF_CUDA_TRY(cudaMalloc(&b->d_chi2_partial, sizeof(double) * b->chi2_parts * std::max<size_t>(1, n_models)));
	PF_CUDA_TRY(cudaMalloc(&b->d_chi2_done, sizeof(unsigned int) * std::max<size_t>(1, n_models)));
	PF_CUDA_TRY(cudaMemset(b->d_chi2_done, 0, sizeof(unsigned int) * std::max<size_t>(1, n_models)));
	PF_CUDA_TRY(cudaMalloc(&b->d_gsrc, elem * std::max<size_t>(1, b->draw_total)));
	PF_CUDA_TRY(cudaMalloc(&b->d_partial, sizeof(double) * pf::backward_slots(b->sersic_only) *
	                                          std::max<long long>(1, rows)));
	PF_CUDA_TRY(cudaMalloc(&b->d_ring_partial, sizeof(double) * pf::backward_ring_slots(b->sersic_only) *
	                                               std::max<size_t>(1, b->profiles.size())));
	PF_CUDA_TRY(cudaMalloc(&b->d_prow_base, sizeof(long long) * prow_base.size()));
	PF_CUDA_TRY(cudaMalloc(&b->d_bwd_counter, 2 * sizeof(unsigned int)));
	PF_CUDA_TRY(cudaMalloc(&b->d_adj_tile_base, sizeof(long long) * adj_tile_base.size()));
	PF_CUDA_TRY(cudaMemcpy(b->d_prow_base, prow_base.data(), sizeof(long long) * prow_base.size(), cudaMemcpyHostToDevice));
	PF_CUDA_TRY(cudaMemcpy(b->d_adj_tile_base, adj_tile_base.data(), sizeof(long long) * adj_tile_base.size(),
	                       cudaMemcpyHostToDevice));
	PF_CUDA_TRY(b->dbl ? pf::conv_configure<double>(b->adj_smem, b->adj_shape, 0)
	                   : pf::conv_configure<float>(b->adj_smem, b->adj_shape, b->conv_kwp));
	if (!b->dbl && !(b->env->flags & PF_ENV_NO_AUTOTUNE) && b->total_out >= (1ull << 22) && tiles > 0 &&
	    forced_conv_shape() < 0) {
		// the autotuner, adjoint convolution: each block shape timed over the
		// batch's directly convolved models (zero cotangents), the fastest kept;
		// or the shape this layout was given before
		int best_shape = b->adj_shape;
		TuneEntry known;
		if (b->tune_key && tune_lookup(b->env, b->tune_key, &known) && known.adj_shape >= 0 &&
		    known.adj_shape < pf::conv_num_shapes<float>()) {
			best_shape = known.adj_shape;
			std::lock_guard<std::mutex> lock(b->env->tune.mu);
			b->env->tune.reused++;
		}
		else {
			PF_CUDA_TRY(cudaMemsetAsync(b->d_gout, 0, sizeof(float) * std::max<uint64_t>(1, b->total_out),
			                            b->env->stream));
			double best = -1;
			std::vector<double> t_shape(pf::conv_num_shapes<float>(), -1.);
			for (int round = 0; round < 2; round++) {  // as for the forward shapes
				for (int sh = 0; sh < pf::conv_num_shapes<float>(); sh++) {
					const double ms = time_adjoint_conv(b, sh);
					if (ms >= 0 && (t_shape[sh] < 0 || ms < t_shape[sh])) t_shape[sh] = ms;
				}
			}
			for (int sh = 0; sh < pf::conv_num_shapes<float>(); sh++) {
				if (t_shape[sh] >= 0 && (best < 0 || t_shape[sh] < best)) {
					best = t_shape[sh];
					best_shape = sh;
				}
			}
			if (b->tune_key) tune_store(b->env, b->tune_key, [&](TuneEntry &t) { t.adj_shape = best_shape; });
		}
		if (best_shape != b->adj_shape) {
			long long t = 0;
			for (size_t i = 0; i < n_models; i++) {
				const pf::ModelDev &m = b->mdev[i];
				adj_tile_base[i] = t;
				if (m.conv_required && !m.use_fft) t += pf::conv_tiles<float>(m.draw_w, m.draw_h, best_shape);
			}
			b->adj_shape = best_shape;
			b->n_adj_tiles = t;
			b->adj_smem = pf::conv_smem<float>(max_kw, max_kh, best_shape);
			PF_CUDA_TRY(cudaMemcpy(b->d_adj_tile_base, adj_tile_base.data(), sizeof(long long) * adj_tile_base.size(),
			                       cudaMemcpyHostToDevice));
		}
		PF_CUDA_TRY(pf::conv_configure<float>(b->adj_smem, b->adj_shape, b->conv_kwp));
	}
	b->adjoint = true;
	return PF_OK;
}

pf_status pf_backward(pf_batch *b, const void *images_dev, const void *data_dev, const void *sigma_dev,
                      const void *cotangent_dev, double *chi2_dev, double *grad_dev, void *stream_ptr)
{
	if (!b) return fail(PF_ERR_INVALID_PARAMETER, "batch is NULL");
	if (!b->adjoint) return fail(PF_ERR_INVALID_PARAMETER, "pf_batch_enable_adjoint has not been called");
	if (!grad_dev || (!cotangent_dev && (!images_dev || !data_dev))) {
		return fail(PF_ERR_INVALID_PARAMETER, "pf_backward: NULL argument");
	}
	cudaStream_t stream = stream_ptr ? (cudaStream_t)stream_ptr : b->env->stream;
	PF_CUDA_TRY(cudaSetDevice(b->env->device));
	clear_stale_error();
	const int n_models = (int)b->mdev.size(), n_profiles = (int)b->profiles.size();
	if (n_models == 0) return PF_OK;
	bool any_conv = false;
	for (const auto &m : b->mdev) any_conv |= m.conv_required != 0;
	long t = stage_begin(b, ST_CHI2, stream);
	if (b->dbl) pf::launch_chi2<double>(b->d_models, n_models, images_dev, data_dev, sigma_dev, cotangent_dev,
	                                    b->d_gout, chi2_dev, b->chi2_parts, b->d_chi2_partial, b->d_chi2_done,
	                                    stream);
	else pf::launch_chi2<float>(b->d_models, n_models, images_dev, data_dev, sigma_dev, cotangent_dev, b->d_gout,
	                            chi2_dev, b->chi2_parts, b->d_chi2_partial, b->d_chi2_done, stream);
	stage_end(b, t, stream);
	if (any_conv) {
		t = stage_begin(b, ST_ADJCONV, stream);
		if (b->dbl) pf::launch_conv<double>(1, b->adj_shape, 0, b->d_models, n_models, b->d_psf_norm,
		                                    (const double *)b->d_gout, nullptr, (double *)b->d_gsrc,
		                                    b->d_adj_tile_base, b->n_adj_tiles, b->adj_smem, b->env->n_sm, stream);
		else {
			if (b->n_adj_tiles > 0) {
				pf::launch_conv<float>(1, b->adj_shape, b->conv_kwp, b->d_models, n_models, b->d_psf32,
				                       (const float *)b->d_gout, nullptr, (float *)b->d_gsrc, b->d_adj_tile_base,
				                       b->n_adj_tiles, b->adj_smem, b->env->n_sm, stream);
			}
			for (int pass = 0; b->any_fft && pass < 3; pass++) {
				for (const auto &j : b->f32_jobs[1][pass]) {
					pf::launch_fft32(pass, 1, j.n, j.d_jobs, j.n_jobs, b->d_models, (const float *)b->d_gout, nullptr,
					                 b->d_fft_work, b->d_fft_spec, nullptr, (float *)b->d_gsrc, b->d_fft_tw, stream);
				}
			}
		}
		stage_end(b, t, stream);
	}
	t = stage_begin(b, ST_BACKWARD, stream);
	PF_CUDA_TRY(cudaMemsetAsync(b->d_bwd_counter, 0, 2 * sizeof(unsigned int), stream));
	if (b->dbl) pf::launch_backward<double>(b->d_models, b->d_profiles, n_profiles, b->d_gout, b->d_gsrc,
	                                        b->d_psf_norm, b->d_prow_base, b->n_ring, b->d_bwd_counter, b->d_partial,
	                                        b->d_ring_partial, grad_dev, b->sersic_only, b->env->n_sm, stream);
	else pf::launch_backward<float>(b->d_models, b->d_profiles, n_profiles, b->d_gout, b->d_gsrc, b->d_psf_norm,
	                                b->d_prow_base, b->n_ring, b->d_bwd_counter, b->d_partial, b->d_ring_partial,
	                                grad_dev, b->sersic_only, b->env->n_sm, stream);
	stage_end(b, t, stream);
	b->backward_calls++;
	{
		uint64_t k = 1 + (n_profiles > 0 ? 2 : 0);  // chi^2, backward, gradient reduction
		if (any_conv) {
			if (b->dbl) k += 1;
			else {
				k += b->n_adj_tiles > 0 ? 1 : 0;
				for (int pass = 0; b->any_fft && pass < 3; pass++) k += b->f32_jobs[1][pass].size();
			}
		}
		b->kernel_launches += k;
	}
	PF_CUDA_TRY(cudaGetLastError());
	return PF_OK;
}

pf_status pf_batch_stats(pf_batch *b, pf_stage_times *times, int reset)
{
	if (!b || !times) return fail(PF_ERR_INVALID_PARAMETER, "pf_batch_stats: NULL argument");
	PF_CUDA_TRY(cudaSetDevice(b->env->device));
	fold_stage_times(b);
	times->setup_ms = b->stage_ms[ST_SETUP];
	times->eval_ms = b->stage_ms[ST_EVAL];
	times->finish_ms = b->stage_ms[ST_FINISH];
	times->chi2_ms = b->stage_ms[ST_CHI2];
	times->adjoint_conv_ms = b->stage_ms[ST_ADJCONV];
	times->backward_ms = b->stage_ms[ST_BACKWARD];
	times->forward_calls = b->forward_calls;
	times->backward_calls = b->backward_calls;
	times->kernel_launches = b->kernel_launches;
	if (reset) {
		for (double &v : b->stage_ms) v = 0;
		b->forward_calls = b->backward_calls = 0;
		b->kernel_launches = 0;
	}
	return PF_OK;
}

pf_status pf_forward_backward(pf_batch *b, void *images_dev, const void *data_dev, const void *sigma_dev,
                              double *chi2_dev, double *grad_dev, void *stream)
{
	pf_status s = pf_forward(b, images_dev, nullptr, stream);
	if (s != PF_OK) return s;
	return pf_backward(b, images_dev, data_dev, sigma_dev, nullptr, chi2_dev, grad_dev, stream);
}

pf_status pf_step_graph(pf_batch *b, const double *params_dev, void *images_dev, const void *data_dev,
                        const void *sigma_dev, double *chi2_dev, double *grad_dev, void *stream_ptr)
{
	if (!b) return fail(PF_ERR_INVALID_PARAMETER, "batch is NULL");
	if (!b->adjoint) return fail(PF_ERR_INVALID_PARAMETER, "pf_batch_enable_adjoint has not been called");
	if (!images_dev || !data_dev || !grad_dev) return fail(PF_ERR_INVALID_PARAMETER, "pf_step_graph: NULL argument");
	cudaStream_t stream = stream_ptr ? (cudaStream_t)stream_ptr : b->env->stream;
	if (stream == cudaStreamLegacy || stream == cudaStreamPerThread) {
		return fail(PF_ERR_INVALID_PARAMETER, "pf_step_graph: a graph is captured on a created stream, not the default one");
	}
	PF_CUDA_TRY(cudaSetDevice(b->env->device));
	clear_stale_error();
	// parameters set on the host since the last step go up outside the graph
	if (b->params_dirty) {
		PF_CUDA_TRY(cudaMemcpyAsync(b->d_profiles, b->h_profiles,
		                            sizeof(pf::ProfileDev) * std::max<size_t>(1, b->profiles.size()),
		                            cudaMemcpyHostToDevice, stream));
		b->params_dirty = false;
	}
	pf_batch::GraphKey key;
	key.params = params_dev;
	key.images = images_dev;
	key.data = data_dev;
	key.sigma = sigma_dev;
	key.chi2 = chi2_dev;
	key.grad = grad_dev;
	key.stream = stream;
	key.record = b->record;
	bool captured = false;
	if (!b->graph || !(key == b->graph_key)) {
		if (b->graph) {
			cudaGraphExecDestroy(b->graph);
			b->graph = nullptr;
		}
		PF_CUDA_TRY(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
		b->capturing = true;
		const uint64_t k0 = b->kernel_launches;
		pf_status s = PF_OK;
		if (params_dev) s = pf_batch_set_params_dev(b, params_dev, stream);
		if (s == PF_OK) s = pf_forward(b, images_dev, nullptr, stream);
		if (s == PF_OK) s = pf_backward(b, images_dev, data_dev, sigma_dev, nullptr, chi2_dev, grad_dev, stream);
		b->capturing = false;
		cudaGraph_t g = nullptr;
		const cudaError_t e = cudaStreamEndCapture(stream, &g);
		if (s != PF_OK) {
			if (g) cudaGraphDestroy(g);
			return s;
		}
		if (e != cudaSuccess) return fail(PF_ERR_CUDA, std::string("pf_step_graph: capture: ") + cudaGetErrorString(e));
		const cudaError_t ei = cudaGraphInstantiate(&b->graph, g, 0);
		cudaGraphDestroy(g);
		if (ei != cudaSuccess) {
			b->graph = nullptr;
			return fail(PF_ERR_CUDA, std::string("pf_step_graph: instantiate: ") + cudaGetErrorString(ei));
		}
		b->graph_key = key;
		b->graph_kernels = b->kernel_launches - k0;
		captured = true;
	}
	PF_CUDA_TRY(cudaGraphLaunch(b->graph, stream));
	if (!captured) {  // the capture counted the first call
		b->forward_calls++;
		b->backward_calls++;
		b->kernel_launches += b->graph_kernels;
	}
	return PF_OK;
}

pf_status pf_model_evaluate(pf_env *env, const pf_model_desc *model, const pf_profile_desc *profiles,
                            const double *psf, double *image, uint32_t *out_w, uint32_t *out_h)
{
	return pf_model_evaluate_masked(env, model, profiles, psf, nullptr, image, out_w, out_h);
}

pf_status pf_model_evaluate_masked(pf_env *env, const pf_model_desc *model, const pf_profile_desc *profiles,
                                   const double *psf, const uint8_t *mask, double *image, uint32_t *out_w,
                                   uint32_t *out_h)
{
	if (!env || !model || !image || (!profiles && model->n_profiles)) {
		return fail(PF_ERR_INVALID_PARAMETER, "pf_model_evaluate: NULL argument");
	}
	pf_model_desc m = *model;
	m.first_profile = 0;
	const bool has_psf = psf && m.psf_w > 0 && m.psf_h > 0;
	m.psf_offset = has_psf ? 0 : -1;
	m.mask_offset = mask ? 0 : -1;
	const size_t psf_len = has_psf ? (size_t)m.psf_w * m.psf_h : 0;
	const size_t mask_len = mask ? (size_t)m.mask_w * m.mask_h : 0;
	PF_CUDA_TRY(cudaSetDevice(env->device));
	pf_env::Cache &c = env->cache;
	std::lock_guard<std::mutex> lock(c.mu);
	// The batch of the previous call is reused when the model differs from it
	// in parameter values only (Model::evaluate in a fitting loop): its
	// constants are recomputed on the device from the new values, nothing is
	// allocated.
	bool hit = c.batch && same_model(c.model, m) && c.profiles.size() == m.n_profiles &&
	           c.psf.size() == psf_len && (!psf_len || std::memcmp(c.psf.data(), psf, sizeof(double) * psf_len) == 0) &&
	           c.has_mask == (mask != nullptr) && c.mask.size() == mask_len &&
	           (!mask_len || std::memcmp(c.mask.data(), mask, mask_len) == 0);
	for (uint32_t i = 0; hit && i < m.n_profiles; i++) hit = same_profile_layout(c.profiles[i], profiles[i]);
	pf_status s = PF_OK;
	if (hit) {
		// the reference's validate() of each profile, as a new batch would run it
		for (uint32_t i = 0; i < m.n_profiles; i++) {
			s = validate_profile(profiles[i], has_psf);
			if (s != PF_OK) return s;
		}
		c.params.resize((size_t)m.n_profiles * PF_NPAR);
		for (uint32_t i = 0; i < m.n_profiles; i++) {
			std::memcpy(&c.params[(size_t)i * PF_NPAR], profiles[i].par, sizeof(double) * PF_NPAR);
		}
		s = pf_batch_set_params(c.batch, c.params.data());
		if (s != PF_OK) return s;
	}
	else {
		if (c.batch) pf_batch_destroy(c.batch);
		c.batch = nullptr;
		s = pf_batch_create_masked(env, &m, 1, profiles, m.n_profiles, has_psf ? psf : nullptr, psf_len, mask,
		                           mask_len, &c.batch);
		if (s != PF_OK) return s;
		if (env->flags & PF_ENV_PROFILE) {
			// Model::get_stats: the profiling environment counts each profile's
			// subsample_pixel calls and evaluations (pf_env_last_model_stats)
			c.batch->count_only = true;
			const cudaError_t e = cudaMalloc(&c.batch->d_counts, sizeof(unsigned long long) * pf::kLevelCounts *
			                                                          std::max<size_t>(1, m.n_profiles));
			if (e != cudaSuccess) return fail(PF_ERR_NO_MEMORY, std::string("pf_model_evaluate: ") + cudaGetErrorString(e));
		}
		c.model = m;
		c.profiles.assign(profiles, profiles + m.n_profiles);
		c.psf.assign(psf, psf + psf_len);
		c.has_mask = mask != nullptr;
		c.mask.assign(mask, mask + mask_len);
	}
	pf_batch *b = c.batch;
	const size_t n = b->total_out;
	const size_t elem = b->dbl ? sizeof(double) : sizeof(float);
	if (c.out_bytes < elem * std::max<size_t>(1, n)) {
		cudaFree(c.d_out);
		c.d_out = nullptr;
		c.out_bytes = 0;
		const cudaError_t e = cudaMalloc(&c.d_out, elem * std::max<size_t>(1, n));
		if (e != cudaSuccess) return fail(PF_ERR_NO_MEMORY, std::string("pf_model_evaluate: ") + cudaGetErrorString(e));
		c.out_bytes = elem * std::max<size_t>(1, n);
	}
	s = pf_forward(b, c.d_out, nullptr, nullptr);
	if (s == PF_OK) s = pf_batch_check(b, nullptr);
	if (s != PF_OK) return s;
	cudaError_t e;
	if (b->dbl) {
		e = cudaMemcpyAsync(image, c.d_out, sizeof(double) * n, cudaMemcpyDeviceToHost, env->stream);
		if (e == cudaSuccess) e = cudaStreamSynchronize(env->stream);
	}
	else {
		c.host32.resize(n);
		e = cudaMemcpyAsync(c.host32.data(), c.d_out, sizeof(float) * n, cudaMemcpyDeviceToHost, env->stream);
		if (e == cudaSuccess) e = cudaStreamSynchronize(env->stream);
		for (size_t i = 0; e == cudaSuccess && i < n; i++) image[i] = c.host32[i];
	}
	if (e != cudaSuccess) return fail(PF_ERR_CUDA, std::string("pf_model_evaluate: ") + cudaGetErrorString(e));
	if (out_w) *out_w = b->mdev[0].out_w;
	if (out_h) *out_h = b->mdev[0].out_h;
	if (env->flags & PF_ENV_PROFILE) {
		s = pf_batch_stats(b, &c.last_times, 1);
		if (s != PF_OK) return s;
		c.last_counts.assign((size_t)pf::kLevelCounts * m.n_profiles, 0);
		if (m.n_profiles && b->d_counts) {
			e = cudaMemcpy(c.last_counts.data(), b->d_counts, sizeof(unsigned long long) * c.last_counts.size(),
			               cudaMemcpyDeviceToHost);
			if (e != cudaSuccess) return fail(PF_ERR_CUDA, std::string("pf_model_evaluate: ") + cudaGetErrorString(e));
		}
	}
	return PF_OK;
}

pf_status pf_env_last_model_stats(pf_env *env, pf_stage_times *times, int64_t *level_counts, size_t n_profiles)
{
	if (!env) return fail(PF_ERR_INVALID_PARAMETER, "env is NULL");
	pf_env::Cache &c = env->cache;
	std::lock_guard<std::mutex> lock(c.mu);
	if (times) *times = c.last_times;
	if (level_counts) {
		const size_t have = c.last_counts.size() / pf::kLevelCounts;
		for (size_t i = 0; i < n_profiles * pf::kLevelCounts; i++) {
			level_counts[i] = i / pf::kLevelCounts < have ? (int64_t)c.last_counts[i] : 0;
		}
	}
	return PF_OK;
}

pf_status pf_convolve(pf_env *env, const double *src, uint32_t w, uint32_t h, const double *krn, uint32_t kw,
                      uint32_t kh, const uint8_t *mask, double *out)
{
	return pf_convolve_crop(env, src, w, h, krn, kw, kh, mask, 1, out, nullptr, nullptr);
}

pf_status pf_convolve_crop(pf_env *env, const double *src, uint32_t w, uint32_t h, const double *krn, uint32_t kw,
                           uint32_t kh, const uint8_t *mask, int crop, double *out, uint32_t *offset_x,
                           uint32_t *offset_y)
{
	if (!env || !src || !krn || !out) return fail(PF_ERR_INVALID_PARAMETER, "pf_convolve: NULL argument");
	if (w == 0 || h == 0 || kw == 0 || kh == 0) return fail(PF_ERR_INVALID_PARAMETER, "pf_convolve: empty image");
	PF_CUDA_TRY(cudaSetDevice(env->device));
	clear_stale_error();
	// Convolver::convolve: an image smaller than the kernel is first extended
	// to max(src, krn), whose y component repeats the x maximum
	// (include/profit/image.h:204-207), and the result cropped back.
	uint32_t ew = w, eh = h;
	if (!(w >= kw && h >= kh)) {
		ew = std::max(w, kw);
		eh = ew;
	}
	// Surface::extend refuses a smaller height (include/profit/image.h:305-311)
	if (eh < h) return fail(PF_ERR_INVALID_PARAMETER, "pf_convolve: new_height should be >= height");
	// crop = false: a direct convolver adds no padding (Convolver::padding is
	// empty, src/convolve.cpp:50-53), so the image is the cropped one and its
	// offset (0, 0) (mask_and_crop, src/convolve.cpp:81-99)
	(void)crop;
	if (offset_x) *offset_x = 0;
	if (offset_y) *offset_y = 0;
	const size_t n = (size_t)ew * eh, kn = (size_t)kw * kh;
	// the environment's scratch (grown when too small, else reused): source,
	// output, kernel, mask, each on a 256-byte boundary
	auto up = [](size_t b) { return (b + 255) & ~(size_t)255; };
	const size_t o_out = up(sizeof(double) * n), o_krn = o_out + up(sizeof(double) * n);
	const size_t o_mask = o_krn + up(sizeof(double) * kn), bytes = o_mask + up(mask ? n : 1);
	pf_env::Cache &c = env->cache;
	std::lock_guard<std::mutex> lock(c.mu);
	if (c.conv_bytes < bytes) {
		cudaFree(c.d_conv);
		c.d_conv = nullptr;
		c.conv_bytes = 0;
		const cudaError_t e = cudaMalloc(&c.d_conv, bytes);
		if (e != cudaSuccess) return fail(PF_ERR_NO_MEMORY, std::string("pf_convolve: ") + cudaGetErrorString(e));
		c.conv_bytes = bytes;
	}
	unsigned char *base = static_cast<unsigned char *>(c.d_conv);
	double *d_src = reinterpret_cast<double *>(base), *d_out = reinterpret_cast<double *>(base + o_out);
	double *d_krn = reinterpret_cast<double *>(base + o_krn);
	uint8_t *d_mask = mask ? base + o_mask : nullptr;
	cudaStream_t st = env->stream;
	const bool extended = ew != w || eh != h;
	const size_t row = sizeof(double) * w, erow = sizeof(double) * ew;
	cudaError_t e = cudaSuccess;
	if (extended) {
		// zero extension, the original at the top left (Surface::extend, start 0)
		e = cudaMemsetAsync(d_src, 0, sizeof(double) * n, st);
		if (e == cudaSuccess) e = cudaMemcpy2DAsync(d_src, erow, src, row, row, h, cudaMemcpyHostToDevice, st);
		if (e == cudaSuccess && mask) e = cudaMemsetAsync(d_mask, 0, n, st);
		if (e == cudaSuccess && mask) e = cudaMemcpy2DAsync(d_mask, ew, mask, w, w, h, cudaMemcpyHostToDevice, st);
	}
	else {
		e = cudaMemcpyAsync(d_src, src, sizeof(double) * n, cudaMemcpyHostToDevice, st);
		if (e == cudaSuccess && mask) e = cudaMemcpyAsync(d_mask, mask, n, cudaMemcpyHostToDevice, st);
	}
	if (e == cudaSuccess) e = cudaMemcpyAsync(d_krn, krn, sizeof(double) * kn, cudaMemcpyHostToDevice, st);
	if (e == cudaSuccess) {
		pf::launch_convolve64(d_src, ew, eh, d_krn, kw, kh, d_mask, d_out, env->n_sm, st);
		e = cudaGetLastError();
	}
	// cropped back to the original size (result.crop(dims - diff), top-left aligned)
	if (e == cudaSuccess) {
		e = extended ? cudaMemcpy2DAsync(out, row, d_out, erow, row, h, cudaMemcpyDeviceToHost, st)
		             : cudaMemcpyAsync(out, d_out, sizeof(double) * n, cudaMemcpyDeviceToHost, st);
	}
	const cudaError_t sync = cudaStreamSynchronize(st);
	if (e == cudaSuccess) e = sync;
	if (e != cudaSuccess) return fail(PF_ERR_CUDA, std::string("pf_convolve: ") + cudaGetErrorString(e));
	return PF_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// pf_convolve_noalloc: pf_convolve with its device buffers in static device
// data, for callers that must not allocate (see include/pf_cuda.h).

namespace {

// Layout of the scratch: source image, output image, kernel, mask; each part
// starts on a 256-byte boundary.
constexpr size_t kNaSrcOff = 0;
constexpr size_t kNaOutOff = kNaSrcOff + sizeof(double) * PF_NOALLOC_MAX_PIXELS;
constexpr size_t kNaKrnOff = kNaOutOff + sizeof(double) * PF_NOALLOC_MAX_PIXELS;
constexpr size_t kNaMaskOff = kNaKrnOff + sizeof(double) * PF_NOALLOC_MAX_KERNEL_PIXELS;
constexpr size_t kNaBytes = kNaMaskOff + PF_NOALLOC_MAX_PIXELS;
static_assert(kNaOutOff % 256 == 0 && kNaKrnOff % 256 == 0 && kNaMaskOff % 256 == 0 && kNaBytes % 256 == 0,
              "scratch parts must start on 256-byte boundaries");

// Reserved with the module on each device, never by a call.
static __device__ __align__(256) unsigned char g_convolve_scratch[kNaBytes];

constexpr int kNaMaxDevices = 64;
std::mutex g_convolve_scratch_mutex;
unsigned char *g_convolve_scratch_addr[kNaMaxDevices] = {};

// Address of g_convolve_scratch on `device`, which must be the current device.
// Looked up on the first call for a device, then read from the table.
pf_status convolve_scratch(int device, unsigned char **addr)
{
	if (device < 0 || device >= kNaMaxDevices) {
		return fail(PF_ERR_DEVICE_LIMIT, "pf_convolve_noalloc: device ordinal beyond the scratch address table");
	}
	std::lock_guard<std::mutex> lock(g_convolve_scratch_mutex);
	if (!g_convolve_scratch_addr[device]) {
		void *p = nullptr;
		cudaError_t e = cudaGetSymbolAddress(&p, g_convolve_scratch);
		if (e != cudaSuccess) {
			return fail(PF_ERR_CUDA, std::string("pf_convolve_noalloc: cudaGetSymbolAddress: ") + cudaGetErrorString(e));
		}
		g_convolve_scratch_addr[device] = static_cast<unsigned char *>(p);
	}
	*addr = g_convolve_scratch_addr[device];
	return PF_OK;
}

}  // namespace

extern "C" {

pf_status pf_convolve_noalloc(pf_env *env, const double *src, uint32_t w, uint32_t h, const double *krn, uint32_t kw,
                              uint32_t kh, const uint8_t *mask, double *out)
{
	if (!env || !src || !krn || !out) return fail(PF_ERR_INVALID_PARAMETER, "pf_convolve_noalloc: NULL argument");
	if (w == 0 || h == 0 || kw == 0 || kh == 0) {
		return fail(PF_ERR_INVALID_PARAMETER, "pf_convolve_noalloc: empty image");
	}
	// the extension of pf_convolve (Convolver::convolve, src/convolve.cpp:63-74)
	uint32_t ew = w, eh = h;
	if (!(w >= kw && h >= kh)) {
		ew = std::max(w, kw);
		eh = ew;
	}
	if (eh < h) return fail(PF_ERR_INVALID_PARAMETER, "pf_convolve_noalloc: new_height should be >= height");
	const size_t n = (size_t)ew * eh, kn = (size_t)kw * kh;
	if (n > PF_NOALLOC_MAX_PIXELS) {
		return fail(PF_ERR_DEVICE_LIMIT, "pf_convolve_noalloc: image of " + std::to_string(n) +
		                                     " pixels (after extension to the kernel's size) exceeds the static "
		                                     "scratch's " + std::to_string(PF_NOALLOC_MAX_PIXELS) +
		                                     "; use pf_convolve");
	}
	if (kn > PF_NOALLOC_MAX_KERNEL_PIXELS) {
		return fail(PF_ERR_DEVICE_LIMIT, "pf_convolve_noalloc: kernel of " + std::to_string(kn) +
		                                     " pixels exceeds the static scratch's " +
		                                     std::to_string(PF_NOALLOC_MAX_KERNEL_PIXELS) + "; use pf_convolve");
	}
	PF_CUDA_TRY(cudaSetDevice(env->device));
	// an earlier failed runtime call of the process (a cudaMalloc that found the
	// device full) leaves its error for cudaGetLastError: cleared here, so that
	// the check after the launch below reports this call's launch only
	(void)cudaGetLastError();
	unsigned char *base = nullptr;
	pf_status s = convolve_scratch(env->device, &base);
	if (s != PF_OK) return s;
	double *d_src = reinterpret_cast<double *>(base + kNaSrcOff);
	double *d_out = reinterpret_cast<double *>(base + kNaOutOff);
	double *d_krn = reinterpret_cast<double *>(base + kNaKrnOff);
	uint8_t *d_mask = mask ? base + kNaMaskOff : nullptr;
	cudaStream_t st = env->stream;
	const bool extended = ew != w || eh != h;
	const size_t row = sizeof(double) * w, erow = sizeof(double) * ew;
	cudaError_t e = cudaSuccess;
	if (extended) {
		// zero extension, the original at the top left (Surface::extend, start 0)
		e = cudaMemsetAsync(d_src, 0, sizeof(double) * n, st);
		if (e == cudaSuccess) e = cudaMemcpy2DAsync(d_src, erow, src, row, row, h, cudaMemcpyHostToDevice, st);
		if (e == cudaSuccess && mask) e = cudaMemsetAsync(d_mask, 0, n, st);
		if (e == cudaSuccess && mask) e = cudaMemcpy2DAsync(d_mask, ew, mask, w, w, h, cudaMemcpyHostToDevice, st);
	}
	else {
		e = cudaMemcpyAsync(d_src, src, sizeof(double) * n, cudaMemcpyHostToDevice, st);
		if (e == cudaSuccess && mask) e = cudaMemcpyAsync(d_mask, mask, n, cudaMemcpyHostToDevice, st);
	}
	if (e == cudaSuccess) e = cudaMemcpyAsync(d_krn, krn, sizeof(double) * kn, cudaMemcpyHostToDevice, st);
	if (e == cudaSuccess) {
		pf::launch_convolve64(d_src, ew, eh, d_krn, kw, kh, d_mask, d_out, env->n_sm, st);
		e = cudaGetLastError();
	}
	// cropped back to the original size (result.crop(dims - diff), top-left aligned)
	if (e == cudaSuccess) {
		e = extended ? cudaMemcpy2DAsync(out, row, d_out, erow, row, h, cudaMemcpyDeviceToHost, st)
		             : cudaMemcpyAsync(out, d_out, sizeof(double) * n, cudaMemcpyDeviceToHost, st);
	}
	const cudaError_t sync = cudaStreamSynchronize(st);  // also on failure: nothing left in flight on the scratch
	if (e == cudaSuccess) e = sync;
	if (e != cudaSuccess) return fail(PF_ERR_CUDA, std::string("pf_convolve_noalloc: ") + cudaGetErrorString(e));
	return PF_OK;
}

}  // extern "C"
