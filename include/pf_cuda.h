/*
 * pf_cuda.h - C ABI of the GB300-native backend for libprofit's
 * image-generation path (profile evaluation with adaptive subsampling, sky and
 * psf profiles, PSF convolution).
 *
 * This is the boundary a libprofit build would bind to add a CUDA environment
 * beside its OpenCL one and a CUDA convolver type:
 *   - pf_env_*            replaces get_opencl_environment / OpenCLEnv
 *                         (include/profit/opencl.h:79-168); PF_ENV_DOUBLE plays
 *                         the role of OpenCLEnvImpl::use_double
 *                         (include/profit/opencl_impl.h:122).
 *   - pf_model_evaluate   is what Model::evaluate (src/model.cpp:259-320) calls
 *                         when a CUDA environment is set, in place of the
 *                         per-profile RadialProfile::evaluate dispatch
 *                         (src/radial.cpp:262-287): one call renders the whole
 *                         model (all profiles, convolution, crop) on the GPU.
 *   - pf_convolve         is Convolver::convolve (src/convolve.cpp:55-79) for
 *                         a ConvolverType::CUDA created by create_convolver
 *                         (src/convolve.cpp:521-584).
 *   - pf_batch_*, pf_forward, pf_backward: the batched path (many models in
 *                         one launch sequence) and its adjoint; they have no
 *                         counterpart in the reference.
 * Parameter names, defaults, validation messages and error categories are the
 * reference's (Profile::parameter, src/profile.cpp:69-163; the validate()
 * methods; include/profit/exceptions.h:41-104). No function throws; each
 * returns a pf_status and leaves a message readable with pf_last_error().
 *
 * All pointers are plain host pointers unless the parameter name ends in _dev
 * (device memory). Streams are cudaStream_t passed as void*.
 */
#ifndef PF_CUDA_H
#define PF_CUDA_H

#include <stddef.h>
#include <stdint.h>

#if defined(__GNUC__) || defined(__clang__)
#define PF_API __attribute__((visibility("default")))
#else
#define PF_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

typedef enum pf_status {
	PF_OK = 0,
	PF_ERR_INVALID_PARAMETER = 1, /* profit::invalid_parameter */
	PF_ERR_UNKNOWN_PARAMETER = 2, /* profit::unknown_parameter */
	PF_ERR_CUDA = 3,              /* a CUDA runtime call failed (profit::opencl_error analogue) */
	PF_ERR_NO_MEMORY = 4,
	PF_ERR_DEVICE_LIMIT = 5,      /* a bounded device-side resource was exceeded */
	PF_ERR_UNSUPPORTED = 6,
	PF_ERR_INTERNAL = 7,
	PF_ERR_INVALID_FILE = 8       /* profit::invalid_file */
} pf_status;

/* Profile kinds, by the names Model::add_profile accepts (src/model.cpp:103-135). */
enum pf_profile_kind {
	PF_SERSIC = 0,
	PF_CORESERSIC = 1,
	PF_MOFFAT = 2,
	PF_FERRER = 3,
	PF_KING = 4,
	PF_BROKENEXP = 5,
	PF_SKY = 6,
	PF_PSF = 7,
	PF_NULL = 8,
	PF_USER = 9   /* the user-defined radial profile compiled into the library, if any
	                 (pf_user_profile_info; libprofit_gb300/user_profiles/example_moffat.cuh) */
};

/* Parameter slots of pf_profile_desc.par. Slots 0-5 are the radial
 * parameters common to all six radial profiles (src/radial.cpp:741-746);
 * slots from 6 on are profile-specific:
 *   sersic      6 re, 7 nser                       (src/sersic.cpp:352-360)
 *   coresersic  6 re, 7 nser, 8 rb, 9 a, 10 b      (src/coresersic.cpp:131-141)
 *   moffat      6 fwhm, 7 con                      (src/moffat.cpp:101-107)
 *   ferrer      6 rout, 7 a, 8 b                   (src/ferrer.cpp:111-122)
 *   king        6 rc, 7 rt, 8 a                    (src/king.cpp:110-118)
 *   brokenexp   6 h1, 7 h2, 8 rb, 9 a              (src/brokenexponential.cpp:141-150)
 *   sky         6 bg                               (src/sky.cpp:65-71)
 *   psf         0 xcen, 1 ycen, 2 mag              (src/psf.cpp:147-156)
 */
enum pf_param_slot {
	PF_P_XCEN = 0, PF_P_YCEN = 1, PF_P_MAG = 2, PF_P_ANG = 3, PF_P_AXRAT = 4, PF_P_BOX = 5,
	PF_P_X0 = 6
};
#define PF_NPAR 12

/* One profile. The sub-pixel integration controls are the reference's
 * (src/radial.cpp:738-751); defaults: rough 0, adjust 1, resolution 9,
 * max_recursions 2, acc 0.1 (1 for ferrer), rscale_switch 1, rscale_max 0. */
typedef struct pf_profile_desc {
	int32_t kind;
	int32_t convolve;      /* Profile "convolve" (default 0, src/profile.cpp:38-45) */
	int32_t rough;
	int32_t adjust;
	int32_t rescale_flux;  /* sersic only */
	uint32_t resolution;
	uint32_t max_recursions;
	double acc;
	double rscale_switch;
	double rscale_max;
	double par[PF_NPAR];
} pf_profile_desc;

enum pf_convolver {
	PF_CONV_AUTO = 0,   /* autotuner choice (direct for the double mode; in single precision
	                       the FFT only where it cuts the convolution's time fourfold, its
	                       rounding being absolute, about 1e-7 x the image peak) */
	PF_CONV_BRUTE = 1,  /* shared-memory-tiled direct convolution */
	PF_CONV_FFT = 2     /* Stockham FFT convolution (a model whose transforms would exceed 8192
	                       points per side in single precision, 4096 in double, takes the
	                       direct convolution: the same cropped image, exactly) */
};

/* One model: Model(width, height) with its setters (include/profit/model.h:130-330). */
typedef struct pf_model_desc {
	uint32_t width, height;
	double scale_x, scale_y;          /* set_image_pixel_scale */
	double magzero;                   /* set_magzero */
	uint32_t finesampling;            /* set_finesampling (>= 1) */
	int32_t return_finesampled;       /* set_return_finesampled */
	uint32_t first_profile;           /* this model's profiles are [first, first + n) */
	uint32_t n_profiles;
	int64_t psf_offset;               /* element offset of the raw PSF in psf_pool, -1: none */
	uint32_t psf_w, psf_h;            /* set_psf (normalised to unit sum on the device) */
	double psf_scale_x, psf_scale_y;  /* set_psf_pixel_scale */
	int32_t convolver;                /* pf_convolver */
	int32_t reserved;
	/* Calculation mask (Model::set_mask, include/profit/model.h:219-246): one
	 * byte per pixel, non-zero = evaluate, at this offset in the mask pool of
	 * pf_batch_create_masked (-1: none; pf_batch_create ignores it).
	 * adjust_mask 1 (the reference's default): the mask has the model's
	 * width x height and is adjusted as Model::evaluate does (PSF padding only
	 * when the mask's bounding box needs it, upsampled by the finesampling,
	 * expanded by half the PSF; the output image masked by it at the end,
	 * src/model.cpp:152-257); 0: the mask is used as given and must have the
	 * drawing dimensions: width x height times the finesampling, plus half the
	 * PSF on each side if the mask is larger than that in both directions
	 * (src/model.cpp:165-167, 277-283). mask_w x mask_h: the mask's
	 * dimensions ("Mask dimensions != model dimensions" / "!= drawing
	 * dimensions" otherwise). */
	int64_t mask_offset;
	int32_t adjust_mask;
	/* Model::set_crop(false) (include/profit/model.h:206-214): 1 = keep the
	 * padding the convolver adds (src/model.cpp:288-306). The direct
	 * convolutions add none (Convolver::padding is empty, src/convolve.cpp:
	 * 50-53), so their image is the cropped one, at offset (0, 0); PF_CONV_FFT
	 * gives the FFT convolver's uncropped frame with only the PSF padding
	 * removed (pf_model_output_dims / pf_model_output_offset give its size
	 * and offset; double precision only). 0 (the default): crop. */
	int32_t no_crop;
	uint32_t mask_w, mask_h;
} pf_model_desc;

typedef struct pf_env pf_env;
typedef struct pf_batch pf_batch;

/* Environment flags */
#define PF_ENV_DOUBLE 0x1u   /* plain FP64 path: the reference's arithmetic and subsampling decisions */
#define PF_ENV_PROFILE 0x2u  /* time every stage with CUDA events (the profiling OpenCL
                                environment's OpenCL_times, include/profit/opencl.h:50-71) */
#define PF_ENV_NO_AUTOTUNE 0x4u  /* single precision, PF_CONV_AUTO: choose brute force or FFT and
                                    the direct block shape by the fixed cost model, never by
                                    timing candidates on the device (reproducible choices) */
#define PF_ENV_NO_SPLIT 0x8u     /* walk every subsampled pixel's tree in the warp that meets
                                    it: in single precision none split off to other warps, in
                                    double precision no level-by-level evaluation (the images
                                    then sum each pixel's profiles strictly in order) */

/* Per-stage device times accumulated since the last reset (PF_ENV_PROFILE). */
typedef struct pf_stage_times {
	double setup_ms;         /* per-profile constants */
	double eval_ms;          /* profile evaluation with subsampling */
	double finish_ms;        /* convolution, add, crop, downsample */
	double chi2_ms;          /* chi^2 and its cotangent */
	double adjoint_conv_ms;  /* transposed convolution */
	double backward_ms;      /* adjoint evaluation and gradient reduction */
	uint64_t forward_calls, backward_calls;
	uint64_t kernel_launches;  /* this library's kernels launched (graph replays included) */
} pf_stage_times;

/* The user-defined radial profile compiled into this library (the CUDA
 * counterpart of a RadialProfile subclass added to libprofit,
 * docs/new_profile.rst): its Model::add_profile name and its own parameters
 * (slots 6, 7, ... of pf_profile_desc.par) with their defaults.
 * PF_ERR_UNSUPPORTED when the library was built without one. Profiles of
 * kind PF_USER are evaluated in PF_ENV_DOUBLE environments only. */
PF_API pf_status pf_user_profile_info(const char **name, const char *const **param_names,
                                      const double **param_defaults, uint32_t *n_params);

/* Last error message of the calling thread. */
PF_API const char *pf_last_error(void);

/* Library version ("<major>.<minor>.<patch>") and build information. */
PF_API const char *pf_version(void);

/* Creates an environment on CUDA device `device` (get_opencl_environment
 * analogue, include/profit/opencl.h:159-168). */
PF_API pf_status pf_env_create(int device, uint32_t flags, pf_env **env);
PF_API void pf_env_destroy(pf_env *env);

/*
 * Model::evaluate for one model with host buffers (src/model.cpp:259-320):
 * validates like analyze_inputs, draws every profile into the padded drawing
 * area, convolves the profiles with convolve=1 by the model's PSF, adds,
 * crops the PSF padding, optionally downsamples. `image` receives
 * out_w * out_h doubles (query the size with pf_model_output_dims, which
 * also checks a mask's declared dimensions: mask_offset >= 0, mask_w x mask_h).
 *
 * The environment keeps the device state of its last call: a model that
 * differs from the previous one in parameter values only (a fitting loop's
 * Model::evaluate) reuses it and allocates nothing -- its parameters are
 * validated as a new model's would be, uploaded, and its constants
 * recomputed on the device. Any other change (dimensions, profiles and their
 * flags, PSF or mask contents) builds the state anew. Calls on one
 * environment are serialised (a mutex), as the reference's Model::evaluate
 * is not re-entrant either.
 */
PF_API pf_status pf_model_output_dims(const pf_model_desc *model, const pf_profile_desc *profiles,
                               uint32_t *out_w, uint32_t *out_h);
/* The offset Model::evaluate(Point &offset_out) reports (src/model.cpp:259-320):
 * where the requested area lies in the returned image. (0, 0) unless crop = 0
 * (no_crop) with the FFT convolver, whose uncropped frame the image is then
 * (double precision only; not with SUM downsampling or an adjustable mask). */
PF_API pf_status pf_model_output_offset(const pf_model_desc *model, const pf_profile_desc *profiles,
                                        uint32_t *offset_x, uint32_t *offset_y);
PF_API pf_status pf_model_evaluate(pf_env *env, const pf_model_desc *model, const pf_profile_desc *profiles,
                            const double *psf, double *image, uint32_t *out_w, uint32_t *out_h);
/* The statistics of the last pf_model_evaluate* call on env, for
 * Model::get_stats (src/model.cpp:362-368, the ProfileStats of
 * include/profit/profile.h:46-73). With PF_ENV_PROFILE: that call's stage
 * times (setup, evaluation, convolution: the fused passes of all its
 * profiles, timed with CUDA events), and per profile 32 counts as
 * pf_batch_depth gives them -- subsample_pixel calls per recursion level in
 * [0, 16), evaluate_at calls on pixel centres [30] and inside
 * subsample_pixel [31] -- by which a caller can attribute the evaluation
 * time to its profiles. Without it, all zero. level_counts: n_profiles x 32,
 * or NULL. */
PF_API pf_status pf_env_last_model_stats(pf_env *env, pf_stage_times *times, int64_t *level_counts,
                                         size_t n_profiles);

/* The autotuner's decisions (single precision: the convolution method per
 * model and the block shapes of large PF_CONV_AUTO batches, whether the
 * subsampling trees split off to other warps) are kept by the environment,
 * keyed by the GPU and the batch's layout (dimensions, PSF sizes, convolvers,
 * masks, profile kinds and subsampling controls; not parameter values): a
 * batch of a layout seen before is created without timing anything, as
 * FFTW reuses a plan. With the environment variable PF_AUTOTUNE_CACHE naming
 * a file when the environment is created, the decisions are read from it
 * and new ones appended to it (one text line each), so that they outlive the
 * process, as FFTW's wisdom does (include/profit/library.h, src/library.cpp:
 * 69-165). timed: decisions made by timing in this environment; reused:
 * decisions taken from the cache. Either pointer may be NULL. */
PF_API pf_status pf_env_autotune_counts(pf_env *env, uint64_t *timed, uint64_t *reused);
/* The same with a calculation mask (host bytes; dimensions as the model's
 * adjust_mask says; NULL: none). */
PF_API pf_status pf_model_evaluate_masked(pf_env *env, const pf_model_desc *model, const pf_profile_desc *profiles,
                                   const double *psf, const uint8_t *mask, double *image, uint32_t *out_w,
                                   uint32_t *out_h);

/*
 * Convolver::convolve with ConvolverType::CUDA and crop = true
 * (src/convolve.cpp:55-79): `out` (w*h) = src convolved with krn, zero
 * boundary, the kernel's centre at (kw/2, kh/2); output pixels whose mask
 * byte is 0 are 0 (mask may be NULL). Host buffers.
 */
PF_API pf_status pf_convolve(pf_env *env, const double *src, uint32_t w, uint32_t h,
                      const double *krn, uint32_t kw, uint32_t kh, const uint8_t *mask,
                      double *out);

/*
 * Convolver::convolve(src, krn, mask, crop, offset_out) with ConvolverType::CUDA
 * (include/profit/convolve.h:65-97): pf_convolve plus the crop flag and the
 * offset of the cropped image in the returned one. The CUDA convolver is a
 * direct convolution, which adds no padding (Convolver::padding is empty,
 * src/convolve.cpp:50-53, as for BRUTE): crop = 0 returns the same w*h image
 * and offset (0, 0), as mask_and_crop does (src/convolve.cpp:81-99).
 * offset_x / offset_y may be NULL (the reference's NO_OFFSET).
 *
 * pf_convolve and pf_convolve_crop keep their device buffers in the
 * environment, growing them only when an image larger than any before comes:
 * repeated calls allocate nothing after the first. Calls on one environment
 * are serialised (a mutex).
 */
PF_API pf_status pf_convolve_crop(pf_env *env, const double *src, uint32_t w, uint32_t h,
                                  const double *krn, uint32_t kw, uint32_t kh, const uint8_t *mask,
                                  int crop, double *out, uint32_t *offset_x, uint32_t *offset_y);

/*
 * pf_convolve_noalloc: pf_convolve that allocates no device memory after its
 * first call on a device. No counterpart in the reference.
 *
 * For callers that cannot allocate device memory at the moment they convolve:
 * a fitting loop running beside a caching allocator that holds almost all of
 * the device's memory (a cudaMalloc there fails), or a host thread feeding
 * other streams whose work must not stall (cudaFree synchronises the whole
 * device). Same arguments, results and errors as pf_convolve; the device work
 * is the same kernel on the environment's stream, and the call returns after
 * that stream has finished it.
 *
 * Its device scratch is a fixed array in this library's static device data,
 * 17.5 MiB on each device: the image (after its extension to the kernel's
 * size) may have at most PF_NOALLOC_MAX_PIXELS pixels and the kernel at most
 * PF_NOALLOC_MAX_KERNEL_PIXELS; larger inputs are refused with
 * PF_ERR_DEVICE_LIMIT and nothing is run (use pf_convolve for them). Nothing
 * in the scratch needs to start at zero: every call writes every scratch
 * element it reads.
 *
 * The first call on each device looks up the scratch's address, which can
 * load this library's device code onto that device and so reserve the array;
 * make that first call before any stream capture. The address is kept for the
 * life of the process: after a cudaDeviceReset of that device this entry
 * point must not be called again. All calls on one device share the one
 * scratch: calls that overlap in time on the same device (from several
 * threads, or through several environments) race and give wrong results;
 * serialise them. A failure records its message for pf_last_error, as every
 * entry point does (that message is host memory).
 */
#define PF_NOALLOC_MAX_PIXELS (1u << 20)
#define PF_NOALLOC_MAX_KERNEL_PIXELS (1u << 16)
PF_API pf_status pf_convolve_noalloc(pf_env *env, const double *src, uint32_t w, uint32_t h,
                              const double *krn, uint32_t kw, uint32_t kh, const uint8_t *mask,
                              double *out);

/*
 * Batched path. pf_batch_create copies the descriptors, the PSF pool (host,
 * psf_pool_len doubles) and sizes every device buffer once; pf_forward then
 * allocates nothing. Output images of all models are packed back to back;
 * pf_batch_layout reports each model's offset (n_models + 1 entries) and
 * output dims (2 per model).
 */
PF_API pf_status pf_batch_create(pf_env *env, const pf_model_desc *models, size_t n_models,
                          const pf_profile_desc *profiles, size_t n_profiles,
                          const double *psf_pool, size_t psf_pool_len, pf_batch **batch);
/* pf_batch_create with calculation masks: each model's mask_offset (if not
 * -1) points into mask_pool (host, mask_pool_len bytes). */
PF_API pf_status pf_batch_create_masked(pf_env *env, const pf_model_desc *models, size_t n_models,
                                 const pf_profile_desc *profiles, size_t n_profiles, const double *psf_pool,
                                 size_t psf_pool_len, const uint8_t *mask_pool, size_t mask_pool_len,
                                 pf_batch **batch);
PF_API void pf_batch_destroy(pf_batch *batch);
PF_API pf_status pf_batch_layout(const pf_batch *batch, uint64_t *offsets, uint32_t *dims,
                          uint64_t *total_pixels);

/* Replaces every profile's par[] (n_profiles * PF_NPAR doubles, host), as a
 * fitting loop does between evaluations. Integration controls keep their
 * batch-creation values. */
PF_API pf_status pf_batch_set_params(pf_batch *batch, const double *params);

/* Same, from device memory, stream-ordered (no host synchronisation). */
PF_API pf_status pf_batch_set_params_dev(pf_batch *batch, const double *params_dev, void *stream);

/*
 * Renders every model of the batch. images_dev: total_pixels floats (double
 * for a PF_ENV_DOUBLE environment). flux_dev (optional): n_models doubles,
 * each model's total flux summed in FP64. Stream-ordered; returns once the
 * work is enqueued (device-side limit violations are reported by
 * pf_batch_check).
 */
PF_API pf_status pf_forward(pf_batch *batch, void *images_dev, double *flux_dev, void *stream);

/*
 * Adjoint (no counterpart in the reference, which has no derivatives).
 * pf_batch_enable_adjoint sizes the adjoint's device buffers once; then
 * pf_backward, given the images pf_forward rendered (images_dev), returns
 *   chi2_dev[m]  = sum over model m's pixels of ((image - data) / sigma)^2
 *                  (sigma_dev may be NULL: sigma = 1), in FP64;
 *   grad_dev[p * PF_NPAR + k] = d L / d par[k] of profile p (FP64), where L
 *                  is the chi^2 above, or, when cotangent_dev is not NULL,
 *                  L = sum cotangent * image (the vector-Jacobian product of
 *                  the images; chi2 is then 0).
 * data/sigma/cotangent have the images' layout and precision. The
 * subsampling tree of every pixel is recomputed, not stored, and held fixed.
 * Supported: the six radial profiles with all their parameters (a sersic
 * with rescale_flux too), sky (bg), psf (xcen, ycen, mag), null.
 * pf_forward_backward = pf_forward followed by pf_backward.
 */
PF_API pf_status pf_batch_enable_adjoint(pf_batch *batch);
PF_API pf_status pf_backward(pf_batch *batch, const void *images_dev, const void *data_dev,
                             const void *sigma_dev, const void *cotangent_dev, double *chi2_dev,
                             double *grad_dev, void *stream);
PF_API pf_status pf_forward_backward(pf_batch *batch, void *images_dev, const void *data_dev,
                                     const void *sigma_dev, double *chi2_dev, double *grad_dev,
                                     void *stream);

/*
 * One fitting step as a CUDA graph: pf_batch_set_params_dev(params_dev) (when
 * params_dev is not NULL), pf_forward(images_dev), pf_backward(images_dev,
 * data_dev, sigma_dev, chi2_dev, grad_dev) -- nine kernels -- captured into a
 * graph on the first call and replayed by every later call with the same
 * buffers, stream and depth recording: one launch per step. A call with other
 * buffers or another stream captures anew. Parameters set on the host
 * (pf_batch_set_params) are uploaded before the launch. The stream must be
 * one the caller created (the default stream cannot be captured); stage
 * times (PF_ENV_PROFILE) are not recorded for graph launches. No counterpart
 * in the reference.
 */
PF_API pf_status pf_step_graph(pf_batch *batch, const double *params_dev, void *images_dev, const void *data_dev,
                               const void *sigma_dev, double *chi2_dev, double *grad_dev, void *stream);

/* Synchronises the batch's work and returns the stage times recorded so far
 * (all zero unless the environment has PF_ENV_PROFILE); `reset` clears them. */
PF_API pf_status pf_batch_stats(pf_batch *batch, pf_stage_times *times, int reset);

/* Synchronises `stream` and reports any device-side error of earlier calls. */
PF_API pf_status pf_batch_check(pf_batch *batch, void *stream);

/* Records, on the next pf_forward, per radial profile and drawing pixel the
 * deepest subsampling level reached (-1: not evaluated, 0: evaluate_at used
 * directly, k: subsample_pixel recursed to level k-1) and the number of
 * subsample_pixel calls per level (PROFIT_DEBUG's n_integrations,
 * src/radial.cpp:71-79). */
PF_API pf_status pf_batch_record_depth(pf_batch *batch, int enable);
PF_API pf_status pf_batch_depth(pf_batch *batch, int8_t *depth, size_t depth_len,
                         int64_t *level_counts /* n_profiles * 32 */);
/* Per model the drawing area (width, height) the depth maps cover: the model's
 * dimensions times the finesampling plus the PSF padding, which an adjustable
 * mask far enough from the edges leaves out. `dims` holds 2 * n_models. */
PF_API pf_status pf_batch_drawing_dims(pf_batch *batch, uint32_t *dims);

/* The convolution plan the batch runs: the direct convolution's block shape
 * for the forward pass and for the adjoint (-1 before
 * pf_batch_enable_adjoint), and how many models use the FFT (chosen per model
 * by the autotuner, or requested). Any pointer may be NULL. */
PF_API pf_status pf_batch_conv_info(const pf_batch *batch, int32_t *forward_shape, int32_t *adjoint_shape,
                                    uint32_t *fft_models);

/* No counterpart: how the last forward pass spread its subsampling trees.
 * Single precision: boxes, sub-pixel boxes split off to other warps; roots,
 * the (profile, pixel) trees they came from; pixels, drawing pixels with at
 * least one; refused, splits walked in place for lack of room in the batch's
 * pool. Double precision: boxes, the boxes evaluated level by level (level 0
 * included); roots, the (profile, pixel) trees; pixels, drawing pixels with
 * at least one; refused, trees or subtrees walked in place for lack of room.
 * Synchronises the batch's stream (stream as in pf_forward). All zero when
 * the batch does not spread its trees: PF_ENV_NO_SPLIT environments, and
 * large automatic single-precision batches whose evaluation the autotuner
 * timed faster with every tree walked where met. Any argument may be NULL. */
PF_API pf_status pf_batch_split_info(pf_batch *batch, void *stream, uint32_t *boxes, uint32_t *roots,
                                     uint32_t *pixels, uint32_t *refused);

/* FITS images on either side of the path (host only, no device work): the
 * PSFs a caller reads in and the images it writes out.
 *
 * pf_fits_write is profit::to_fits (src/fits_utils.cpp:150-205): a primary
 * HDU of BITPIX -64, NAXIS 2 (NAXIS1 = width), the pixel scale as CDELT1/2 and
 * the origin's offset (whole pixels, the reference's unsigned Point,
 * include/profit/image.h:47-61) as CRVAL1/2 = (0.5 - offset) * scale, big-endian
 * doubles in row-major order, header and data each padded after their end
 * to the 2880-byte block (a whole block when they already end on one), and
 * ".fits" appended to `filename` unless it ends in it. The bytes written are
 * the reference's.
 *
 * pf_fits_read is profit::from_fits (src/fits_utils.cpp:60-126): 80-byte
 * header cards up to END, NAXIS1/NAXIS2/CDELT1/CDELT2 taken when present
 * (scale 1 by default), BITPIX taken to be -64, the data starting at the
 * 2880-byte block after END's card (a whole block further when END ends on
 * one, as the reference reads). With `image` NULL only the dimensions and
 * scale are reported; otherwise `image_len` must hold width * height.
 * A file that cannot be opened or read returns PF_ERR_INVALID_FILE with the
 * reference's messages (and a failed write with its own). */
PF_API pf_status pf_fits_write(const char *filename, const double *image, uint32_t width, uint32_t height,
                               uint32_t offset_x, uint32_t offset_y, double scale_x, double scale_y);
PF_API pf_status pf_fits_read(const char *filename, double *image, size_t image_len, uint32_t *width,
                              uint32_t *height, double *scale_x, double *scale_y);

#ifdef __cplusplus
}
#endif

#endif /* PF_CUDA_H */
