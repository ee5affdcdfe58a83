/*
 * CPU oracle for libprofit's image-generation path: TEST INFRASTRUCTURE ONLY.
 * Only tests/, the smoke check and the CPU-baseline leg of the benchmark load
 * this library; the CUDA product never links or calls it.
 *
 * It restates, in plain C and with the reference's own operation order,
 *   Model::evaluate / produce_image        (src/model.cpp:152-184, 259-360)
 *   RadialProfile::evaluate_cpu            (src/radial.cpp:291-344)
 *   RadialProfile::subsample_pixel         (src/radial.cpp:55-135)
 *   RadialProfile::initial_calculations    (src/radial.cpp:137-199)
 *   the six evaluate_at / get_lumtot / adjust_* families
 *     (src/sersic.cpp, src/coresersic.cpp, src/moffat.cpp, src/ferrer.cpp,
 *      src/king.cpp, src/brokenexponential.cpp)
 *   SkyProfile::evaluate                   (src/sky.cpp:42-63)
 *   PsfProfile::evaluate                   (src/psf.cpp:58-145)
 *   BruteForceConvolver / AssociativeBruteForceConvolver (src/convolve.cpp:101-231)
 *   Image::downsample(SUM)                 (src/image.cpp:250-262)
 * and additionally reports, per radial profile, the deepest subsampling level
 * reached at each pixel and the number of subsample_pixel calls per level
 * (the quantity PROFIT_DEBUG builds record in n_integrations,
 * src/radial.cpp:71-79).
 */
#ifndef PF_ORACLE_H
#define PF_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* profile kinds (names as accepted by Model::add_profile, src/model.cpp:103-135) */
enum {
	ORC_SERSIC = 0,
	ORC_CORESERSIC = 1,
	ORC_MOFFAT = 2,
	ORC_FERRER = 3,
	ORC_KING = 4,
	ORC_BROKENEXP = 5,
	ORC_SKY = 6,
	ORC_PSF = 7,
	ORC_NULL = 8
};

/* parameter slots in orc_profile.par */
enum {
	ORC_P_XCEN = 0, ORC_P_YCEN = 1, ORC_P_MAG = 2, ORC_P_ANG = 3, ORC_P_AXRAT = 4, ORC_P_BOX = 5,
	ORC_P_X0 = 6 /* first profile-specific slot */
};
/* profile-specific slots:
 *   sersic      6 re, 7 nser
 *   coresersic  6 re, 7 nser, 8 rb, 9 a, 10 b
 *   moffat      6 fwhm, 7 con
 *   ferrer      6 rout, 7 a, 8 b
 *   king        6 rc, 7 rt, 8 a
 *   brokenexp   6 h1, 7 h2, 8 rb, 9 a
 *   sky         6 bg
 *   psf         0 xcen, 1 ycen, 2 mag
 */
#define ORC_NPAR 12

typedef struct {
	int kind;
	int convolve;
	int rough;
	int adjust;
	int rescale_flux;
	unsigned int resolution;
	unsigned int max_recursions;
	double acc;
	double rscale_switch;
	double rscale_max;
	double par[ORC_NPAR];
} orc_profile;

typedef struct {
	unsigned int width, height;
	double scale_x, scale_y;
	double magzero;
	unsigned int finesampling;
	int return_finesampled;
	/* PSF (raw; normalised here as Model::set_psf does, include/profit/model.h:148-158) */
	const double *psf;
	unsigned int psf_w, psf_h;
	double psf_scale_x, psf_scale_y;
	/* optional calculation mask (non-zero = evaluate), or NULL. With
	 * adjust_mask (the reference's default, Model::set_adjust_mask) it has the
	 * model's dimensions and is adjusted as Model::evaluate does
	 * (src/model.cpp:152-257: padding decided by its bounding box, upsampled,
	 * extended, expanded by half the PSF) and the final image is masked by it;
	 * without, it is used as given and must have the drawing dimensions, which
	 * include the PSF padding only if the mask is larger than the model's
	 * dimensions times the finesampling in both directions
	 * (src/model.cpp:165-167, 277-283). mask_w x mask_h: its dimensions. */
	const unsigned char *mask;
	int adjust_mask;
	unsigned int mask_w, mask_h;
	/* 0: BRUTE (associative row dot products), 1: BRUTE_OLD */
	int convolver;
	int omp_threads;
} orc_model;

/* Per-profile constants after initial_calculations (for tests). */
typedef struct {
	double rscale, ie, bn, lumtot, rescale_factor;
	double rscale_switch, rscale_max, acc;
	unsigned int resolution;
	double cos_ang, sin_ang;
	double flux_scale;
} orc_constants;

/*
 * Evaluates the model. `out` receives the final image (out_w x out_h, written
 * to *out_w / *out_h; callers size it with orc_output_dims).
 * `depth` (optional) receives n_profiles maps of the drawing dimensions:
 * -1 where the pixel was not evaluated (masked or beyond rscale_max),
 * 0 where evaluate_at was used directly, k >= 1 where subsample_pixel recursed
 * down to level k-1.
 * `level_counts` (optional) receives n_profiles x 32 counts of subsample_pixel
 * calls per recursion level.
 * Returns 0, or a negative code with a message in orc_last_error().
 */
int orc_evaluate(const orc_model *m, const orc_profile *profiles, int n_profiles,
                 double *out, unsigned int *out_w, unsigned int *out_h,
                 signed char *depth, long long *level_counts);

int orc_output_dims(const orc_model *m, const orc_profile *profiles, int n_profiles,
                     unsigned int *out_w, unsigned int *out_h,
                     unsigned int *draw_w, unsigned int *draw_h);

int orc_profile_constants(const orc_model *m, const orc_profile *p, orc_constants *c);

/* Direct ("same") convolution as the BRUTE convolvers compute it. */
void orc_convolve_brute(const double *src, unsigned int w, unsigned int h,
                        const double *krn, unsigned int kw, unsigned int kh,
                        const unsigned char *mask, double *out, int old_variant, int omp_threads);

const char *orc_last_error(void);

/* special functions (re-exported for tests) */
double orc_api_qgamma(double p, double a);
double orc_api_pgamma(double x, double a);
double orc_api_gammafn(double x);
double orc_api_beta(double a, double b);

#ifdef __cplusplus
}
#endif

#endif
