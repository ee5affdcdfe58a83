/*
 * C-callable driver around the UNMODIFIED libprofit sources, compiled from the
 * reference tree by oracle/Makefile into oracle/_ref/. TEST INFRASTRUCTURE
 * ONLY: it pins the oracle restatement (oracle/profit_oracle.c) and generates
 * the golden fixtures under tests/golden/. It drives the reference through its
 * public C++ API exactly as a user would: profit::Model, add_profile,
 * Profile::parameter, set_psf, set_convolver(create_convolver(...)),
 * Model::evaluate (include/profit/model.h, include/profit/profile.h,
 * include/profit/convolve.h), and profit::from_fits / to_fits
 * (include/profit/fits_utils.h) for the FITS fixtures.
 */
#include <cstring>
#include <exception>
#include <string>
#include <vector>

#include "profit/fits_utils.h"
#include "profit/profit.h"
#include "profit_oracle.h"

namespace {

const char *kind_name(int kind)
{
	switch (kind) {
	case ORC_SERSIC: return "sersic";
	case ORC_CORESERSIC: return "coresersic";
	case ORC_MOFFAT: return "moffat";
	case ORC_FERRER: return "ferrer";
	case ORC_KING: return "king";
	case ORC_BROKENEXP: return "brokenexp";
	case ORC_SKY: return "sky";
	case ORC_PSF: return "psf";
	default: return "null";
	}
}

void set_params(profit::ProfilePtr &p, const orc_profile &d)
{
	const double *v = d.par;
	p->parameter("convolve", d.convolve != 0);
	if (d.kind >= ORC_SERSIC && d.kind <= ORC_BROKENEXP) {
		p->parameter("xcen", v[ORC_P_XCEN]);
		p->parameter("ycen", v[ORC_P_YCEN]);
		p->parameter("mag", v[ORC_P_MAG]);
		p->parameter("ang", v[ORC_P_ANG]);
		p->parameter("axrat", v[ORC_P_AXRAT]);
		p->parameter("box", v[ORC_P_BOX]);
		p->parameter("rough", d.rough != 0);
		p->parameter("adjust", d.adjust != 0);
		p->parameter("acc", d.acc);
		p->parameter("rscale_switch", d.rscale_switch);
		p->parameter("rscale_max", d.rscale_max);
		p->parameter("resolution", d.resolution);
		p->parameter("max_recursions", d.max_recursions);
	}
	switch (d.kind) {
	case ORC_SERSIC:
		p->parameter("re", v[6]);
		p->parameter("nser", v[7]);
		p->parameter("rescale_flux", d.rescale_flux != 0);
		break;
	case ORC_CORESERSIC:
		p->parameter("re", v[6]);
		p->parameter("nser", v[7]);
		p->parameter("rb", v[8]);
		p->parameter("a", v[9]);
		p->parameter("b", v[10]);
		break;
	case ORC_MOFFAT:
		p->parameter("fwhm", v[6]);
		p->parameter("con", v[7]);
		break;
	case ORC_FERRER:
		p->parameter("rout", v[6]);
		p->parameter("a", v[7]);
		p->parameter("b", v[8]);
		break;
	case ORC_KING:
		p->parameter("rc", v[6]);
		p->parameter("rt", v[7]);
		p->parameter("a", v[8]);
		break;
	case ORC_BROKENEXP:
		p->parameter("h1", v[6]);
		p->parameter("h2", v[7]);
		p->parameter("rb", v[8]);
		p->parameter("a", v[9]);
		break;
	case ORC_SKY:
		p->parameter("bg", v[6]);
		break;
	case ORC_PSF:
		p->parameter("xcen", v[ORC_P_XCEN]);
		p->parameter("ycen", v[ORC_P_YCEN]);
		p->parameter("mag", v[ORC_P_MAG]);
		break;
	}
}

} // namespace

extern "C" int ref_evaluate(const orc_model *m, const orc_profile *profiles, int n_profiles,
                            double *out, size_t out_cap, unsigned int *out_w, unsigned int *out_h,
                            long long *level_counts, char *err, int err_len)
{
	try {
		profit::Model model(m->width, m->height);
		model.set_image_pixel_scale({m->scale_x, m->scale_y});
		model.set_magzero(m->magzero);
		model.set_finesampling(m->finesampling ? m->finesampling : 1);
		model.set_return_finesampled(m->return_finesampled != 0);
		model.set_omp_threads(m->omp_threads > 0 ? (unsigned int)m->omp_threads : 0U);
		if (m->psf && m->psf_w && m->psf_h) {
			std::vector<double> psf(m->psf, m->psf + (size_t)m->psf_w * m->psf_h);
			model.set_psf(profit::Image(psf, m->psf_w, m->psf_h));
			model.set_psf_pixel_scale({m->psf_scale_x, m->psf_scale_y});
		}
		profit::ConvolverCreationPreferences prefs;
		prefs.omp_threads = m->omp_threads > 0 ? (unsigned int)m->omp_threads : 1U;
		model.set_convolver(profit::create_convolver(
		    m->convolver == 1 ? profit::ConvolverType::BRUTE_OLD : profit::ConvolverType::BRUTE, prefs));
		for (int i = 0; i < n_profiles; i++) {
			auto p = model.add_profile(kind_name(profiles[i].kind));
			set_params(p, profiles[i]);
		}
		if (m->mask) {
			// Model::set_mask with the mask's own dimensions, adjusted or used
			// as given (Model::set_adjust_mask)
			std::vector<bool> mk((size_t)m->mask_w * m->mask_h);
			for (size_t q = 0; q < mk.size(); q++) mk[q] = m->mask[q] != 0;
			model.set_mask(profit::Mask(mk, m->mask_w, m->mask_h));
			model.set_adjust_mask(m->adjust_mask != 0);
		}
		profit::Image image = model.evaluate();
		auto dims = image.getDimensions();
		if ((size_t)dims.x * dims.y > out_cap) {
			std::strncpy(err, "output buffer too small", err_len);
			return -2;
		}
		std::memcpy(out, image.data(), sizeof(double) * dims.x * dims.y);
		*out_w = dims.x;
		*out_h = dims.y;
#ifdef PROFIT_DEBUG
		if (level_counts) {
			/* profiles of the same kind share a name, so only one radial
			 * profile per model gives unambiguous counts */
			auto integrations = model.get_profile_integrations();
			for (int i = 0; i < n_profiles; i++) {
				auto it = integrations.find(kind_name(profiles[i].kind));
				if (it == integrations.end()) {
					continue;
				}
				for (auto &kv : it->second) {
					if (kv.first >= 0 && kv.first < 32) {
						level_counts[(size_t)i * 32 + kv.first] = kv.second;
					}
				}
			}
		}
#else
		(void)level_counts;
#endif
		return 0;
	}
	catch (const std::exception &e) {
		std::strncpy(err, e.what(), err_len - 1);
		err[err_len - 1] = 0;
		return -1;
	}
}

// profit::to_fits (src/fits_utils.cpp:150-205) on a row-major image.
extern "C" int ref_to_fits(const double *image, unsigned int w, unsigned int h, unsigned int offset_x,
                           unsigned int offset_y, double scale_x, double scale_y, const char *fname, char *err,
                           int err_len)
{
	try {
		std::vector<double> data(image, image + (size_t)w * h);
		profit::Point offset(offset_x, offset_y);
		profit::to_fits(profit::Image(data, w, h), offset, {scale_x, scale_y}, fname);
		return 0;
	}
	catch (const std::exception &e) {
		std::strncpy(err, e.what(), err_len - 1);
		err[err_len - 1] = 0;
		return -1;
	}
}

// profit::from_fits (src/fits_utils.cpp:60-126): dimensions and scale, and the
// pixels when they fit in `cap` values.
extern "C" int ref_from_fits(const char *fname, double *out, size_t cap, unsigned int *w, unsigned int *h,
                             double *scale_x, double *scale_y, char *err, int err_len)
{
	try {
		profit::PixelScale scale;
		profit::Image image = profit::from_fits(fname, scale);
		*w = image.getWidth();
		*h = image.getHeight();
		*scale_x = scale.first;
		*scale_y = scale.second;
		if (image.size() > cap) {
			std::strncpy(err, "output buffer too small", err_len);
			return -2;
		}
		std::memcpy(out, image.data(), sizeof(double) * image.size());
		return 0;
	}
	catch (const std::exception &e) {
		std::strncpy(err, e.what(), err_len - 1);
		err[err_len - 1] = 0;
		return -1;
	}
}
