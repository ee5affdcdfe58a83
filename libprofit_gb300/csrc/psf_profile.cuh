// PsfProfile::evaluate for one drawing pixel, shared by both precisions.
#pragma once

#include <cmath>

#include "pf_device.cuh"

namespace pf {

__device__ __forceinline__ unsigned int bind_psf(double value, unsigned int max)  // src/psf.cpp:47-55
{
	int intval = (int)floor(value);
	if (intval < 0) return 0;
	unsigned int u = (unsigned int)intval;
	return u < max ? u : max;
}

// PsfProfile::evaluate for one drawing pixel (src/psf.cpp:58-145, including
// the offset.x / offset.y mix-up of lines 79-82). Returns false if the pixel
// is outside the stamp.
__device__ __forceinline__ bool psf_pixel64(const ProfileDev &P, const ModelDev &m, const double *psf, unsigned int pix_x,
                            unsigned int pix_y, double &out)
{
	const double xcen = P.par[PF_P_XCEN], ycen = P.par[PF_P_YCEN];
	const double scale_x = m.sx, scale_y = m.sy;
	const double psf_scale_x = m.psf_scale_x, psf_scale_y = m.psf_scale_y;
	const unsigned int width = m.draw_w, height = m.draw_h;
	const unsigned int psf_width = m.psf_w, psf_height = m.psf_h;
	const double off_x = m.pad_x, off_y = m.pad_y;
	const double origin_x = xcen + off_x * scale_x - psf_width * psf_scale_x / 2;
	const double end_x = xcen + off_y * scale_y + psf_width * psf_scale_x / 2;
	const double origin_y = ycen + off_x * scale_x - psf_height * psf_scale_y / 2;
	const double end_y = ycen + off_y * scale_y + psf_height * psf_scale_y / 2;
	const unsigned int x0 = bind_psf(origin_x / scale_x, width - 1);
	const unsigned int y0 = bind_psf(origin_y / scale_y, height - 1);
	const unsigned int x1 = bind_psf(end_x / scale_x, width - 1);
	const unsigned int y1 = bind_psf(end_y / scale_y, height - 1);
	if (pix_x < x0 || pix_x > x1 || pix_y < y0 || pix_y > y1) {
		return false;
	}
	const double y = pix_y * scale_y;
	const double x = pix_x * scale_x;
	const int psf_pix_x0 = (int)bind_psf(floor((x - origin_x) / psf_scale_x), psf_width - 1);
	const int psf_pix_x1 = (int)bind_psf(floor((x - origin_x + scale_x) / psf_scale_x), psf_height - 1);
	const int psf_pix_y0 = (int)bind_psf(floor((y - origin_y) / psf_scale_y), psf_width - 1);
	const int psf_pix_y1 = (int)bind_psf(floor((y - origin_y + scale_y) / psf_scale_y), psf_height - 1);
	double val = 0;
	for (int py = psf_pix_y0; py <= psf_pix_y1; py++) {
		const double psf_y = py * psf_scale_y + origin_y;
		for (int px = psf_pix_x0; px <= psf_pix_x1; px++) {
			const double psf_x = px * psf_scale_x + origin_x;
			const double ix = fmin(x + scale_x, psf_x + psf_scale_x) - fmax(x, psf_x);
			const double iy = fmin(y + scale_y, psf_y + psf_scale_y) - fmax(y, psf_y);
			val += psf[px + py * psf_width] * (ix * iy) / (psf_scale_x * psf_scale_y);
		}
	}
	out = val * P.psf_mag_scale;
	return true;
}

}  // namespace pf
