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

// The stamp's drawing rows [y0, y1] and columns [x0, x1] (the loop bounds of
// src/psf.cpp:75-90, with the same offset mix-up).
__device__ __forceinline__ void psf_stamp(const ProfileDev &P, const ModelDev &m, int &x0, int &x1, int &y0, int &y1)
{
	const double xcen = P.par[PF_P_XCEN], ycen = P.par[PF_P_YCEN];
	const double origin_x = xcen + m.pad_x * m.sx - m.psf_w * m.psf_scale_x / 2;
	const double end_x = xcen + m.pad_y * m.sy + m.psf_w * m.psf_scale_x / 2;
	const double origin_y = ycen + m.pad_x * m.sx - m.psf_h * m.psf_scale_y / 2;
	const double end_y = ycen + m.pad_y * m.sy + m.psf_h * m.psf_scale_y / 2;
	x0 = (int)bind_psf(origin_x / m.sx, m.draw_w - 1);
	y0 = (int)bind_psf(origin_y / m.sy, m.draw_h - 1);
	x1 = (int)bind_psf(end_x / m.sx, m.draw_w - 1);
	y1 = (int)bind_psf(end_y / m.sy, m.draw_h - 1);
}

// The psf profile's unscaled value at drawing pixel (pix_x, pix_y) and its
// derivatives with respect to xcen and ycen: the PSF pixels overlapping the
// image pixel move with the centre, so each overlap length changes at rate
// +1 where the PSF pixel's far edge is the nearer one and -1 where its near
// edge is the farther one (piecewise linear in the centre; the pixel sets
// are those of psf_pixel64). False outside the stamp.
__device__ __forceinline__ bool psf_pixel_grad64(const ProfileDev &P, const ModelDev &m, const double *psf,
                                                 unsigned int pix_x, unsigned int pix_y, double &val, double &dx,
                                                 double &dy)
{
	const double xcen = P.par[PF_P_XCEN], ycen = P.par[PF_P_YCEN];
	const double scale_x = m.sx, scale_y = m.sy;
	const double psf_scale_x = m.psf_scale_x, psf_scale_y = m.psf_scale_y;
	const unsigned int psf_width = m.psf_w, psf_height = m.psf_h;
	const double origin_x = xcen + m.pad_x * scale_x - psf_width * psf_scale_x / 2;
	const double origin_y = ycen + m.pad_x * scale_x - psf_height * psf_scale_y / 2;
	int x0, x1, y0, y1;
	psf_stamp(P, m, x0, x1, y0, y1);
	if ((int)pix_x < x0 || (int)pix_x > x1 || (int)pix_y < y0 || (int)pix_y > y1) return false;
	const double y = pix_y * scale_y;
	const double x = pix_x * scale_x;
	const int psf_pix_x0 = (int)bind_psf(floor((x - origin_x) / psf_scale_x), psf_width - 1);
	const int psf_pix_x1 = (int)bind_psf(floor((x - origin_x + scale_x) / psf_scale_x), psf_height - 1);
	const int psf_pix_y0 = (int)bind_psf(floor((y - origin_y) / psf_scale_y), psf_width - 1);
	const int psf_pix_y1 = (int)bind_psf(floor((y - origin_y + scale_y) / psf_scale_y), psf_height - 1);
	const double inv_area = 1. / (psf_scale_x * psf_scale_y);
	val = dx = dy = 0;
	for (int py = psf_pix_y0; py <= psf_pix_y1; py++) {
		const double psf_y = py * psf_scale_y + origin_y;
		const double iy = fmin(y + scale_y, psf_y + psf_scale_y) - fmax(y, psf_y);
		const double diy = (psf_y + psf_scale_y < y + scale_y ? 1. : 0.) - (psf_y > y ? 1. : 0.);
		for (int px = psf_pix_x0; px <= psf_pix_x1; px++) {
			const double psf_x = px * psf_scale_x + origin_x;
			const double ix = fmin(x + scale_x, psf_x + psf_scale_x) - fmax(x, psf_x);
			const double dix = (psf_x + psf_scale_x < x + scale_x ? 1. : 0.) - (psf_x > x ? 1. : 0.);
			const double w = psf[px + py * psf_width] * inv_area;
			val += w * (ix * iy);
			dx += w * (dix * iy);
			dy += w * (ix * diy);
		}
	}
	return true;
}

}  // namespace pf
