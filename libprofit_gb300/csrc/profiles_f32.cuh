// FP32 profile functions for the batched single-precision path.
//
// Same mathematics as the reference's evaluate_at (src/sersic.cpp:191-198,
// src/coresersic.cpp:51-59, src/moffat.cpp:52-58, src/ferrer.cpp:50-60,
// src/king.cpp:51-59, src/brokenexponential.cpp:38-94, boxy radius
// include/profit/radial.h:93-102), rewritten as exp2 / log2 chains so that
// every power runs on the special-function unit, with the per-profile
// constants (1/re^2, bn*log2(e), 0.5/nser, ...) folded once by the setup
// kernel into ProfileDev::fpar. Accuracy: a few 1e-7 relative in the bulk;
// every decision that could flip because of it is re-taken in FP64 by the
// caller (see eval_f32.cu).
#pragma once

#include <cmath>

#include "pf_device.cuh"

namespace pf {
namespace f32 {

__device__ __forceinline__ float ex2(float x) { return exp2f(x); }
__device__ __forceinline__ float lg2(float x) { return __log2f(x); }

// |x|^p for p > 0 (0 for x = 0)
__device__ __forceinline__ float powabs(float x, float p) { return ex2(p * lg2(fabsf(x))); }

// boxy radius: sqrt(x^2+y^2) or (|x|^B + |y|^B)^(1/B)
__device__ __forceinline__ float boxy_r(const ProfileDev &p, float x, float y)
{
	if (!p.fboxy) {
		return sqrtf(x * x + y * y);
	}
	const float B = p.fpar[FP_B], invB = p.fpar[FP_INVB];
	return ex2(invB * lg2(powabs(x, B) + powabs(y, B)));
}

__device__ __forceinline__ float evaluate_at(const ProfileDev &p, float x, float y)
{
	const float *c = p.fpar;
	switch (p.kind) {
	case PF_SERSIC: {
		float base, e;
		if (!p.fboxy) {
			base = (x * x + y * y) * c[FP_S_INV_RE2];  // (r/re)^2
			e = c[FP_S_HALF_INV_N];                     // 1 / (2 n)
		}
		else {
			base = powabs(x * c[FP_S_INV_RE], c[FP_B]) + powabs(y * c[FP_S_INV_RE], c[FP_B]);
			e = c[FP_S_INV_NB];                          // 1 / (n B)
		}
		const float rf = ex2(e * lg2(base));
		return ex2(c[FP_S_K] - c[FP_S_K] * rf);          // exp(-bn (rf - 1)), K = bn log2(e)
	}
	case PF_CORESERSIC: {
		const float r = boxy_r(p, x, y);
		const float a = c[FP_C_A];
		const float core = ex2(c[FP_C_B_OVER_A] * lg2(1.f + ex2(-a * lg2(r * c[FP_C_INV_RB]))));
		const float inner = (ex2(a * lg2(r)) + c[FP_C_RB_A]) * c[FP_C_INV_RE_A];
		return core * ex2(-c[FP_C_K] * ex2(c[FP_C_INV_NA] * lg2(inner)));
	}
	case PF_MOFFAT: {
		float r2;
		if (!p.fboxy) {
			r2 = (x * x + y * y) * c[FP_M_INV_RS2];
		}
		else {
			const float rf = boxy_r(p, x, y) * c[FP_M_INV_RS];
			r2 = rf * rf;
		}
		return ex2(-c[FP_M_CON] * lg2(1.f + r2));
	}
	case PF_FERRER: {
		// (1 - rf^(2-b))^a with 1 - rf^(2-b) = -expm1((2-b) ln rf): no cancellation near rf = 1
		const float rf = boxy_r(p, x, y) * c[FP_F_INV_ROUT];
		if (rf < 1.f) {
			return ex2(c[FP_F_A] * lg2(-expm1f(c[FP_F_2MB] * logf(rf))));
		}
		return 0.f;
	}
	case PF_KING: {
		// u^(-1/a) - ut^(-1/a) = temp * expm1(ln(ut/u) / a), ln(ut/u) = log1p((rt^2 - r^2) / (rc^2 u)),
		// with u = 1 + (r/rc)^2: accurate up to the truncation radius rt
		const float r = boxy_r(p, x, y);
		const float rt = c[FP_K_RT];
		if (r < rt) {
			const float q = r * c[FP_K_INV_RC];
			const float u = 1.f + q * q;
			const float w = (rt - r) * (rt + r) * (c[FP_K_INV_RC] * c[FP_K_INV_RC]) / u;
			const float diff = c[FP_K_TEMP] * expm1f(c[FP_K_INV_A] * log1pf(w));
			return ex2(c[FP_K_A] * lg2(diff));
		}
		return 0.f;
	}
	case PF_BROKENEXP: {
		const float r = boxy_r(p, x, y);
		float base = r - c[FP_E_RB];
		const float ab = c[FP_E_A] * base;
		if (ab < 40.f) {
			base = log1pf(__expf(ab)) * c[FP_E_INV_A];
		}
		return __expf(-r * c[FP_E_INV_H1] + c[FP_E_EXPO] * base);
	}
	}
	return 0.f;
}

}  // namespace f32
}  // namespace pf
