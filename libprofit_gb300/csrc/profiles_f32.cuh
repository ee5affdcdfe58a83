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
//
// Every multiply-add is written as fmaf, so that the rounding is the same in
// every kernel these are compiled into (eval_f32.cu is built without the
// compiler's own contraction: a batch and a single model, drawn by kernels
// built for different kinds, give the same bits).
//
// The kernels copy a profile's constants once into a Shape, held in
// registers, and evaluate through value<KINDS>(), where KINDS is the set of
// profile kinds the kernel is built for: a batch of sersic profiles only runs
// code without the other five kinds' branches.
#pragma once

#include <cmath>
#include <cstddef>

#include "pf_device.cuh"

namespace pf {
namespace f32 {

constexpr unsigned int kAllKinds = (1u << PF_SERSIC) | (1u << PF_CORESERSIC) | (1u << PF_MOFFAT) |
                                   (1u << PF_FERRER) | (1u << PF_KING) | (1u << PF_BROKENEXP);
constexpr unsigned int kSersicOnly = 1u << PF_SERSIC;

__device__ __forceinline__ float ex2(float x) { return exp2f(x); }
__device__ __forceinline__ float lg2(float x) { return __log2f(x); }

// |x|^p for p > 0 (0 for x = 0)
__device__ __forceinline__ float powabs(float x, float p) { return ex2(p * lg2(fabsf(x))); }

// One profile's single-precision constants, copied once into registers.
struct Shape {
	int kind, boxy;
	float c[12];           // ProfileDev::fpar, FP_* slots
	float cs, sn, iq;      // cos, sin of the position angle + 90 deg; 1 / axrat
	float acc;             // subsampling accuracy
	float bn, dbn;         // sersic bn and d bn / d nser (adjoint)
};

// The FP32 block of ProfileDev (fxc_hi .. fpar[11], 26 words from a 16-byte
// boundary) as seven float4 loads instead of word by word.
static_assert(offsetof(ProfileDev, fxc_hi) % 16 == 0 && sizeof(ProfileDev) % 16 == 0, "float4 block");
static_assert(offsetof(ProfileDev, fpar) == offsetof(ProfileDev, fxc_hi) + 14 * sizeof(float), "FP32 block layout");

__device__ __forceinline__ Shape load_shape(const ProfileDev &p)
{
	const float4 *v = reinterpret_cast<const float4 *>(&p.fxc_hi);
	const float4 a = v[1], b = v[2], c = v[3], d = v[4], e = v[5], f = v[6];
	Shape s;
	s.kind = p.kind;
	s.cs = a.x;
	s.sn = a.y;
	s.iq = a.z;
	s.acc = b.z;
	s.boxy = __float_as_int(c.y);
	s.c[0] = c.z;
	s.c[1] = c.w;
	s.c[2] = d.x;
	s.c[3] = d.y;
	s.c[4] = d.z;
	s.c[5] = d.w;
	s.c[6] = e.x;
	s.c[7] = e.y;
	s.c[8] = e.z;
	s.c[9] = e.w;
	s.c[10] = f.x;
	s.c[11] = f.y;
	s.bn = p.fbn;
	s.dbn = p.fdbn;
	return s;
}

// boxy radius: sqrt(x^2+y^2) or (|x|^B + |y|^B)^(1/B)
__device__ __forceinline__ float boxy_r(const Shape &s, float x, float y)
{
	if (!s.boxy) {
		return sqrtf(fmaf(x, x, y * y));
	}
	const float B = s.c[FP_B], invB = s.c[FP_INVB];
	return ex2(invB * lg2(powabs(x, B) + powabs(y, B)));
}

__device__ __forceinline__ float sersic(const Shape &s, float x, float y)
{
	const float *c = s.c;
	float base, e;
	if (!s.boxy) {
		base = fmaf(x, x, y * y) * c[FP_S_INV_RE2];  // (r/re)^2
		e = c[FP_S_HALF_INV_N];                     // 1 / (2 n)
	}
	else {
		base = powabs(x * c[FP_S_INV_RE], c[FP_B]) + powabs(y * c[FP_S_INV_RE], c[FP_B]);
		e = c[FP_S_INV_NB];                          // 1 / (n B)
	}
	const float rf = ex2(e * lg2(base));
	return ex2(fmaf(-c[FP_S_K], rf, c[FP_S_K]));     // exp(-bn (rf - 1)), K = bn log2(e)
}

__device__ __forceinline__ float coresersic(const Shape &s, float x, float y)
{
	const float *c = s.c;
	const float r = boxy_r(s, x, y);
	const float a = c[FP_C_A];
	const float core = ex2(c[FP_C_B_OVER_A] * lg2(1.f + ex2(-a * lg2(r * c[FP_C_INV_RB]))));
	const float inner = (ex2(a * lg2(r)) + c[FP_C_RB_A]) * c[FP_C_INV_RE_A];
	return core * ex2(-c[FP_C_K] * ex2(c[FP_C_INV_NA] * lg2(inner)));
}

__device__ __forceinline__ float moffat(const Shape &s, float x, float y)
{
	const float *c = s.c;
	float r2;
	if (!s.boxy) {
		r2 = fmaf(x, x, y * y) * c[FP_M_INV_RS2];
	}
	else {
		const float rf = boxy_r(s, x, y) * c[FP_M_INV_RS];
		r2 = rf * rf;
	}
	return ex2(-c[FP_M_CON] * lg2(1.f + r2));
}

__device__ __forceinline__ float ferrer(const Shape &s, float x, float y)
{
	// (1 - rf^(2-b))^a with 1 - rf^(2-b) = -expm1((2-b) ln rf): no cancellation near rf = 1
	const float *c = s.c;
	const float rf = boxy_r(s, x, y) * c[FP_F_INV_ROUT];
	if (rf < 1.f) {
		return ex2(c[FP_F_A] * lg2(-expm1f(c[FP_F_2MB] * logf(rf))));
	}
	return 0.f;
}

__device__ __forceinline__ float king(const Shape &s, float x, float y)
{
	// u^(-1/a) - ut^(-1/a) = temp * expm1(ln(ut/u) / a), ln(ut/u) = log1p((rt^2 - r^2) / (rc^2 u)),
	// with u = 1 + (r/rc)^2: accurate up to the truncation radius rt
	const float *c = s.c;
	const float r = boxy_r(s, x, y);
	const float rt = c[FP_K_RT];
	if (r < rt) {
		const float q = r * c[FP_K_INV_RC];
		const float u = fmaf(q, q, 1.f);
		const float w = (rt - r) * (rt + r) * (c[FP_K_INV_RC] * c[FP_K_INV_RC]) / u;
		const float diff = c[FP_K_TEMP] * expm1f(c[FP_K_INV_A] * log1pf(w));
		return ex2(c[FP_K_A] * lg2(diff));
	}
	return 0.f;
}

__device__ __forceinline__ float brokenexp(const Shape &s, float x, float y)
{
	const float *c = s.c;
	const float r = boxy_r(s, x, y);
	float base = r - c[FP_E_RB];
	const float ab = c[FP_E_A] * base;
	if (ab < 40.f) {
		base = log1pf(__expf(ab)) * c[FP_E_INV_A];
	}
	return __expf(fmaf(-r, c[FP_E_INV_H1], c[FP_E_EXPO] * base));
}

// The profile value at profile coordinates (x, y), for a kernel built for the
// profile kinds in KINDS.
template <unsigned int KINDS>
__device__ __forceinline__ float value(const Shape &s, float x, float y)
{
	if constexpr (KINDS == kSersicOnly) {
		return sersic(s, x, y);
	}
	else {
		switch (s.kind) {
		case PF_SERSIC: return sersic(s, x, y);
		case PF_CORESERSIC: return coresersic(s, x, y);
		case PF_MOFFAT: return moffat(s, x, y);
		case PF_FERRER: return ferrer(s, x, y);
		case PF_KING: return king(s, x, y);
		case PF_BROKENEXP: return brokenexp(s, x, y);
		}
		return 0.f;
	}
}

__device__ __forceinline__ float evaluate_at(const ProfileDev &p, float x, float y)
{
	return value<kAllKinds>(load_shape(p), x, y);
}

}  // namespace f32
}  // namespace pf
