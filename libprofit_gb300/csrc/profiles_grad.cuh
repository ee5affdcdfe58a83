// Adjoint of the coresersic, moffat, ferrer, king and brokenexp profiles:
// at one point of profile coordinates (xp, yp) the value f and the products
// f * d ln f / d theta for every parameter theta of the profile, in the slots
//   0 value, 1 xcen, 2 ycen, 3 ang, 4 axrat, 5 box, 6 + k  par[6 + k]
// (the sersic's own functions in adjoint.cu fill the first eight the same way).
//
// Each profile is written as ln f = g(r; shape) of the boxy radius
// r = (|xp|^B + |yp|^B)^(1/B), B = box + 2 (include/profit/radial.h:93-102),
// so the geometric parameters enter through G = r dg/dr only:
//   d ln f / d xp = G sgn(xp) |xp|^(B-1) / r^B,   likewise yp,
//   d ln f / d B  = G ((|xp|^B ln|xp| + |yp|^B ln|yp|) / (B r^B) - ln(r^B) / B^2),
// and (xp, yp) = R(ang + 90) (x - xcen, y - ycen) with yp divided by axrat
// (src/radial.cpp:201-217), the same chain as the sersic's.
// The profile forms (the reference's evaluate_at):
//   coresersic (1 + (r/rb)^-a)^(b/a) exp(-bn ((r^a + rb^a) / re^a)^(1/(n a)))
//              (src/coresersic.cpp:51-59)
//   moffat     (1 + (r/rs)^2)^-con, rs = fwhm / (2 sqrt(2^(1/con) - 1))
//              (src/moffat.cpp:52-58, 81-83)
//   ferrer     (1 - (r/rout)^(2-b))^a for r < rout (src/ferrer.cpp:50-60)
//   king       ((1 + (r/rc)^2)^(-1/a) - (1 + (rt/rc)^2)^(-1/a))^a for r < rt
//              (src/king.cpp:51-59)
//   brokenexp  exp(-r/h1 + (1/h1 - 1/h2) S), S = ln(1 + e^(a (r - rb))) / a, or
//              r - rb when a (r - rb) >= 40 (src/brokenexponential.cpp:38-94)
// The same code serves the FP64 (T = double) and FP32 (T = float) adjoints
// and compiles for the host, where its derivatives can be checked against
// finite differences of its own values.
#pragma once

#include <cmath>

#include "pf_device.cuh"

namespace pf {
namespace grad {

constexpr int kSlots = 12;

// single precision on the device: the special-function unit's exp2 / log2
// (a few 1e-7 relative, plus |x| eps for exp): the terms feed gradients
// checked at 1e-3, and the value used for decisions comes from
// profiles_f32.cuh, not from here
#ifdef __CUDA_ARCH__
__device__ inline float g_exp(float x) { return __expf(x); }
__device__ inline float g_log(float x) { return __logf(x); }
#else
inline float g_exp(float x) { return expf(x); }
inline float g_log(float x) { return logf(x); }
#endif
__host__ __device__ inline double g_exp(double x) { return exp(x); }
__host__ __device__ inline double g_log(double x) { return log(x); }
__host__ __device__ inline float g_log1p(float x) { return log1pf(x); }
__host__ __device__ inline double g_log1p(double x) { return log1p(x); }
__host__ __device__ inline float g_expm1(float x) { return expm1f(x); }
__host__ __device__ inline double g_expm1(double x) { return expm1(x); }
__host__ __device__ inline float g_sqrt(float x) { return sqrtf(x); }
__host__ __device__ inline double g_sqrt(double x) { return sqrt(x); }
__host__ __device__ inline float g_fabs(float x) { return fabsf(x); }
__host__ __device__ inline double g_fabs(double x) { return fabs(x); }
__host__ __device__ inline float g_copysign(float x, float y) { return copysignf(x, y); }
__host__ __device__ inline double g_copysign(double x, double y) { return copysign(x, y); }

// One profile's constants for the adjoint, in T.
template <typename T>
struct GShape {
	int kind;
	T B;             // box + 2
	T cs, sn, iq, q; // cos, sin of ang + 90 deg; 1 / axrat; axrat
	T p[5];          // par[6..10]
	T k[4];          // per kind: see make_gshape
};

// From a profile after the setup kernel (rscale, bn, dbn, cos_ang, sin_ang).
template <typename T>
__host__ __device__ inline GShape<T> make_gshape(const ProfileDev &P)
{
	GShape<T> s;
	s.kind = P.kind;
	s.B = (T)(P.par[PF_P_BOX] + 2);
	s.cs = (T)P.cos_ang;
	s.sn = (T)P.sin_ang;
	s.q = (T)P.par[PF_P_AXRAT];
	s.iq = (T)(1. / P.par[PF_P_AXRAT]);
	for (int i = 0; i < 5; i++) s.p[i] = (T)P.par[PF_P_X0 + i];
	for (int i = 0; i < 4; i++) s.k[i] = (T)0;
	switch (P.kind) {
	case PF_CORESERSIC:
		s.k[0] = (T)P.bn;
		s.k[1] = (T)P.dbn;
		s.k[2] = (T)log(P.par[6]);  // ln re
		s.k[3] = (T)log(P.par[8]);  // ln rb
		break;
	case PF_MOFFAT: {
		// d ln rs / d con = ln 2 2^(1/con) / (2 con^2 (2^(1/con) - 1))
		const double con = P.par[7], t = pow(2., 1. / con);
		s.k[0] = (T)(1. / P.rscale);
		s.k[1] = (T)(0.5 * log(2.) * t / (con * con * (t - 1.)));
		break;
	}
	case PF_FERRER:
		s.k[0] = (T)(1. / P.par[6]);
		break;
	case PF_KING: {
		const double rc = P.par[6], rt = P.par[7], a = P.par[8];
		const double ut = 1. + (rt / rc) * (rt / rc);
		s.k[0] = (T)ut;
		s.k[1] = (T)pow(ut, -1. / a);  // ut^(-1/a)
		s.k[2] = (T)(1. / (rc * rc));
		s.k[3] = (T)log(ut);
		break;
	}
	case PF_BROKENEXP:
		s.k[0] = (T)(1. / P.par[6] - 1. / P.par[7]);
		break;
	default:
		break;
	}
	return s;
}

// ln f and its derivatives for radius r: G = r d ln f / d r and d[k] =
// d ln f / d par[6 + k]. Returns false where f = 0 (outside the profile's
// support), leaving lnf, G and d unset.
template <typename T>
__host__ __device__ inline bool radial_terms(const GShape<T> &s, T r, T &lnf, T &G, T *d)
{
	switch (s.kind) {
	case PF_CORESERSIC: {
		const T n = s.p[1], rb = s.p[2], a = s.p[3], b = s.p[4];
		const T bn = s.k[0], dbn = s.k[1], lre = s.k[2], lrb = s.k[3];
		const T lr = g_log(r);
		const T P = g_exp(-a * (lr - lrb));            // (r/rb)^-a
		const T ra = g_exp(a * lr), rba = g_exp(a * lrb);
		const T sum = ra + rba;
		const T lQ = g_log(sum) - a * lre;               // ln((r^a + rb^a) / re^a)
		const T W = g_exp(lQ / (n * a));
		const T l1p = g_log1p(P);
		lnf = (b / a) * l1p - bn * W;
		const T fr = ra / sum, frb = rba / sum;
		G = -b * P / ((T)1 + P) - bn * W * fr / n;
		d[0] = bn * W / (n * s.p[0]);
		d[1] = -dbn * W + bn * W * lQ / (n * n * a);
		d[2] = b * P / (rb * ((T)1 + P)) - bn * W * frb / (rb * n);
		const T dT1 = -(b / (a * a)) * l1p + (b / a) * P * (lrb - lr) / ((T)1 + P);
		const T dlW = -lQ / (n * a * a) + (fr * lr + frb * lrb - lre) / (n * a);
		d[3] = dT1 - bn * W * dlW;
		d[4] = l1p / a;
		return true;
	}
	case PF_MOFFAT: {
		const T con = s.p[1];
		const T u = r * s.k[0];
		const T u2 = u * u;
		const T l1p = g_log1p(u2);
		lnf = -con * l1p;
		G = (T)-2 * con * u2 / ((T)1 + u2);
		d[0] = -G / s.p[0];
		d[1] = -l1p - G * s.k[1];
		return true;
	}
	case PF_FERRER: {
		const T a = s.p[1], b = s.p[2];
		const T v = r * s.k[0];
		if (!(v < (T)1)) return false;
		const T lv = g_log(v);
		const T w = v > (T)0 ? g_exp(((T)2 - b) * lv) : (T)0;  // v^(2-b)
		const T l1m = g_log1p(-w);
		lnf = a * l1m;
		const T iw = w / ((T)1 - w);
		G = -a * ((T)2 - b) * iw;
		d[0] = -G / s.p[0];
		d[1] = l1m;
		d[2] = v > (T)0 ? a * iw * lv : (T)0;
		return true;
	}
	case PF_KING: {
		const T rc = s.p[0], rt = s.p[1], a = s.p[2];
		if (!(r < rt)) return false;
		const T ut = s.k[0], uta = s.k[1], irc2 = s.k[2], lut = s.k[3];
		const T u = (T)1 + r * r * irc2;
		// D = u^(-1/a) - ut^(-1/a) = ut^(-1/a) expm1(ln(ut/u) / a), without cancellation
		const T lr = g_log1p((rt - r) * (rt + r) * irc2 / u);  // ln(ut / u)
		const T D = uta * g_expm1(lr / a);
		const T ua = D + uta;                                   // u^(-1/a)
		const T lD = g_log(D);
		lnf = a * lD;
		const T uia1 = ua / u, utia1 = uta / ut;                // u^(-1/a-1), ut^(-1/a-1)
		G = (T)-2 * r * r * irc2 * uia1 / D;
		d[0] = (T)2 * irc2 / rc * (r * r * uia1 - rt * rt * utia1) / D;
		d[1] = (T)2 * rt * irc2 * utia1 / D;
		d[2] = lD + (ua * g_log(u) - uta * lut) / (a * D);
		return true;
	}
	case PF_BROKENEXP: {
		const T h1 = s.p[0], h2 = s.p[1], rb = s.p[2], a = s.p[3];
		const T expo = s.k[0];
		const T dr = r - rb, ab = a * dr;
		T S, sig, dSa;
		if (ab < (T)40) {
			const T e = g_exp(ab);
			S = g_log1p(e) / a;
			sig = e / ((T)1 + e);
			dSa = (sig * dr - S) / a;
		}
		else {
			S = dr;
			sig = (T)1;
			dSa = (T)0;
		}
		lnf = -r / h1 + expo * S;
		G = r * (-(T)1 / h1 + expo * sig);
		d[0] = (r - S) / (h1 * h1);
		d[1] = S / (h2 * h2);
		d[2] = -expo * sig;
		d[3] = expo * dSa;
		return true;
	}
	default:
		return false;
	}
}

// t[0..11] = f and f * d ln f / d theta at profile coordinates (xp, yp).
// Returns f.
template <typename T>
__host__ __device__ inline T terms(const GShape<T> &s, T xp, T yp, T *t)
{
	for (int k = 0; k < kSlots; k++) t[k] = (T)0;
	const T ux = g_fabs(xp), uy = g_fabs(yp);
	const T B = s.B;
	T axm, aym;  // |x|^(B-1), |y|^(B-1)
	if (B == (T)2) {
		axm = ux;
		aym = uy;
	}
	else {
		axm = ux > (T)0 ? g_exp((B - (T)1) * g_log(ux)) : (T)0;
		aym = uy > (T)0 ? g_exp((B - (T)1) * g_log(uy)) : (T)0;
	}
	const T ax = axm * ux, ay = aym * uy;
	const T base = ax + ay;  // r^B
	const T r = B == (T)2 ? g_sqrt(base) : (base > (T)0 ? g_exp(g_log(base) / B) : (T)0);
	T lnf, G, d[5] = {0, 0, 0, 0, 0};
	if (!radial_terms(s, r, lnf, G, d)) return (T)0;
	const T f = g_exp(lnf);
	t[0] = f;
	if (base > (T)0) {
		const T ib = (T)1 / base;
		const T Dx = G * g_copysign(axm, xp) * ib;
		const T Dy = G * g_copysign(aym, yp) * ib;
		const T xl = ax > (T)0 ? ax * g_log(ux) : (T)0, yl = ay > (T)0 ? ay * g_log(uy) : (T)0;
		const T dB = G * ((xl + yl) * ib / B - g_log(base) / (B * B));
		const T deg = (T)(3.14159265358979323846 / 180.0);
		t[1] = f * (-s.cs * Dx + s.sn * s.iq * Dy);
		t[2] = f * (-s.sn * Dx - s.cs * s.iq * Dy);
		t[3] = f * deg * (s.q * yp * Dx - xp * s.iq * Dy);
		t[4] = f * (-(yp * s.iq) * Dy);
		t[5] = f * dB;
	}
	for (int k = 0; k < 5; k++) t[6 + k] = f * d[k];
	return f;
}

}  // namespace grad
}  // namespace pf
