// FP64 device physics of the P3T step: cutoff functions, sun force, Hermite
// predictor/corrector and time-step criteria.  Every expression keeps the
// operand order of the reference formula it restates (file:line beside it);
// the translation units that include this header are compiled with
// -fmad=false, so products and sums round separately as in GPLUM's build and
// only the transcendental functions (log, sin, cos, atan2, pow, exp) can
// differ in the last bit from the host C library.
#pragma once
#include <cuda_runtime.h>

#include "p3t_state.cuh"

namespace p3t {

struct V3 {
    double x, y, z;
};
__device__ __forceinline__ V3 v3(double a, double b, double c) { return V3{a, b, c}; }
__device__ __forceinline__ V3 operator+(V3 a, V3 b) { return v3(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ V3 operator-(V3 a, V3 b) { return v3(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ V3 operator*(double s, V3 a) { return v3(s * a.x, s * a.y, s * a.z); }
__device__ __forceinline__ V3 operator*(V3 a, double s) { return v3(a.x * s, a.y * s, a.z * s); }
__device__ __forceinline__ V3 operator/(V3 a, double s) { return v3(a.x / s, a.y / s, a.z / s); }
__device__ __forceinline__ double dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ void addto(V3 &a, V3 b) { a.x += b.x; a.y += b.y; a.z += b.z; }
__device__ __forceinline__ void subfrom(V3 &a, V3 b) { a.x -= b.x; a.y -= b.y; a.z -= b.z; }
__device__ __forceinline__ V3 ld3(const double *p, int i) { return v3(p[3 * i], p[3 * i + 1], p[3 * i + 2]); }
__device__ __forceinline__ void st3(double *p, int i, V3 v) {
    p[3 * i] = v.x;
    p[3 * i + 1] = v.y;
    p[3 * i + 2] = v.z;
}
// std::min / std::max semantics
__device__ __forceinline__ double dmin(double a, double b) { return (b < a) ? b : a; }
__device__ __forceinline__ double dmax(double a, double b) { return (a < b) ? b : a; }

// ---- cutoff functions, src/cutfunc.h:4-66 ----------------------------------
__device__ __forceinline__ double cut_f(const Params &P, double y) {
    const double g = P.gamma, g2 = g * g;
    return (((((((-10. / 3. * y + 14. * (g + 1.)) * y - 21. * ((g + 3.) * g + 1.)) * y +
                35. / 3. * (((g + 9.) * g + 9.) * g + 1.)) * y - 70. * ((g + 3.) * g + 1.) * g) * y +
              210. * (g + 1.) * g2) * y - 140. * g2 * g * log(y)) * y +
            (((g - 7.) * g + 21.) * g - 35.) * g2 * g2) * P.g_1_inv7;
}
__device__ __forceinline__ double cut_W(const Params &P, double rij, double r_out_inv) {
    const double y = rij * r_out_inv;
    if (1.0 <= y) return 1.0;
    if (y <= P.gamma) return y * P.w_y;
    return cut_f(P, y) + y * (1. - P.f1);
}
__device__ __forceinline__ double cut_Kx(double x) {
    if (x < 0.) return 0.;
    if (x >= 1.) return 1.;
    const double x2 = x * x;
    return (((-20. * x + 70.) * x - 84.) * x + 35.) * x2 * x2;
}
__device__ __forceinline__ double cut_K(const Params &P, double rij, double r_out_inv) {
    return cut_Kx((P.gamma - rij * r_out_inv) * P.g_1_inv);
}
__device__ __forceinline__ double cut_dKdt(const Params &P, double rij, double r_out_inv, double alpha) {
    const double x = (P.gamma - rij * r_out_inv) * P.g_1_inv;
    const double x_1 = x - 1.;
    const double dKdr = (x < 0. || x >= 1.) ? 0. : (140. * x * x * x * x_1 * x_1 * x_1 * r_out_inv * P.g_1_inv);
    return alpha * rij * dKdr;
}

// ---- sun, src/gravity_hard.h:5-111 ---------------------------------------------
__device__ __forceinline__ void sun_force(const Params &P, V3 x, V3 v, V3 &acc_s, V3 &jerk_s, double *phi_s) {
    const V3 dr = v3(-x.x, -x.y, -x.z), dv = v3(-v.x, -v.y, -v.z);
    const double r2inv = 1. / (dot(dr, dr) + P.eps2_sun);
    const double rinv = sqrt(r2inv);
    const double r3inv = rinv * r2inv;
    const double mr3 = P.m_sun * r3inv;
    const double alpha = dot(dr, dv) * r2inv;
    if (phi_s) *phi_s = -P.m_sun * rinv;
    acc_s = mr3 * dr;
    jerk_s = mr3 * (dv - 3. * alpha * dr);
}

// ---- time-step criteria, src/particle.h:345-383 --------------------------------
__device__ __forceinline__ double dt2nd(double eta, double alpha2, double acc0, V3 acc, V3 jerk) {
    const double Acc2 = dot(acc, acc) + alpha2 * acc0 * acc0;
    const double Jerk2 = dot(jerk, jerk);
    return (Jerk2 > 0.) ? eta * sqrt(Acc2 / Jerk2) : 1.7976931348623157e308;
}
__device__ __forceinline__ double dt4th(double eta, double alpha2, double acc0, V3 acc, V3 jerk, V3 snap, V3 crac) {
    const double Acc = sqrt(dot(acc, acc) + alpha2 * acc0 * acc0);
    const double Jerk2 = dot(jerk, jerk);
    const double Jerk = sqrt(Jerk2);
    const double Snap2 = dot(snap, snap);
    const double Snap = sqrt(Snap2);
    const double Crac = sqrt(dot(crac, crac));
    return (Jerk > 0.) ? eta * sqrt((Acc * Snap + Jerk2) / (Jerk * Crac + Snap2)) : 1.7976931348623157e308;
}

// 1 / x, the same double as the IEEE quotient: by the exponent alone when x
// is a power of two (a block step's length; its reciprocal is exact), else
// by the division
__device__ __forceinline__ double recip_pow2_or_div(double x) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const unsigned e = (unsigned)((b >> 52) & 0x7ff);
    if ((b & 0x800fffffffffffffULL) == 0ULL && e != 0 && e < 0x7fe)
        return __longlong_as_double((long long)(0x7FE0000000000000ULL - b));
    return 1. / x;
}

// fmod(t, d) for the time-step quantisation.  d is a power of two there
// (dt_tree, dt_min and every halving of them); then t - floor(t/d)*d is
// computed exactly (scaling by a power of two, floor and the product are
// exact, and the difference is representable), which is the exact value
// IEEE fmod returns for t >= 0.  Any other d takes the library fmod.
__device__ __forceinline__ double rem_pow2(double t, double d) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(d);
    const unsigned e = (unsigned)((b >> 52) & 0x7ff);
    const bool pow2 = d > 0. && (b & 0x000fffffffffffffULL) == 0ULL && e != 0 && e < 0x7fe;
    if (!pow2 || !(t >= 0.) || t >= 1e300) return fmod(t, d);
    // t / d as t times 1/d: for d = 2^k (normal, k < 1023) the reciprocal
    // 2^-k is exact (its biased exponent is 2046 minus d's), and so is the
    // product -- the same double as the quotient, without a division
    const double rd = __longlong_as_double((long long)(0x7FE0000000000000ULL - b));
    return t - floor(t * rd) * d;
}

// FPGrav::calcDeltatInitial, src/particle.h:886-914.  The fmod loops are
// bounded (time and dt are commensurate powers of two within 64 halvings).
__device__ __forceinline__ double dt_initial(const Params &P, double time, double dt_old, double acc0, V3 acc_d,
                                             V3 jerk_d, V3 acc_s, V3 jerk_s) {
    double dt_next = 0.5 * P.dt_tree;
    const double dt_1 = dmin(dt2nd(P.eta_0, P.alpha2, acc0, acc_d, jerk_d), dt2nd(P.eta_sun0, P.alpha2, 0., acc_s, jerk_s));
    double rem = rem_pow2(time, dt_next);
    for (int k = 0; rem != 0.0 && k < 1100; k++) {
        dt_next *= 0.5;
        rem = rem_pow2(time, dt_next);
    }
    if (dt_old > 0.)
        for (int k = 0; 2. * dt_old < dt_next && k < 1100; k++) dt_next *= 0.5;
    for (int k = 0; dt_1 < dt_next && k < 1100; k++) dt_next *= 0.5;
    if (dt_next < 2. * P.dt_min) dt_next = P.dt_min;
    return dt_next;
}

}  // namespace p3t
