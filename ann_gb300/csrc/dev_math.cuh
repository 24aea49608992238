// Device math for the two precisions.
//  double: the reference's own special functions (math/special.cpp) restated with explicit
//          round-to-nearest operations (no contraction), so that the FP64 pipeline follows the
//          reference's arithmetic: fmexp (Pade exp2, special.cpp:236-285), coscut/sincut (Taylor
//          series about pi/2, special.cpp:22-42).
//  float : hardware fast paths (ex2.approx via __expf, MUFU sin/cos) for the mixed pipeline.
#pragma once
#include <cuda_runtime.h>
#include <cstdint>
#include "plan.hpp"
#include "potential.hpp"

namespace ann {

constexpr double kPI = 3.141592653589793;   // math/const.hpp:10
constexpr double kRad2 = 1.414213562373095; // math/const.hpp:12
constexpr double kLOG2 = 0.693147180559945; // math/const.hpp:16

// ------------------------------------------------------------------ FP64 reference special functions
__device__ __forceinline__ double d_exp2_pade(double x) {
    const double P0 = 2.30933477057345225087e-2, P1 = 2.02020656693165307700e1, P2 = 1.51390680115615096133e3;
    const double Q0 = 2.33184211722314911771e2, Q1 = 4.36821166879210612817e3;
    const double ip = floor(__dadd_rn(x, 0.5));
    const double fp = __dsub_rn(x, ip);
    const double scale = __hiloint2double((((int)ip) + 1023) << 20, 0);
    const double x2 = __dmul_rn(fp, fp);
    double px = P0;
    px = __dadd_rn(__dmul_rn(px, x2), P1);
    double qx = __dadd_rn(x2, Q0);
    px = __dadd_rn(__dmul_rn(px, x2), P2);
    qx = __dadd_rn(__dmul_rn(qx, x2), Q1);
    px = __dmul_rn(px, fp);
    return __dmul_rn(scale, __dadd_rn(1.0, __dmul_rn(2.0, __ddiv_rn(px, __dsub_rn(qx, px)))));
}
__device__ __forceinline__ double d_fmexp(double x) {
    const double LOG2E = 1.4426950408889634074;
    if (x < -1022.0 / LOG2E) return 0.0;
    if (x > 1023.0 / LOG2E) return __longlong_as_double(0x7ff0000000000000ULL);
    return d_exp2_pade(__dmul_rn(LOG2E, x));
}
__device__ __forceinline__ double d_coscut(double x) {
    x = __dsub_rn(x, 0.5 * kPI);
    const double x2 = __dmul_rn(x, x);
    double p = 1.0 / 1307674368000.0;
    p = __dadd_rn(-1.0 / 6227020800.0, __dmul_rn(x2, p));
    p = __dadd_rn(1.0 / 39916800.0, __dmul_rn(x2, p));
    p = __dadd_rn(-1.0 / 362880.0, __dmul_rn(x2, p));
    p = __dadd_rn(1.0 / 5040.0, __dmul_rn(x2, p));
    p = __dadd_rn(-1.0 / 120.0, __dmul_rn(x2, p));
    p = __dadd_rn(1.0 / 6.0, __dmul_rn(x2, p));
    p = __dadd_rn(-1.0, __dmul_rn(x2, p));
    return __dmul_rn(x, p);
}
__device__ __forceinline__ double d_sincut(double x) {
    x = __dsub_rn(x, 0.5 * kPI);
    const double x2 = __dmul_rn(x, x);
    double p = 1.0 / 20922789888000.0;
    p = __dadd_rn(-1.0 / 87178291200.0, __dmul_rn(x2, p));
    p = __dadd_rn(1.0 / 479001600.0, __dmul_rn(x2, p));
    p = __dadd_rn(-1.0 / 3628800.0, __dmul_rn(x2, p));
    p = __dadd_rn(1.0 / 40320.0, __dmul_rn(x2, p));
    p = __dadd_rn(-1.0 / 720.0, __dmul_rn(x2, p));
    p = __dadd_rn(1.0 / 24.0, __dmul_rn(x2, p));
    p = __dadd_rn(-1.0 / 2.0, __dmul_rn(x2, p));
    return __dadd_rn(1.0, __dmul_rn(x2, p));
}

// ------------------------------------------------------------------ precision traits
template <typename real> struct M;
template <> struct M<double> {
    static __device__ __forceinline__ double bexp(double x) { return d_fmexp(x); }      // basis exp = fmexp
    static __device__ __forceinline__ double exp(double x) { return ::exp(x); }         // std::exp (activations)
    static __device__ __forceinline__ double pow(double x, double y) { return ::pow(x, y); }
    static __device__ __forceinline__ double tanh(double x) { return ::tanh(x); }
    static __device__ __forceinline__ double log1p(double x) { return ::log1p(x); }
    static __device__ __forceinline__ double sqrt(double x) { return ::sqrt(x); }
    static __device__ __forceinline__ double log(double x) { return ::log(x); }
    static __device__ __forceinline__ double atan(double x) { return ::atan(x); }
    static __device__ __forceinline__ double erf(double x) { return ::erf(x); }
    static __device__ __forceinline__ double rcp(double x) { return 1.0 / x; }
    static __device__ __forceinline__ double coscut(double x) { return d_coscut(x); }   // ~cos(x), x in [0,pi]
    static __device__ __forceinline__ double sincut(double x) { return d_sincut(x); }
};
template <> struct M<float> {
    static __device__ __forceinline__ float bexp(float x) { return __expf(x); }
    static __device__ __forceinline__ float exp(float x) { return __expf(x); }
    // x >= 0 here; pow(x, 0) = 1 also for x = 0 (as std::pow), where exp2(0 * log2(0)) is NaN
    static __device__ __forceinline__ float pow(float x, float y) { return (y == 0.0f) ? 1.0f : __powf(x, y); }
    static __device__ __forceinline__ float tanh(float x) { return ::tanhf(x); }
    static __device__ __forceinline__ float log1p(float x) { return ::log1pf(x); }
    static __device__ __forceinline__ float sqrt(float x) { return ::sqrtf(x); }
    static __device__ __forceinline__ float log(float x) { return ::logf(x); }
    static __device__ __forceinline__ float atan(float x) { return ::atanf(x); }
    static __device__ __forceinline__ float erf(float x) { return ::erff(x); }
    static __device__ __forceinline__ float rcp(float x) { return __frcp_rn(x); }
    static __device__ __forceinline__ float coscut(float x) { return __cosf(x); }
    static __device__ __forceinline__ float sincut(float x) { return __sinf(x); }
};

template <typename real> struct V4;
template <> struct V4<float> { typedef Vec4f T; };
template <> struct V4<double> { typedef Vec4d T; };

// ------------------------------------------------------------------ cutoff (nnp/cutoff.cpp:62-156)
template <typename real>
__device__ __forceinline__ void cutoff_fg(int name, real rc, real dr, real& f, real& g) {
    f = real(0); g = real(0);
    if (!(dr < rc)) return;
    switch (name) {
        case CUT_STEP: f = real(1); g = real(0); return;
        case CUT_COS: {
            const real pirci = real(kPI) / rc;
            const real arg = dr * pirci;
            f = real(0.5) * (M<real>::coscut(arg) + real(1));
            g = real(-0.5) * pirci * M<real>::sincut(arg);
            return;
        }
        case CUT_TANH: {
            const real rci = real(1) / rc;
            const real t = M<real>::tanh(real(1) - dr * rci);
            f = t * t * t;
            g = real(-3) * t * t * (real(1) - t * t) * rci;
            return;
        }
        case CUT_POLY3: {
            const real rci = real(1) / rc;
            const real x = dr * rci;
            f = (real(2) * x - real(3)) * x * x + real(1);
            g = real(6) * x * (x - real(1)) * rci;
            return;
        }
        default: return;
    }
}

// ------------------------------------------------------------------ radial functions (basis_radial.cpp:263-376)
// value and derivative d/dr of one radial function times the cutoff
template <typename real>
__device__ __forceinline__ void radial_vd(int name, real eta, real rs, real dr, real fc, real fcg, real& val, real& der) {
    switch (name) {
        case R_GAUSSIAN: {
            const real a = eta * (dr - rs);
            const real e = M<real>::bexp(-a * a);
            val = e * fc;
            der = e * (real(-2) * eta * a * fc + fcg);
            return;
        }
        case R_SECH: {
            const real e = M<real>::bexp(-eta * (dr - rs));
            const real e2 = e * e;
            const real den = real(1) / (real(1) + e2);
            val = real(2) * e * den * fc;
            der = real(2) * e * den * (-eta * (real(1) - e2) * den * fc + fcg);
            return;
        }
        case R_LOGISTIC: {
            const real e = M<real>::bexp(real(-2) * eta * (dr - rs));
            const real den = real(1) / (real(1) + e);
            const real th = (real(1) - e) * den;
            const real s2 = real(4) * e * den * den;
            val = s2 * fc;
            der = s2 * (real(-2) * eta * th * fc + fcg);
            return;
        }
        case R_TANH: {
            const real th = M<real>::tanh(-eta * (dr - rs));
            val = real(0.5) * (th + real(1)) * fc;
            der = real(0.5) * (-eta * (real(1) - th * th) * fc + (real(1) + th) * fcg);
            return;
        }
        case R_LOGCOSH: {
            const real e = M<real>::bexp(real(-2) * eta * (dr - rs));
            const real l = real(0.5) * M<real>::log1p(e);
            val = l * fc;
            der = -eta * e / (real(1) + e) * fc + l * fcg;
            return;
        }
        case R_LOGCOSH2: {
            const real a = -eta * (dr - rs);
            const real e = M<real>::bexp(real(2) * real(kRad2) * a);
            if (a == real(0)) {
                val = real(0.5) * fc / real(kRad2);
                der = real(0.5) * (-eta * fcg + fc / real(kRad2));
            } else {
                const real den = real(1) / (e - real(1));
                val = a * e * den * fc;
                der = e * (eta * (real(1) + real(2) * real(kRad2) * a - e) * den * fc + a * fcg) * den;
            }
            return;
        }
        default: val = real(0); der = real(0); return;
    }
}

// radial_vd with the form fixed at compile time when it is GAUSSIAN (NAME = R_GAUSSIAN), so that
// unrolled loops over a block's functions carry no per-function dispatch; NAME = -1: any form
template <int NAME, typename real>
__device__ __forceinline__ void radial_vd_t(int name, real eta, real rs, real dr, real fc, real fcg, real& val, real& der) {
    if (NAME == R_GAUSSIAN) {
        const real a = eta * (dr - rs);
        const real e = M<real>::bexp(-a * a);
        val = e * fc;
        der = e * (real(-2) * eta * a * fc + fcg);
    } else {
        radial_vd<real>(name, eta, rs, dr, fc, fcg, val, der);
    }
}

// ------------------------------------------------------------------ angular damping of the generic path
// returns the radial damping value h(r2s) of one angular function and dh/dr2s-based factors
// following basis_angular.cpp:212-364: value part multiplies |1/2+lambda/2 cos|^zeta * fc_j fc_k,
// dq = coefficient such that dG/drij = fa * (-dq * 2 rij fc_j + g_j) * fc_k  (see angular_generic)
template <typename real>
__device__ __forceinline__ void angular_damp(int name, real ie2, real r2s, real& h, real& dq) {
    switch (name) {
        case A_GAUSS: h = M<real>::bexp(-ie2 * r2s); dq = ie2; return;
        case A_GAUSS2: {
            const real e = M<real>::bexp(real(-0.5) * real(kPI) * ie2 * r2s);
            const real den = real(1) / (real(1) + e);
            h = real(2) * e * den; dq = real(0.5) * real(kPI) * ie2 * den; return;
        }
        case A_SECH: {
            const real e = M<real>::bexp(real(-0.5) * real(kPI) * ie2 * r2s);
            const real e2 = e * e;
            const real den = real(1) / (real(1) + e2);
            h = real(2) * e * den; dq = real(0.5) * real(kPI) * ie2 * (real(1) - e2) * den; return;
        }
        default: {  // STUDENT3/4/5: powint(1/sqrt(1+ie2 r2s), p), p = 4/5/6
            const int p = (name == A_STUDENT3) ? 4 : (name == A_STUDENT4) ? 5 : 6;
            const real den = real(1) / M<real>::sqrt(real(1) + ie2 * r2s);
            const real d2 = den * den;
            real hv = d2 * d2;
            if (p >= 5) hv *= den;
            if (p >= 6) hv *= den;
            h = hv; dq = real(p) * real(0.5) * ie2 * d2; return;
        }
    }
}

// activation value, first and second derivative: a and d follow AFFPBP::af_* (nn.cpp:149-810),
// d2 is the exact derivative of d (where AFFPBP2 sets 0 or an inexact form, nn.cpp:282-812); the
// same formulas as the oracle's activate()
template <typename real>
__device__ __forceinline__ void act_fd(int neuron, real c, real z, real& a, real& d, real& d2) {
    const real PI = real(3.141592653589793), RADPI = real(1.772453850905516), one = real(1), two = real(2), half = real(0.5);
    switch (neuron) {
        case N_SIGMOID: {
            if (z >= real(0)) { const real e = M<real>::exp(-c * z); const real f = one / (one + e); a = f; d = c * e * f * f; d2 = -c * c * e * (one - e) * f * f * f; }
            else { const real e = M<real>::exp(c * z); const real f = one / (one + e); a = e * f; d = c * e * f * f; d2 = -c * c * e * (e - one) * f * f * f; }
            return;
        }
        case N_TANH: { const real t = M<real>::tanh(c * z); a = t; d = c * (one - t * t); d2 = c * c * (-two * t * (one - t * t)); return; }
        case N_ISRU: {
            const real zz = c * z, isr = one / M<real>::sqrt(one + zz * zz), isr3 = isr * isr * isr;
            if (zz < real(-100)) a = -one / (one + one / (zz * zz));
            else if (zz > real(100)) a = one / (one + one / (zz * zz));
            else a = zz * isr;
            d = c * isr3; d2 = real(-3) * c * c * zz * isr3 * isr * isr;
            return;
        }
        case N_ARCTAN: {
            const real zz = c * z * PI / two, fr = one / (one + zz * zz);
            a = (two / PI) * M<real>::atan(zz); d = c * fr; d2 = -PI * c * c * zz * fr * fr;
            return;
        }
        case N_RELU: if (z > real(0)) { a = z; d = one; } else { a = real(0); d = real(0); } d2 = real(0); return;
        case N_ELU: {
            if (z >= real(0)) { a = z; d = one; d2 = real(0); }
            else { const real e = M<real>::exp(c * z); a = e - one; d = c * e; d2 = c * c * e; }
            return;
        }
        case N_TANHRE: {
            if (z >= real(0)) { a = z; d = one; d2 = real(0); }
            else { const real fe = M<real>::exp(two * c * z); a = (fe - one) / (fe + one); d = c * (one - a * a); d2 = -two * c * a * d; }
            return;
        }
        case N_SQRE: {
            if (z >= real(0)) { a = z; d = one; d2 = real(0); }
            else { const real den = one / M<real>::sqrt(one + z * z), den3 = den * den * den; a = z * den; d = den3; d2 = real(-3) * z * den3 * den * den; }
            return;
        }
        case N_SWISH: {
            const real zz = c * z;
            if (zz > real(0)) {
                const real e = M<real>::exp(-zz), den = one / (one + e);
                a = z * den; d = (one + e * (one + zz)) * den * den; d2 = c * e * (two - zz + e * (two + zz)) * den * den * den;
            } else {
                const real e = M<real>::exp(zz), den = one / (one + e);
                a = z * e * den; d = e * (one + zz + e) * den * den; d2 = c * e * (two + zz + e * (two - zz)) * den * den * den;
            }
            return;
        }
        case N_GELU: {
            const real zz = half * RADPI * c * z, erfp1 = one + M<real>::erf(zz), g = M<real>::exp(-zz * zz);
            a = half * z * erfp1; d = half * (erfp1 + c * z * g); d2 = c * g * (one - zz * zz);
            return;
        }
        case N_MISH: {
            const real zz = c * z;
            if (zz > real(0)) {
                const real e = M<real>::exp(-zz), e2 = e * e, den = one / ((one + e) * (one + e) + e2);
                a = z * (one - two * e2 * den);
                d = one - two * e2 * den * (one - two * zz * (one + e) * den);
                const real t1 = real(4) * e2 * (one + e) * den * den;
                const real t2 = real(4) * e2 * den * den * den * (-two - real(3) * e + two * e2 + two * e2 * e);
                d2 = c * (two * t1 + zz * t2);
            } else {
                const real e = M<real>::exp(zz), den = one / (e * (e + two) + two);
                a = z * e * (e + two) * den;
                d = one + two * den * (-one + two * zz * (one - (e + two) * den));
                const real t1 = real(4) * e * (e + one) * den * den;
                const real t2 = real(4) * den * den * den * e * (two + two * e - real(3) * e * e - two * e * e * e);
                d2 = c * (two * t1 + zz * t2);
            }
            return;
        }
        case N_PFLU: {
            const real zz = c * z, z2 = zz * zz, fs = one / M<real>::sqrt(z2 + one), fs3 = fs * fs * fs;
            a = half * z * (one + zz * fs); d = half * (zz * (z2 + two) * fs3 + one); d2 = -half * c * (z2 - two) * fs3 * fs * fs;
            return;
        }
        case N_SERF: {
            const real fe = M<real>::exp(z), fl = M<real>::log1p(fe), ef = M<real>::erf(fl), g = M<real>::exp(-fl * fl), sg = one / (one + one / fe);
            a = z * ef; d = ef + two / RADPI * g * z * sg; d2 = two / RADPI * g * sg * (two - two * z * fl * sg + z * (one - sg));
            return;
        }
        case N_LOGISH: {
            const real l2i = one / real(kLOG2), e = M<real>::exp(-z), lf = M<real>::log(one + one / (one + e));
            const real q = e / ((one + e) * (two + e)), qp = e * (e * e - two) / ((one + e) * (one + e) * (two + e) * (two + e));
            a = l2i * z * lf; d = l2i * (lf + z * q); d2 = l2i * (two * q + z * qp);
            return;
        }
        case N_SOFTPLUS: {
            const real ci = one / c;
            if (z > real(0)) { const real e = M<real>::exp(-c * z); const real den = one / (e + one); a = z + ci * (M<real>::log1p(e) - real(kLOG2)); d = den; d2 = c * e * den * den; }
            else { const real e = M<real>::exp(c * z); const real den = one / (e + one); a = ci * (M<real>::log1p(e) - real(kLOG2)); d = e * den; d2 = c * e * den * den; }
            return;
        }
        case N_SQPLUS: {
            const real zz = c * z, fs = M<real>::sqrt(one + zz * zz);
            a = half / c * (zz - one + fs); d = half * (zz / fs + one); d2 = half * c / (fs * fs * fs);
            return;
        }
        case N_ATISH: {
            const real zz = half * PI * z, fr = one / (one + zz * zz), at = M<real>::atan(zz);
            a = z * half * (one + two / PI * at); d = half * (one + z * fr) + at / PI; d2 = fr * fr;
            return;
        }
        case N_TEST: {
            const real zz = c * z, z2 = zz * zz, z4 = z2 * z2, den = one / M<real>::sqrt(M<real>::sqrt(z4 + one));
            const real den4 = den * den * den * den;
            a = half * z * (one + zz * den); d = half * (zz * den * (one + one / (z4 + one)) + one);
            d2 = half * c * (den + (one - z4) * den * den4 - real(5) * z4 * den * den4 * den4);
            return;
        }
        default: a = z; d = one; d2 = real(0); return;  // LINEAR
    }
}

}  // namespace ann
