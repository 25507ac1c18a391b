// Deterministic single-precision helpers for the detector's few
// transcendental steps (edge-line angle, probe directions, side lengths).
//
// Every function below is built only from IEEE-754 binary32 +, -, *, / and
// sqrt, evaluated in source order.  Those operations are correctly rounded
// on the GPU (nvcc's default -prec-div/-prec-sqrt, and this project builds
// its kernels with -fmad=false so nothing is fused) and on a CPU compiled
// with -ffp-contract=off, so the same inputs give the same bits on both.
// That is what lets the CUDA pipeline and the CPU oracle agree bit for bit
// on corners and decision margins.  Accuracy is about 1-2 ulp over the
// ranges the detector uses; tests/test_tables_and_math.py checks the error
// against libm.
//
// Methods (all from the mathematics, no vendor code):
//  * sin/cos: Cody & Waite additive range reduction by pi/2 (pi/2 split into
//    three floats, the first two with 12 significant bits so k*C is exact),
//    then the Taylor series of sin and cos on |r| <= pi/4 (terms to r^13 /
//    r^14, truncation error < 3e-13).
//  * atan2: octant reduction to t = min/max in [0, 1], the identity
//    atan(t) = pi/4 + atan((t - 1) / (t + 1)) for t > tan(pi/8), then the
//    Taylor series of atan on |z| <= tan(pi/8) to z^21 (error < 5e-10).
//    Signed zeros follow C99 Annex F (atan2(+-0, -0) = +-pi).
//  * hypot: sqrt(x*x + y*y); the detector's operands are pixel distances,
//    far from overflow or underflow.
#pragma once

#include <math.h>
#include <stdint.h>
#include <string.h>

#if defined(__CUDACC__)
#define BDM_FN __host__ __device__ __forceinline__
#else
#define BDM_FN static inline
#endif

namespace bdmath {

BDM_FN bool sign_bit(float x) {
    uint32_t u;
    memcpy(&u, &x, sizeof(u));
    return (u >> 31) != 0u;
}

BDM_FN float quiet_nan() {
    const uint32_t u = 0x7fc00000u;
    float f;
    memcpy(&f, &u, sizeof(f));
    return f;
}

#if defined(BDGB_CUDA_LIBM) && defined(__CUDA_ARCH__)
// The reference-arithmetic build (build.py, variant "refarith"): the
// kernels call CUDA's own sinf, cosf, atan2f and hypotf, as the reference's
// kernels do, and are compiled with multiply-add contraction on.  It exists
// to measure, on the GPU, how far the reference's rounding moves results
// from this project's default arithmetic; the oracle does not reproduce it.
BDM_FN void sincos(float x, float* s_out, float* c_out) {
    *s_out = ::sinf(x);
    *c_out = ::cosf(x);
}
BDM_FN float atan2(float y, float x) { return ::atan2f(y, x); }
BDM_FN float hypot(float x, float y) { return ::hypotf(x, y); }
#else
// sin and cos of x for |x| < 1000.
BDM_FN void sincos(float x, float* s_out, float* c_out) {
    const float kTwoOverPi = 0x1.45f306p-1f;
    const float kC1 = 0x1.92p+0f;       // pi/2, first 12 bits
    const float kC2 = 0x1.fb4p-12f;     // next 12 bits
    const float kC3 = 0x1.4442d2p-24f;  // remainder
    const float k = rintf(x * kTwoOverPi);
    float r = x - k * kC1;
    r = r - k * kC2;
    r = r - k * kC3;
    const float r2 = r * r;
    // sin(r) = r + r^3 * (-1/3! + r^2 (1/5! + r^2 (-1/7! + r^2 (1/9! + r^2 (-1/11! + r^2/13!)))))
    float ps = 1.6059043836821613e-10f;
    ps = ps * r2 + -2.5052108385441720e-08f;
    ps = ps * r2 + 2.7557319223985893e-06f;
    ps = ps * r2 + -1.9841269841269841e-04f;
    ps = ps * r2 + 8.3333333333333333e-03f;
    ps = ps * r2 + -1.6666666666666667e-01f;
    const float s = r + (r * r2) * ps;
    // cos(r) = 1 - r^2/2 + r^4 * (1/4! + r^2 (-1/6! + r^2 (1/8! + r^2 (-1/10! + r^2 (1/12! - r^2/14!)))))
    float pc = -1.1470745597729725e-11f;
    pc = pc * r2 + 2.0876756987868099e-09f;
    pc = pc * r2 + -2.7557319223985891e-07f;
    pc = pc * r2 + 2.4801587301587302e-05f;
    pc = pc * r2 + -1.3888888888888889e-03f;
    pc = pc * r2 + 4.1666666666666667e-02f;
    const float c = (1.0f - 0.5f * r2) + (r2 * r2) * pc;
    const int q = static_cast<int>(k) & 3;
    if (q == 0) {
        *s_out = s;
        *c_out = c;
    } else if (q == 1) {
        *s_out = c;
        *c_out = -s;
    } else if (q == 2) {
        *s_out = -s;
        *c_out = -c;
    } else {
        *s_out = -c;
        *c_out = s;
    }
}

BDM_FN float sin(float x) {
    float s, c;
    sincos(x, &s, &c);
    return s;
}

BDM_FN float cos(float x) {
    float s, c;
    sincos(x, &s, &c);
    return c;
}

BDM_FN float atan2(float y, float x) {
    const float kPi = 0x1.921fb6p+1f;
    const float kHalfPi = 0x1.921fb6p+0f;
    const float kQuarterPi = 0x1.921fb6p-1f;
    const float kTanPi8 = 0x1.a8279ap-2f;  // tan(pi/8) = sqrt(2) - 1
    const float ax = fabsf(x);
    const float ay = fabsf(y);
    if (ax == 0.0f && ay == 0.0f) {
        const float a = sign_bit(x) ? kPi : 0.0f;
        return sign_bit(y) ? -a : a;
    }
    const bool swap = ay > ax;
    const float num = swap ? ax : ay;
    const float den = swap ? ay : ax;
    float t = num / den;
    float base = 0.0f;
    if (t > kTanPi8) {
        t = (t - 1.0f) / (t + 1.0f);
        base = kQuarterPi;
    }
    const float t2 = t * t;
    // atan(t) = t + t^3 * (-1/3 + t^2 (1/5 + t^2 (-1/7 + ... + t^2 (1/21))))
    float p = 1.0f / 21.0f;
    p = p * t2 + -1.0f / 19.0f;
    p = p * t2 + 1.0f / 17.0f;
    p = p * t2 + -1.0f / 15.0f;
    p = p * t2 + 1.0f / 13.0f;
    p = p * t2 + -1.0f / 11.0f;
    p = p * t2 + 1.0f / 9.0f;
    p = p * t2 + -1.0f / 7.0f;
    p = p * t2 + 1.0f / 5.0f;
    p = p * t2 + -1.0f / 3.0f;
    float a = base + (t + (t * t2) * p);
    if (swap) a = kHalfPi - a;
    if (sign_bit(x)) a = kPi - a;
    return sign_bit(y) ? -a : a;
}

BDM_FN float hypot(float x, float y) { return sqrtf(x * x + y * y); }
#endif

}  // namespace bdmath
