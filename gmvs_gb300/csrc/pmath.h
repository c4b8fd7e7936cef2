// Portable elementary functions for the PatchMatch arithmetic.
//
// The CUDA kernels and the CPU oracle both use these so that they round
// identically: the functions use only IEEE-754 add, subtract, multiply,
// divide, square root and fused multiply-add, which round the same on every
// conforming host and device.  Accuracy (tested against the C library):
// pm_expf within 2 ulp, pm_sinf / pm_cosf within 2 ulp on |a| <= 1 (their
// domain here: perturbation angles below 0.1 rad), pm_acosf within 4 ulp.
//
//  exp:  Cody-Waite reduction x = k ln2 + r, |r| <= ln2/2 (ln2 split into a
//        16-bit head and a tail), exp(r) by its degree-7 Taylor polynomial,
//        scaled by 2^k.
//  sin/cos: Taylor polynomials of degree 11 / 10.
//  acos: pi/2 - asin(x) for |x| <= 1/2, else 2 asin(sqrt((1 -/+ x) / 2)),
//        asin by its Taylor series to degree 27.
#pragma once

#include <stdint.h>
#include <string.h>

#if defined(__CUDACC__)
#define PM_HD __host__ __device__ __forceinline__
#else
#define PM_HD inline
#include <cmath>
#endif

namespace pmath {

PM_HD float fma_(float a, float b, float c) {
#if defined(__CUDA_ARCH__)
    return __fmaf_rn(a, b, c);
#else
    return std::fma(a, b, c);
#endif
}

PM_HD float rint_(float x) {
#if defined(__CUDA_ARCH__)
    return rintf(x);
#else
    return std::nearbyint(x);
#endif
}

PM_HD float sqrt_(float x) {
#if defined(__CUDA_ARCH__)
    return __fsqrt_rn(x);
#else
    return std::sqrt(x);
#endif
}

PM_HD float bits_to_float(uint32_t u) {
#if defined(__CUDA_ARCH__)
    return __uint_as_float(u);
#else
    float f;
    memcpy(&f, &u, 4);
    return f;
#endif
}

// 2^k for k in [-126, 127]
PM_HD float pow2i(int k) { return bits_to_float((uint32_t)(k + 127) << 23); }

PM_HD float expf_(float x) {
    if (x != x) return x;
    if (x > 88.7228394f) return bits_to_float(0x7f800000u);
    if (x < -103.972084f) return 0.0f;
    const float k = rint_(x * 1.44269504f);
    float r = fma_(-k, 0.693145751953125f, x);
    r = fma_(-k, 1.42860677e-06f, r);
    float p = 1.98412698e-04f;  // 1/7!
    p = fma_(p, r, 1.38888889e-03f);  // 1/6!
    p = fma_(p, r, 8.33333333e-03f);  // 1/5!
    p = fma_(p, r, 4.16666667e-02f);  // 1/4!
    p = fma_(p, r, 1.66666667e-01f);  // 1/3!
    p = fma_(p, r, 0.5f);
    p = fma_(p, r, 1.0f);
    p = fma_(p, r, 1.0f);
    const int ki = (int)k;
    if (ki > 127) return (p * pow2i(127)) * 2.0f;
    if (ki < -126) return (p * pow2i(ki + 64)) * pow2i(-64);
    return p * pow2i(ki);
}

PM_HD float sinf_(float a) {
    const float a2 = a * a;
    float p = -2.50521084e-08f;               // -1/11!
    p = fma_(p, a2, 2.75573192e-06f);         // 1/9!
    p = fma_(p, a2, -1.98412698e-04f);        // -1/7!
    p = fma_(p, a2, 8.33333333e-03f);         // 1/5!
    p = fma_(p, a2, -1.66666667e-01f);        // -1/3!
    return fma_(p * a2, a, a);
}

PM_HD float cosf_(float a) {
    const float a2 = a * a;
    float p = -2.75573192e-07f;               // -1/10!
    p = fma_(p, a2, 2.48015873e-05f);         // 1/8!
    p = fma_(p, a2, -1.38888889e-03f);        // -1/6!
    p = fma_(p, a2, 4.16666667e-02f);         // 1/4!
    p = fma_(p, a2, -0.5f);
    return fma_(p, a2, 1.0f);
}

// asin on |t| <= 1/2: t + t^3 * sum_{n=1..13} c_n t^(2n-2),
// c_n = (2n)! / (4^n (n!)^2 (2n+1))
PM_HD float asin_small(float t) {
    const float t2 = t * t;
    float p = 5.740037671e-03f;  // n = 13
    p = fma_(p, t2, 6.447210312e-03f);  // n = 12
    p = fma_(p, t2, 7.312525874e-03f);  // n = 11
    p = fma_(p, t2, 8.390335810e-03f);  // n = 10
    p = fma_(p, t2, 9.761609529e-03f);  // n = 9
    p = fma_(p, t2, 1.155180090e-02f);  // n = 8
    p = fma_(p, t2, 1.396484375e-02f);  // n = 7
    p = fma_(p, t2, 1.735276442e-02f);  // n = 6
    p = fma_(p, t2, 2.237215909e-02f);  // n = 5
    p = fma_(p, t2, 3.038194444e-02f);  // n = 4
    p = fma_(p, t2, 4.464285714e-02f);  // n = 3
    p = fma_(p, t2, 7.500000000e-02f);  // n = 2
    p = fma_(p, t2, 1.666666667e-01f);  // n = 1
    return fma_(p * t2, t, t);
}

PM_HD float acosf_(float x) {
    if (!(x >= -1.0f && x <= 1.0f)) return bits_to_float(0x7fc00000u);
    const float half_pi = 1.57079637f, pi = 3.14159274f;
    if (x <= 0.5f && x >= -0.5f) return half_pi - asin_small(x);
    if (x > 0.5f) return 2.0f * asin_small(sqrt_((1.0f - x) * 0.5f));
    return pi - 2.0f * asin_small(sqrt_((1.0f + x) * 0.5f));
}

}  // namespace pmath
