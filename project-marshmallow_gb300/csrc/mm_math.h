/*
 * mm_math.h - elementary functions written for bit-reproducibility between host and device.
 *
 * GLSL leaves exp/pow/acos/cos accuracy implementation-defined; compute-clouds.comp uses them in
 * the sky colour (:88-127), the coverage bias (:206-208), Beer's law (:456-458) and the in-scatter
 * term (:461-462).  The functions below use only IEEE-754 +, -, *, /, sqrt, floor and exact bit
 * manipulation, never fused multiply-add, so the same source gives the same bits when compiled
 * by g++ (-ffp-contract=off) on x86-64 or aarch64 and by nvcc (-fmad=false) for the GPU.
 *
 * Methods (textbook, coefficients derived from the series below, not taken from any library):
 *  - exp: Cody-Waite range reduction x = k ln2 + r (ln2 split in a 16-bit head and a tail),
 *         then the Taylor series of e^r to degree 7 on |r| <= ln2/2 (truncation < 6e-9).
 *  - exp2: x = n + f, |f| <= 1/2, Taylor series of e^(f ln2) to degree 7.
 *  - log2: x = m 2^e with m in [sqrt(1/2), sqrt(2)), ln m = 2 atanh(s), s = (m-1)/(m+1), odd
 *          series of atanh to s^13 (truncation < 1e-11).
 *  - pow: exp2(y log2 x), the GLSL definition (GLSL 4.50 section 8.2).
 *  - asin/acos: Maclaurin series of asin on |x| <= 1/2 and acos(x) = 2 asin(sqrt((1-x)/2)) above.
 *  - sin/cos: Cody-Waite reduction by pi/2 (three-part split), Taylor series on |r| <= pi/4.
 *  - mm_sinf_cr: sin evaluated in double with a three-part double split of pi/2 and the Taylor
 *          series to r^23, then rounded once to float: the correctly rounded sinf except when the
 *          exact value falls within ~1e-16 (relative) of a float rounding boundary.
 *
 * Accuracy (checked against libm in the tests): exp/exp2 <= 2 ulp, log2 <= 2 ulp away from 1,
 * pow <= ~3e-7 relative for |y log2 x| < 32, acos/cos/sin <= 2 ulp on the ranges used.
 */
#ifndef MM_MATH_H_
#define MM_MATH_H_

#include <stdint.h>

#if defined(__CUDACC__)
#define MM_HD __host__ __device__ __forceinline__
#else
#define MM_HD inline
#endif

#if !defined(__CUDA_ARCH__)
#include <math.h>
#include <string.h>
#endif

namespace mmx {

MM_HD uint32_t f2u(float x) {
#if defined(__CUDA_ARCH__)
    return __float_as_uint(x);
#else
    uint32_t u;
    memcpy(&u, &x, 4);
    return u;
#endif
}

MM_HD float u2f(uint32_t u) {
#if defined(__CUDA_ARCH__)
    return __uint_as_float(u);
#else
    float x;
    memcpy(&x, &u, 4);
    return x;
#endif
}

MM_HD float ffloor(float x) {
#if defined(__CUDA_ARCH__)
    return floorf(x);
#else
    return floorf(x);
#endif
}

MM_HD double dfloor(double x) { return floor(x); }

MM_HD float fsqrt(float x) {
#if defined(__CUDA_ARCH__)
    return __fsqrt_rn(x);
#else
    return sqrtf(x);
#endif
}

MM_HD bool fisnan(float x) { return x != x; }

/* 2^n as a float for n in [-126, 127]. */
MM_HD float pow2i(int n) { return u2f((uint32_t)(n + 127) << 23); }

/* p * 2^n for n in [-151, 128] without intermediate overflow/underflow of the scale. */
MM_HD float scale2(float p, int n) {
    if (n > 127) return p * pow2i(127) * pow2i(n - 127);
    if (n < -126) return p * pow2i(-126) * pow2i(n + 126);
    return p * pow2i(n);
}

/* ---------------------------------------------------------------- exp / exp2 */

MM_HD float mm_expf(float x) {
    if (fisnan(x)) return x;
    if (x > 88.72284f) return u2f(0x7f800000u);
    if (x < -103.97208f) return 0.0f;
    const float LOG2E = 0x1.715476p+0f;
    const float LN2_HI = 0x1.62e4p-1f;  /* 16 significant bits: k*LN2_HI is exact */
    const float LN2_LO = 0x1.7f7d1cp-20f;
    float k = ffloor(x * LOG2E + 0.5f);
    float r = (x - k * LN2_HI) - k * LN2_LO;
    /* e^r, Taylor to degree 7, Horner */
    float p = 0x1.a01a02p-13f;          /* 1/7! */
    p = p * r + 0x1.6c16c2p-10f;        /* 1/6! */
    p = p * r + 0x1.111112p-7f;         /* 1/5! */
    p = p * r + 0x1.555556p-5f;         /* 1/4! */
    p = p * r + 0x1.555556p-3f;         /* 1/3! */
    p = p * r + 0.5f;
    p = p * r + 1.0f;
    p = p * r + 1.0f;
    return scale2(p, (int)k);
}

MM_HD float mm_exp2f(float x) {
    if (fisnan(x)) return x;
    if (x >= 128.0f) return u2f(0x7f800000u);
    if (x < -151.0f) return 0.0f;
    float n = ffloor(x + 0.5f);
    float f = x - n; /* exact */
    /* 2^f = sum (f ln2)^k / k!, coefficients ln2^k/k! */
    float p = 0x1.ffcbfcp-17f;
    p = p * f + 0x1.430912p-13f;
    p = p * f + 0x1.5d87fep-10f;
    p = p * f + 0x1.3b2ab6p-7f;
    p = p * f + 0x1.c6b08ep-5f;
    p = p * f + 0x1.ebfbe0p-3f;
    p = p * f + 0x1.62e430p-1f;
    p = p * f + 1.0f;
    return scale2(p, (int)n);
}

/* ---------------------------------------------------------------- log2 / pow */

MM_HD float mm_log2f(float x) {
    if (fisnan(x)) return x;
    if (x < 0.0f) return u2f(0x7fc00000u);
    if (x == 0.0f) return u2f(0xff800000u);
    uint32_t u = f2u(x);
    if (u == 0x7f800000u) return x;
    int e = 0;
    if (u < 0x00800000u) { /* subnormal */
        x = x * 0x1p+24f;
        u = f2u(x);
        e = -24;
    }
    e += (int)(u >> 23) - 127;
    float m = u2f((u & 0x007fffffu) | 0x3f800000u); /* [1,2) */
    if (m > 0x1.6a09e6p+0f) { /* > sqrt(2) */
        m = m * 0.5f;
        e += 1;
    }
    float s = (m - 1.0f) / (m + 1.0f);
    float z = s * s;
    float q = 0x1.3b13b2p-4f;          /* 1/13 */
    q = q * z + 0x1.745d18p-4f;        /* 1/11 */
    q = q * z + 0x1.c71c72p-4f;        /* 1/9 */
    q = q * z + 0x1.24924ap-3f;        /* 1/7 */
    q = q * z + 0x1.99999ap-3f;        /* 1/5 */
    q = q * z + 0x1.555556p-2f;        /* 1/3 */
    q = q * z;
    /* log2(m) = (2/ln2) * (s + s*q) */
    float l = 0x1.715476p+1f * (s + s * q);
    return (float)e + l;
}

/* GLSL pow: undefined for x < 0 (returns NaN here) and for x == 0, y <= 0 (returns 1 for y == 0,
 * +inf for y < 0). */
MM_HD float mm_powf(float x, float y) {
    if (x == 0.0f) return y > 0.0f ? 0.0f : (y == 0.0f ? 1.0f : u2f(0x7f800000u));
    if (x == 1.0f || y == 0.0f) return 1.0f;
    return mm_exp2f(y * mm_log2f(x));
}

/* ---------------------------------------------------------------- asin / acos */

/* asin on |x| <= 1/2: x + x^3 sum a_n x^(2n-2), a_n = (2n)! / (4^n (n!)^2 (2n+1)). */
MM_HD float asin_half(float x) {
    float z = x * x;
    float p = 0x1.782ddap-8f;
    p = p * z + 0x1.a6863ep-8f;
    p = p * z + 0x1.df3bd4p-8f;
    p = p * z + 0x1.12ef3cp-7f;
    p = p * z + 0x1.3fde50p-7f;
    p = p * z + 0x1.7a8788p-7f;
    p = p * z + 0x1.c9999ap-7f;
    p = p * z + 0x1.1c4ec4p-6f;
    p = p * z + 0x1.6e8ba2p-6f;
    p = p * z + 0x1.f1c71cp-6f;
    p = p * z + 0x1.6db6dcp-5f;
    p = p * z + 0x1.333334p-4f;
    p = p * z + 0x1.555556p-3f;
    return x + x * (z * p);
}

MM_HD float mm_acosf(float x) {
    if (fisnan(x) || x > 1.0f || x < -1.0f) return u2f(0x7fc00000u);
    const float PIO2 = 0x1.921fb6p+0f;
    const float PI = 0x1.921fb6p+1f;
    float a = x < 0.0f ? -x : x;
    if (a <= 0.5f) return PIO2 - asin_half(x);
    float h = fsqrt((1.0f - a) * 0.5f);
    float r = 2.0f * asin_half(h);
    return x < 0.0f ? PI - r : r;
}

/* ---------------------------------------------------------------- sin / cos (float) */

/* sin and cos of r, |r| <= pi/4, Taylor to r^13 / r^12. */
MM_HD float sin_kernel(float r) {
    float z = r * r;
    float p = 0x1.612462p-33f;
    p = p * z - 0x1.ae6456p-26f;
    p = p * z + 0x1.71de3ap-19f;
    p = p * z - 0x1.a01a02p-13f;
    p = p * z + 0x1.111112p-7f;
    p = p * z - 0x1.555556p-3f;
    return r + r * (z * p);
}

MM_HD float cos_kernel(float r) {
    float z = r * r;
    float p = 0x1.1eed8ep-29f;
    p = p * z - 0x1.27e4fcp-22f;
    p = p * z + 0x1.a01a02p-16f;
    p = p * z - 0x1.6c16c2p-10f;
    p = p * z + 0x1.555556p-5f;
    p = p * z - 0.5f;
    return 1.0f + z * p;
}

/* Quadrant and reduced argument for |x| < 2^15. */
MM_HD int reduce_pio2(float x, float* r) {
    float k = ffloor(x * 0x1.45f306p-1f + 0.5f);
    /* pi/2 = P1 + P2 + P3; P1, P2 have 12-bit significands so k*P1, k*P2 are exact. */
    float t = x - k * 0x1.921p+0f;
    t = t - k * 0x1.f6ap-13f;
    t = t - k * 0x1.110b46p-26f;
    *r = t;
    return ((int)k) & 3;
}

MM_HD float mm_sinf(float x) {
    if (fisnan(x)) return x;
    float r;
    int q = reduce_pio2(x, &r);
    switch (q) {
        case 0: return sin_kernel(r);
        case 1: return cos_kernel(r);
        case 2: return -sin_kernel(r);
        default: return -cos_kernel(r);
    }
}

MM_HD float mm_cosf(float x) {
    if (fisnan(x)) return x;
    float r;
    int q = reduce_pio2(x, &r);
    switch (q) {
        case 0: return cos_kernel(r);
        case 1: return -sin_kernel(r);
        case 2: return -cos_kernel(r);
        default: return sin_kernel(r);
    }
}

/* ---------------------------------------------------------------- correctly rounded sinf */

MM_HD double sin_kernel_d(double r) {
    double z = r * r;
    double p = 0x1.71b8ef6dcf572p-66;
    p = p * z - 0x1.2f49b46814157p-57;
    p = p * z + 0x1.952c77030ad4ap-49;
    p = p * z - 0x1.ae7f3e733b81fp-41;
    p = p * z + 0x1.6124613a86d09p-33;
    p = p * z - 0x1.ae64567f544e4p-26;
    p = p * z + 0x1.71de3a556c734p-19;
    p = p * z - 0x1.a01a01a01a01ap-13;
    p = p * z + 0x1.1111111111111p-7;
    p = p * z - 0x1.5555555555555p-3;
    return r + r * (z * p);
}

MM_HD double cos_kernel_d(double r) {
    double z = r * r;
    double p = -0x1.0ce396db7f853p-70;
    p = p * z + 0x1.e542ba4020225p-62;
    p = p * z - 0x1.6827863b97d97p-53;
    p = p * z + 0x1.ae7f3e733b81fp-45;
    p = p * z - 0x1.93974a8c07c9dp-37;
    p = p * z + 0x1.1eed8eff8d898p-29;
    p = p * z - 0x1.27e4fb7789f5cp-22;
    p = p * z + 0x1.a01a01a01a01ap-16;
    p = p * z - 0x1.6c16c16c16c17p-10;
    p = p * z + 0x1.5555555555555p-5;
    p = p * z - 0.5;
    return 1.0 + z * p;
}

/* sinf(x) for |x| < 2^20, evaluated in double and rounded once. */
MM_HD float mm_sinf_cr(float xf) {
    if (fisnan(xf)) return xf;
    double x = (double)xf;
    double k = dfloor(x * 0x1.45f306dc9c883p-1 + 0.5);
    /* pi/2 = D1 + D2 + D3 with 33-bit D1, D2: k*D1 and k*D2 are exact for |k| < 2^20. */
    double r = x - k * 0x1.921fb544p+0;
    r = r - k * 0x1.0b4611a6p-34;
    r = r - k * 0x1.3198a2e037073p-69;
    int q = ((int)k) & 3;
    double s;
    switch (q) {
        case 0: s = sin_kernel_d(r); break;
        case 1: s = cos_kernel_d(r); break;
        case 2: s = -sin_kernel_d(r); break;
        default: s = -cos_kernel_d(r); break;
    }
    return (float)s;
}

}  // namespace mmx

#endif /* MM_MATH_H_ */
