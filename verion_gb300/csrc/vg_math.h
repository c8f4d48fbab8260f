// Portable single-precision elementary functions for the path tracer.
//
// The same source compiles for the GPU (nvcc, sm_103a) and for host C++ (gcc). Every function is
// a fixed sequence of IEEE-754 single-precision adds, multiplies, divides and square roots, so
// with FMA contraction disabled (nvcc --fmad=false, gcc -ffp-contract=off) and correctly rounded
// division and square root (nvcc's defaults without fast-math) a CPU build and a GPU build return
// bit-identical results. That is what lets a CPU restatement of the integrator be compared with
// the CUDA kernels bit for bit instead of within a tolerance.
//
// Methods (all public, textbook):
//   sin/cos  Cody & Waite (1980) argument reduction by pi/2 with a three-part constant, then the
//            Taylor series of sin and cos on [-pi/4, pi/4] (truncation error < 2e-9).
//   atan     reduction to [0, 1] by atan(x) = pi/2 - atan(1/x), then to [0, tan(pi/12)] by
//            atan(x) = pi/6 + atan((sqrt(3) x - 1) / (x + sqrt(3))) (Hart et al., Computer
//            Approximations, 1968), then the Taylor series of atan.
//   acos     acos(x) = atan2(sqrt((1 - x)(1 + x)), x).
//   log2     split into exponent and mantissa m in [sqrt(1/2), sqrt(2)), then
//            ln m = 2 atanh((m - 1) / (m + 1)) by its series.
//   exp2     split y = n + f with n = rint(y), |f| <= 1/2, e^(f ln 2) by its Taylor series, ldexp.
//   pow      exp2(y log2 x) for x >= 0.
// Accuracy against double precision is checked by the test suite (a few ulp at most).
#pragma once
#include <stdint.h>
#include <math.h>
#include <string.h>

#if defined(__CUDACC__)
#define VG_HD __host__ __device__ __forceinline__
#else
#define VG_HD inline
#endif

namespace vgm {

VG_HD float as_float(uint32_t u)
{
#if defined(__CUDA_ARCH__)
    return __uint_as_float(u);
#else
    float f;
    memcpy(&f, &u, 4);
    return f;
#endif
}

VG_HD uint32_t as_uint(float f)
{
#if defined(__CUDA_ARCH__)
    return __float_as_uint(f);
#else
    uint32_t u;
    memcpy(&u, &f, 4);
    return u;
#endif
}

// Polynomials on |r| <= pi/4, Horner form, coefficients 1/n!.
VG_HD float sin_poly(float r)
{
    float r2 = r * r;
    float p = 2.7557319e-06f;               //  1/9!
    p = p * r2 + -1.9841270e-04f;           // -1/7!
    p = p * r2 + 8.3333333e-03f;            //  1/5!
    p = p * r2 + -1.6666667e-01f;           // -1/3!
    return r + (r * r2) * p;
}

VG_HD float cos_poly(float r)
{
    float r2 = r * r;
    float p = -2.7557319e-07f;              // -1/10!
    p = p * r2 + 2.4801587e-05f;            //  1/8!
    p = p * r2 + -1.3888889e-03f;           // -1/6!
    p = p * r2 + 4.1666668e-02f;            //  1/4!
    p = p * r2 + -0.5f;                     // -1/2!
    return 1.0f + r2 * p;
}

// x reduced to r in [-pi/4, pi/4] and the quadrant k (x = k pi/2 + r).
VG_HD float reduce_half_pi(float x, int& k)
{
    float kf = rintf(x * 0.63661975f);
    k = (int)kf;
    // pi/2 = C1 + C2 + C3; C1 and C2 have 12 significant bits, so k*C1 and k*C2 are exact
    // for |k| < 2^12 (|x| < ~6400, far beyond what the integrator passes).
    float r = x - kf * 1.57080078125f;
    r = r - kf * -4.4535846e-06f;
    r = r - kf * -8.7055158e-10f;
    return r;
}

VG_HD float sinf_(float x)
{
    int k;
    float r = reduce_half_pi(x, k);
    switch (k & 3) {
    case 0: return sin_poly(r);
    case 1: return cos_poly(r);
    case 2: return -sin_poly(r);
    default: return -cos_poly(r);
    }
}

VG_HD float cosf_(float x)
{
    int k;
    float r = reduce_half_pi(x, k);
    switch (k & 3) {
    case 0: return cos_poly(r);
    case 1: return -sin_poly(r);
    case 2: return -cos_poly(r);
    default: return sin_poly(r);
    }
}

// atan on [0, 1].
VG_HD float atan_unit(float x)
{
    float base = 0.0f;
    if (x > 0.26794919f) {
        x = (x * 1.7320508f - 1.0f) / (x + 1.7320508f);
        base = 0.52359879f; // pi/6
    }
    float x2 = x * x;
    float p = 7.6923080e-02f;               //  1/13
    p = p * x2 + -9.0909094e-02f;           // -1/11
    p = p * x2 + 1.1111111e-01f;            //  1/9
    p = p * x2 + -1.4285715e-01f;           // -1/7
    p = p * x2 + 2.0000000e-01f;            //  1/5
    p = p * x2 + -3.3333334e-01f;           // -1/3
    return base + (x + (x * x2) * p);
}

// atan2 with the C library's conventions for signed zeros (infinities are not expected).
VG_HD float atan2f_(float y, float x)
{
    float ax = fabsf(x);
    float ay = fabsf(y);
    float t;
    if (ax == 0.0f && ay == 0.0f)
        t = 0.0f;
    else if (ay <= ax)
        t = atan_unit(ay / ax);
    else
        t = 1.5707964f - atan_unit(ax / ay);
    if (signbit(x))
        t = 3.1415927f - t;
    return signbit(y) ? -t : t;
}

VG_HD float acosf_(float x)
{
    return atan2f_(sqrtf((1.0f - x) * (1.0f + x)), x);
}

VG_HD float log2f_(float x)
{
    if (!(x > 0.0f))
        return x == 0.0f ? -INFINITY : NAN;
    if (isinf(x))
        return x;
    int e = 0;
    if (x < 1.17549435e-38f) { // subnormal: scale into the normal range
        x = x * 16777216.0f;
        e = -24;
    }
    uint32_t b = as_uint(x);
    e += (int)((b >> 23) & 0xffu) - 127;
    float m = as_float((b & 0x7fffffu) | 0x3f800000u);
    if (m > 1.4142135f) {
        m = m * 0.5f;
        e += 1;
    }
    float f = (m - 1.0f) / (m + 1.0f);
    float f2 = f * f;
    float p = 1.1111111e-01f;               // 1/9
    p = p * f2 + 1.4285715e-01f;            // 1/7
    p = p * f2 + 2.0000000e-01f;            // 1/5
    p = p * f2 + 3.3333334e-01f;            // 1/3
    float ln = 2.0f * (f + (f * f2) * p);
    return (float)e + ln * 1.4426950f;
}

VG_HD float exp2f_(float y)
{
    if (y != y)
        return y;
    if (y > 128.0f)
        return INFINITY;
    if (y < -152.0f)
        return 0.0f;
    float n = rintf(y);
    float z = (y - n) * 0.69314718f;
    float p = 2.7557319e-06f;               // 1/9!
    p = p * z + 2.4801587e-05f;             // 1/8!
    p = p * z + 1.9841270e-04f;             // 1/7!
    p = p * z + 1.3888889e-03f;             // 1/6!
    p = p * z + 8.3333333e-03f;             // 1/5!
    p = p * z + 4.1666668e-02f;             // 1/4!
    p = p * z + 1.6666667e-01f;             // 1/3!
    p = p * z + 0.5f;                       // 1/2!
    p = p * z + 1.0f;
    p = p * z + 1.0f;
    return ldexpf(p, (int)n);
}

VG_HD float powf_(float x, float y)
{
    if (x == 0.0f)
        return y > 0.0f ? 0.0f : (y == 0.0f ? 1.0f : INFINITY);
    return exp2f_(y * log2f_(x));
}

} // namespace vgm
