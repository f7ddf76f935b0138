// pt_trig.h -- single-precision sin, cos, atan2 and acos of the path tracer,
// written so that the GPU kernels and a host build of the same source return
// the same bits.
//
// The reference calls the platform's sinf/cosf/atan2f/acosf (CUDA's device
// math on the GPU, the C library's on a host build).  Those differ from each
// other by an ulp here and there, and an ulp in a sampled direction is enough
// to send a path elsewhere a few bounces later.  Every operation below is one
// that IEEE 754 defines exactly (+, -, *, /, sqrt, fused multiply-add,
// round-to-integer, comparisons), with no contraction left to the compiler,
// so any conforming host and the GPU agree bit for bit.
//
// Methods (the mathematics only; no library's constants or steps):
//  * sin / cos: argument reduction by multiples of pi/2 after Cody and Waite
//    ("Software Manual for the Elementary Functions", 1980), with pi/2 split
//    into three floats and the products taken inside fused multiply-adds;
//    then the Taylor series of sin (to x^9) and cos (to x^10) on
//    [-pi/4, pi/4], whose truncation errors (< 2.5e-9 and < 1.2e-10 relative)
//    are far below half an ulp, evaluated by Horner's rule.
//  * atan2: reduction to t = min/max in [0, 1], the identity
//    atan(t) = pi/4 + atan((t - 1) / (t + 1)) for t > tan(pi/8), and the Taylor
//    series of atan to z^19 on |z| <= tan(pi/8) (truncation < 3e-9), then the
//    octant is restored.
//  * acos: acos(x) = pi/2 - asin(x) for |x| <= 1/2, and
//    acos(x) = 2 asin(sqrt((1 - x) / 2)) (or pi minus that for x < 0) above,
//    with the Taylor series of asin to x^21 on [0, 1/2] (truncation < 2e-9).
// Accuracy: within 2 ulp of the exact value for |x| < 1e5 (sin, cos) and for
// every input in [-1, 1] (acos), within 3 ulp for every finite pair (atan2); checked against the C library on the host
// and against CUDA's sinf/cosf/atan2f/acosf on the GPU.  Larger sin/cos
// arguments lose accuracy as in any three-part reduction, but both sides still
// agree.  Non-finite inputs give NaN (sin, cos of +-inf) as usual.
#pragma once

#include <cmath>

#if defined(__CUDACC__)
#define PT_TRIG_FN __host__ __device__ __forceinline__
#else
#define PT_TRIG_FN inline
#endif

namespace pt_trig {

// pi/2 = kPio2Hi + kPio2Mid + kPio2Lo (each the float nearest the remainder)
constexpr float kPio2Hi = 1.57079637e+00f;
constexpr float kPio2Mid = -4.37113883e-08f;
constexpr float kPio2Lo = -1.71512451e-15f;
constexpr float kTwoOverPi = 6.36619747e-01f;
constexpr float kPio2 = 1.57079637e+00f;
constexpr float kPio4 = 7.85398185e-01f;
constexpr float kPi = 3.14159274e+00f;
constexpr float kTanPio8 = 4.14213568e-01f;
// the remainders pi/4 - kPio4, pi/2 - kPio2, pi - kPi
constexpr float kPio4Lo = -2.18556941e-08f;
constexpr float kPio2Lo2 = -4.37113883e-08f;
constexpr float kPiLo = -8.74227766e-08f;

// Products that must stay separate roundings whatever the contraction
// setting (device code: the _rn intrinsics are never fused; host code: this
// header is compiled with -ffp-contract=off, as every host file here is).
#if defined(__CUDA_ARCH__)
PT_TRIG_FN float fma_(float a, float b, float c) { return __fmaf_rn(a, b, c); }
PT_TRIG_FN float mul_(float a, float b) { return __fmul_rn(a, b); }
#else
PT_TRIG_FN float fma_(float a, float b, float c) { return fmaf(a, b, c); }
PT_TRIG_FN float mul_(float a, float b) { return a * b; }
#endif
PT_TRIG_FN float rint_(float x) { return rintf(x); }  // round half to even

// Taylor polynomial of sin on [-pi/4, pi/4]: x + x^3 (c3 + x^2 (c5 + x^2 (c7 + x^2 c9)))
PT_TRIG_FN float sin_poly(float r) {
    const float s = mul_(r, r);
    float p = fma_(s, 2.75573192e-06f, -1.98412698e-04f);  // 1/9!, -1/7!
    p = fma_(s, p, 8.33333333e-03f);                        // 1/5!
    p = fma_(s, p, -1.66666667e-01f);                       // -1/3!
    return fma_(mul_(r, s), p, r);
}
// Taylor polynomial of cos on [-pi/4, pi/4]: 1 + x^2 (-1/2 + x^2 (1/4! + ...))
PT_TRIG_FN float cos_poly(float r) {
    const float s = mul_(r, r);
    float p = fma_(s, -2.75573192e-07f, 2.48015873e-05f);  // -1/10!, 1/8!
    p = fma_(s, p, -1.38888889e-03f);                       // -1/6!
    p = fma_(s, p, 4.16666667e-02f);                        // 1/4!
    p = fma_(s, p, -0.5f);                                  // -1/2!
    return fma_(s, p, 1.0f);
}

// x = q * pi/2 + r with |r| <= ~pi/4; returns r and the quadrant q mod 4.
PT_TRIG_FN float reduce(float x, int &quadrant) {
    const float q = rint_(mul_(x, kTwoOverPi));
    float r = fma_(q, -kPio2Hi, x);
    r = fma_(q, -kPio2Mid, r);
    r = fma_(q, -kPio2Lo, r);
    // q mod 4, exact for every finite q (floor and the products are exact)
    const float m = q - mul_(4.0f, floorf(mul_(q, 0.25f)));
    quadrant = (int)m;
    return r;
}

PT_TRIG_FN bool finite_(float x) { return fabsf(x) <= 3.40282347e+38f; }
PT_TRIG_FN bool negative_(float x) { return copysignf(1.0f, x) < 0.0f; }  // sign bit set (-0 too)

}  // namespace pt_trig

PT_TRIG_FN float pt_sinf(float x) {
    using namespace pt_trig;
    if (!finite_(x)) return x - x;  // NaN
    int n;
    const float r = reduce(x, n);
    const float s = sin_poly(r), c = cos_poly(r);
    switch (n & 3) {
        case 0: return s;
        case 1: return c;
        case 2: return -s;
        default: return -c;
    }
}

PT_TRIG_FN float pt_cosf(float x) {
    using namespace pt_trig;
    if (!finite_(x)) return x - x;
    int n;
    const float r = reduce(x, n);
    const float s = sin_poly(r), c = cos_poly(r);
    switch (n & 3) {
        case 0: return c;
        case 1: return -s;
        case 2: return -c;
        default: return s;
    }
}

namespace pt_trig {
// Taylor series of atan on |z| <= tan(pi/8): z + z^3 * sum_k (-1)^k z^(2k) / (2k + 3)
PT_TRIG_FN float atan_small(float z) {
    const float s = mul_(z, z);
    float p = fma_(s, -5.26315789e-02f, 5.88235294e-02f);  // -1/19, 1/17
    p = fma_(s, p, -6.66666667e-02f);                       // -1/15
    p = fma_(s, p, 7.69230769e-02f);                        // 1/13
    p = fma_(s, p, -9.09090909e-02f);                       // -1/11
    p = fma_(s, p, 1.11111111e-01f);                        // 1/9
    p = fma_(s, p, -1.42857143e-01f);                       // -1/7
    p = fma_(s, p, 2.00000000e-01f);                        // 1/5
    p = fma_(s, p, -3.33333333e-01f);                       // -1/3
    return fma_(mul_(z, s), p, z);
}
// Taylor series of asin on [0, 1/2]: x + x^3 * sum_n c_n x^(2n-2),
// c_n = (2n)! / (4^n (n!)^2 (2n + 1))
PT_TRIG_FN float asin_small(float x) {
    const float s = mul_(x, x);
    float p = fma_(s, 8.39034061e-03f, 9.76160072e-03f);  // c_10, c_9
    p = fma_(s, p, 1.15518009e-02f);                      // c_8
    p = fma_(s, p, 1.39648438e-02f);                      // c_7
    p = fma_(s, p, 1.73527644e-02f);                      // c_6
    p = fma_(s, p, 2.23721591e-02f);                      // c_5
    p = fma_(s, p, 3.03819444e-02f);                      // c_4
    p = fma_(s, p, 4.46428571e-02f);                      // c_3
    p = fma_(s, p, 7.50000000e-02f);                      // c_2
    p = fma_(s, p, 1.66666667e-01f);                      // c_1
    return fma_(mul_(x, s), p, x);
}
}  // namespace pt_trig

PT_TRIG_FN float pt_atan2f(float y, float x) {
    using namespace pt_trig;
    if (x != x || y != y) return x + y;  // NaN
    const float ax = fabsf(x), ay = fabsf(y);
    const float mx = fmaxf(ax, ay), mn = fminf(ax, ay);
    float a;
    if (mx == 0.0f) {
        a = 0.0f;
    } else if (mx > 3.40282347e+38f) {  // an infinite argument
        a = (mn > 3.40282347e+38f) ? kPio4 : 0.0f;
    } else {
        const float t = mn / mx;
        a = (t > kTanPio8) ? kPio4 + (atan_small((t - 1.0f) / (t + 1.0f)) + kPio4Lo) : atan_small(t);
    }
    if (ay > ax) a = kPio2 + (kPio2Lo2 - a);
    if (negative_(x)) a = kPi + (kPiLo - a);
    return negative_(y) ? -a : a;
}

PT_TRIG_FN float pt_acosf(float x) {
    using namespace pt_trig;
    const float ax = fabsf(x);
    if (ax <= 0.5f) return kPio2 + (kPio2Lo2 - asin_small(x));
    if (!(ax <= 1.0f)) return (x - x) / (x - x);  // NaN outside [-1, 1] and for NaN
    const float h = sqrtf(mul_(1.0f - ax, 0.5f));
    const float a = mul_(2.0f, asin_small(h));
    return x > 0.0f ? a : kPi + (kPiLo - a);
}

#undef PT_TRIG_FN
