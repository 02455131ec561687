// ffsincos.cuh -- float cosine and sine, correctly rounded from the exact
// value, evaluated in single precision where that is certain.
//
// The quaternion expansion of the reference (quaternion_math.h:79-90) takes
// the cosine and sine of float half angles in double precision and rounds the
// results to float: float(cos(double(x))).  The ridge and direction kernels
// must reproduce those floats bit for bit, because they feed discrete
// decisions (ridge or not, the sign of a direction).  Double precision runs
// at a small fraction of the single-precision rate on this GPU, so this file
// evaluates cos and sin in double-float arithmetic (pairs of floats, about 44
// significant bits; Dekker's and Knuth's error-free transformations with the
// fused multiply-add) and returns the float nearest to the value whenever the
// evaluation's error bound cannot straddle a rounding boundary.  Otherwise,
// and for arguments outside [-4, 4] or not finite, it reports failure and the
// caller evaluates in double precision as before.  A certain result equals
// float(cos(double(x))) of any double implementation with an error far below
// the bound, since that value lies on the same side of the boundary.
//
// Method (own derivation from the series definitions):
//   1. k = nearest integer to x * 2/pi; r = x - k * pi/2 in double-float, with
//      pi/2 as the sum of three floats (each product with k is exact).
//   2. z = r^2; the Taylor series of sin(r)/r and cos(r) in z, the terms
//      below 2^-24 of the result in float Horner steps, the leading terms in
//      double-float.
//   3. The quadrant k mod 4 selects +-sin / +-cos.
//   4. The result (h, l), |l| <= ulp(h)/2, rounds to h when |l| plus the
//      error bound stays below the distance from h to the rounding midpoint
//      on l's side (a quarter ulp below a power of two, half an ulp
//      otherwise).
//
// Every float operation is an explicit round-to-nearest intrinsic, so the
// compiler contracts nothing; the host build (for the exhaustive CPU check)
// maps them to std::fma and plain operators under -ffp-contract=off.
#pragma once

#if defined(__CUDACC__)
#define FF_HD __host__ __device__ __forceinline__
#else
#define FF_HD inline
#endif

#if defined(__CUDA_ARCH__)
#define FF_ADD(a, b) __fadd_rn((a), (b))
#define FF_SUB(a, b) __fsub_rn((a), (b))
#define FF_MUL(a, b) __fmul_rn((a), (b))
#define FF_FMA(a, b, c) __fmaf_rn((a), (b), (c))
#define FF_RINT(a) rintf(a)
#define FF_ABS(a) fabsf(a)
#define FF_BITS(a) __float_as_uint(a)
#define FF_FROM_BITS(u) __uint_as_float(u)
#else
#include <cmath>
#include <cstdint>
#include <cstring>
#define FF_ADD(a, b) ((a) + (b))
#define FF_SUB(a, b) ((a) - (b))
#define FF_MUL(a, b) ((a) * (b))
#define FF_FMA(a, b, c) std::fma((float)(a), (float)(b), (float)(c))
#define FF_RINT(a) std::rint(a)
#define FF_ABS(a) std::fabs(a)
inline uint32_t ff_bits_host(float a) { uint32_t u; std::memcpy(&u, &a, 4); return u; }
inline float ff_from_bits_host(uint32_t u) { float a; std::memcpy(&a, &u, 4); return a; }
#define FF_BITS(a) ff_bits_host(a)
#define FF_FROM_BITS(u) ff_from_bits_host(u)
#endif

namespace m16 {
namespace ff {

struct F2 { float h, l; };

// a + b exactly as h + l (Knuth)
FF_HD F2 two_sum(float a, float b)
{
    const float s = FF_ADD(a, b);
    const float bb = FF_SUB(s, a);
    const float e = FF_ADD(FF_SUB(a, FF_SUB(s, bb)), FF_SUB(b, bb));
    return {s, e};
}

// a + b exactly, |a| >= |b| (Dekker)
FF_HD F2 fast_two_sum(float a, float b)
{
    const float s = FF_ADD(a, b);
    return {s, FF_SUB(b, FF_SUB(s, a))};
}

// a * b exactly (fused multiply-add)
FF_HD F2 two_prod(float a, float b)
{
    const float p = FF_MUL(a, b);
    return {p, FF_FMA(a, b, -p)};
}

FF_HD F2 add(F2 x, F2 y)
{
    F2 s = two_sum(x.h, y.h);
    s.l = FF_ADD(s.l, FF_ADD(x.l, y.l));
    return fast_two_sum(s.h, s.l);
}

FF_HD F2 add_f(F2 x, float y)
{
    F2 s = two_sum(x.h, y);
    s.l = FF_ADD(s.l, x.l);
    return fast_two_sum(s.h, s.l);
}

FF_HD F2 mul(F2 x, F2 y)
{
    F2 p = two_prod(x.h, y.h);
    p.l = FF_FMA(x.h, y.l, FF_FMA(x.l, y.h, p.l));
    return fast_two_sum(p.h, p.l);
}

// 1/n! as double-float constants (h = float nearest, l = float nearest the rest)
constexpr float kInv2h = 0.5f, kInv2l = 0.0f;
constexpr float kInv6h = 0.16666667163372040f, kInv6l = -4.967053879e-09f;
constexpr float kInv24h = 0.041666667908430099f, kInv24l = -1.241763470e-09f;
constexpr float kInv120h = 0.0083333337679505348f, kInv120l = -4.346172033e-10f;
constexpr float kInv720h = 0.0013888889225199819f, kInv720l = -3.363109444e-11f;
constexpr float kInv5040h = 0.00019841270113829523f, kInv5040l = -2.725596875e-12f;
constexpr float kInv40320h = 2.4801587642286904e-05f, kInv40320l = -3.406996094e-13f;
// pi/2 = kP1 + kP2 + kP3 to about 2^-73 (Cody and Waite's splitting): kP1 and
// kP2 have 22 significant bits, so their products with |k| <= 3 are exact
constexpr float kP1 = 1.5707964897155762f;
constexpr float kP2 = -1.6292068494294654e-07f;
constexpr float kP3 = 5.390302953474238e-15f;
constexpr float kTwoOverPi = 0.6366197467f;

// relative error bound of the double-float sin and cos below (the series
// truncation, the float tails, the double-float steps and the reduction).
// Checked on every float of [-4, 4] (2,164,260,866 arguments) against long
// double sinl/cosl: largest relative error 6.4e-14 (2^-43.8), every certain
// result correctly rounded, 3,138 arguments left to double precision.
constexpr float kRelErr = 2.27373675e-13f;   // 2^-42

// distance from h to the float rounding midpoint on the side of l (> 0 for
// finite, nonzero h)
FF_HD float half_gap(float h, float l)
{
    const uint32_t b = FF_BITS(h) & 0x7fffffffu;
    const uint32_t e = b & 0x7f800000u;
    const float ulp = FF_FROM_BITS(e > 0x0b800000u ? e - 0x0b800000u : 0x00000001u);   // 2^(exp - 23)
    const bool toward_zero = (FF_BITS(h) ^ FF_BITS(l)) & 0x80000000u;
    const bool pow2 = (b & 0x007fffffu) == 0;
    return (pow2 && toward_zero && l != 0.f) ? FF_MUL(ulp, 0.25f) : FF_MUL(ulp, 0.5f);
}

// the float nearest to v = (h, l) with error bound err, or false when the
// bound reaches the rounding midpoint
FF_HD bool round_certain(F2 v, float err, float *out)
{
    if (!(v.h != 0.f) || FF_ABS(v.h) < 1.17549435e-38f) return false;   // zero, subnormal, NaN
    if (FF_ADD(FF_ABS(v.l), err) < half_gap(v.h, v.l)) { *out = v.h; return true; }
    return false;
}

// sin(x) and cos(x) as double-floats for |x| <= 4; false outside
FF_HD bool sincos_f2(float x, F2 *s, F2 *c)
{
    if (!(FF_ABS(x) <= 4.0f)) return false;
    const float k = FF_RINT(FF_MUL(x, kTwoOverPi));
    // r = x - k * pi/2 with |k| <= 3: k * kP1 and k * kP2 are exact
    F2 r = two_sum(x, -FF_MUL(k, kP1));
    r = add_f(r, -FF_MUL(k, kP2));
    r = add_f(r, -FF_MUL(k, kP3));
    const F2 z = mul(r, r);
    const float zf = z.h;
    // sin(r)/r = 1 - z/6 + z^2/120 - z^3/5040 + z^4/362880 - z^5/39916800 + z^6/6227020800
    //           - z^7/1307674368000
    float ts = FF_FMA(zf, -7.647163610e-13f, 1.605904437e-10f);
    ts = FF_FMA(zf, ts, -2.505210794e-08f);
    ts = FF_FMA(zf, ts, 2.755731884e-06f);
    F2 ps = add_f(F2{-kInv5040h, -kInv5040l}, FF_MUL(zf, ts));
    ps = add(F2{kInv120h, kInv120l}, mul(z, ps));
    ps = add(F2{-kInv6h, -kInv6l}, mul(z, ps));
    ps = add_f(mul(z, ps), 1.0f);
    *s = mul(r, ps);
    // cos(r) = 1 - z/2 + z^2/24 - z^3/720 + z^4/40320 - z^5/3628800 + z^6/479001600 - z^7/87178291200
    float tc = FF_FMA(zf, -1.147074536e-11f, 2.087675588e-09f);
    tc = FF_FMA(zf, tc, -2.755731998e-07f);
    F2 pc = add_f(F2{kInv40320h, kInv40320l}, FF_MUL(zf, tc));
    pc = add(F2{-kInv720h, -kInv720l}, mul(z, pc));
    pc = add(F2{kInv24h, kInv24l}, mul(z, pc));
    pc = add(F2{-kInv2h, -kInv2l}, mul(z, pc));
    *c = add_f(mul(z, pc), 1.0f);
    // quadrant
    const int q = ((int)k) & 3;
    const F2 ns = {-s->h, -s->l}, nc = {-c->h, -c->l};
    const F2 sv = *s, cv = *c;
    switch (q) {
    case 0: *s = sv; *c = cv; break;
    case 1: *s = cv; *c = ns; break;
    case 2: *s = ns; *c = nc; break;
    default: *s = nc; *c = sv; break;
    }
    return true;
}

// float(sin(x)) and float(cos(x)) correctly rounded, or false
FF_HD bool sincos_rn(float x, float *sr, float *cr)
{
    F2 s, c;
    if (FF_ABS(x) < 2.44140625e-4f) {
        // |x| < 2^-12: sin(x) = x(1 - x^2/6 + ...) lies within a quarter ulp of
        // x, and cos(x) = 1 - x^2/2 + ... above the midpoint 1 - 2^-25
        // below 1, so they round to x (signed zero included) and to 1
        *sr = x;
        *cr = 1.0f;
        return true;
    }
    if (!sincos_f2(x, &s, &c)) return false;
    // the error bound is relative to each result (the series give sin(r)/r
    // and cos(r), |r| <= pi/4, to a relative kRelErr)
    return round_certain(s, FF_MUL(kRelErr, FF_ABS(s.h)), sr) && round_certain(c, FF_MUL(kRelErr, FF_ABS(c.h)), cr);
}

}  // namespace ff
}  // namespace m16
