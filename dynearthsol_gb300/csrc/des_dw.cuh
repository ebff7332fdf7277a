// des_dw.cuh -- double-word ("float-float") arithmetic on the FP32 pipe.
//
// A double-word value is the unevaluated sum hi + lo of two floats with
// |lo| <= ulp(hi) / 2: about 48 significand bits, against FP64's 53, from
// instructions that issue at the FP32 rate (64x the FP64 rate on GB300).
// The building blocks are the published error-free transformations and the
// double-word algorithms with proven bounds, u = 2^-24:
//   * two_sum: Knuth, TAOCP vol. 2, 4.2.2 (TwoSum, 6 operations, exact);
//   * fast_two_sum: Dekker, "A floating-point technique for extending the
//     available precision", Numer. Math. 18 (1971) (3 operations, exact when
//     the exponent of a is at least that of b);
//   * two_prod: the product's exact error by one fused multiply-add (the
//     FMA form of Dekker's product);
//   * dw_add: Joldes, Muller, Popescu, "Tight and rigorous error bounds for
//     basic building blocks of double-word arithmetic", ACM TOMS 44(2), 2017,
//     Algorithm 6 (AccurateDWPlusDW): relative error below 3u^2 + 13u^3 of the
//     exact sum, cancellation included;
//   * dw_mul: the same paper, Algorithm 12 (DWTimesDW3): relative error
//     below 4u^2.
// The library is compiled with --fmad=false: no multiply and add below is
// contracted beyond the fmaf calls written out.
#pragma once
#include "des_common.cuh"

namespace des {

struct dw {
    float hi, lo;
};

__device__ __forceinline__ dw fast_two_sum(float a, float b)
{
    const float s = a + b;
    const float z = s - a;
    return {s, b - z};
}

__device__ __forceinline__ dw two_sum(float a, float b)
{
    const float s = a + b;
    const float ap = s - b;
    const float bp = s - ap;
    return {s, (a - ap) + (b - bp)};
}

__device__ __forceinline__ dw two_prod(float a, float b)
{
    const float p = a * b;
    return {p, fmaf(a, b, -p)};
}

__device__ __forceinline__ dw dw_add(dw x, dw y)
{
    const dw s = two_sum(x.hi, y.hi);
    const dw t = two_sum(x.lo, y.lo);
    const float c = s.lo + t.hi;
    const dw v = fast_two_sum(s.hi, c);
    const float w = t.lo + v.lo;
    return fast_two_sum(v.hi, w);
}

__device__ __forceinline__ dw dw_mul(dw x, dw y)
{
    const dw c = two_prod(x.hi, y.hi);
    const float tl0 = x.lo * y.lo;
    const float tl1 = fmaf(x.hi, y.lo, tl0);
    const float cl2 = fmaf(x.lo, y.hi, tl1);
    const float cl3 = c.lo + cl2;
    return fast_two_sum(c.hi, cl3);
}

__device__ __forceinline__ dw dw_neg(dw x) { return {-x.hi, -x.lo}; }

// a0 b0 + a1 b1 + a2 b2, three products and two sums
__device__ __forceinline__ dw dw_dot3(dw a0, dw b0, dw a1, dw b1, dw a2, dw b2)
{
    return dw_add(dw_add(dw_mul(a0, b0), dw_mul(a1, b1)), dw_mul(a2, b2));
}

// The double-word form of an FP64 value without an FP64 instruction: hi =
// f32_of(x), the nearest float (ties away from zero: f32_of rounds up exactly
// when bit 28 of the low word is set), and lo = the remainder x - hi, which is
// the low 29 significand bits less 2^29 when hi was rounded up, in units of
// 2^(E - 52) for x's exponent E, converted with one integer-to-float rounding
// and scaled by a power of two built from bits.  |lo| <= ulp(hi) / 2 and
// |x - (hi + lo)| <= 2^-48 |x|.  For |x| in [2^-126, 2^128); smaller
// magnitudes give (0, 0), infinities and NaN give (hi, 0).
__device__ __forceinline__ dw dw_of(double x)
{
    const unsigned hw = (unsigned)__double2hiint(x), lw = (unsigned)__double2loint(x);
    const unsigned mag = hw & 0x7fffffffu;
    const float h = f32_of(x);
    const int r = (int)(lw & 0x1fffffffu) - (int)((lw & 0x10000000u) << 1);
    const float fr = __int2float_rn(r);
    const int ef = (int)(mag >> 20) - 948;   // biased FP32 exponent of 2^(E - 52)
    float l = ef >= 1 ? fr * __uint_as_float((unsigned)ef << 23)
                      : (fr * __uint_as_float((unsigned)(ef + 64) << 23)) * 0x1p-64f;
    if (mag < (897u << 20) || mag >= (1151u << 20)) l = 0.0f;
    l = __int_as_float(__float_as_int(l) ^ (int)(hw & 0x80000000u));
    return {h, l};
}

// hi + lo rounded to FP64 (one FP64 addition; both conversions are exact)
__device__ __forceinline__ double f64_of(dw x) { return f64_of(x.hi) + f64_of(x.lo); }

}  // namespace des
