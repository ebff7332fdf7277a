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
//     below 4u^2;
//   * dw_dot3c, dw_diff2, dw_sum3, dw_sum: the compensated dot product and
//     sum Dot2 / Sum2 of Ogita, Rump, Oishi, "Accurate sum and dot product",
//     SIAM J. Sci. Comput. 26(6), 2005, on the high parts, with the low
//     parts' terms added to the compensation.
// tests/test_dw_arith.py restates each in numpy and holds it to its bound
// against exact rational arithmetic.
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

// The double-word form of an FP64 value by truncation, without an FP64
// instruction:
// hi = x's sign, exponent and top 23 stored significand bits (x truncated to
// 24 significant bits), lo = the remaining 29 bits, of x's sign, rounded to
// float (2^23 + b - 2^23 gives the halves exactly, one fma joins them) and
// scaled by a power of two; then normalised by fast_two_sum.
// |lo| <= ulp(hi) / 2 and |x - (hi + lo)| <= 2^-47 |x| for |x| in [2^-97, 2^128);
// in [2^-126, 2^-97) lo is subnormal and the error below 2^-149 + 2^-47 |x|;
// smaller magnitudes give (0, 0), larger ones and NaN (inf / NaN, 0).
__device__ __forceinline__ dw dw_split(double x)
{
    const unsigned hw = (unsigned)__double2hiint(x), lw = (unsigned)__double2loint(x);
    const unsigned mag = hw & 0x7fffffffu, sg = hw & 0x80000000u;
    unsigned hb = ((mag - (896u << 20)) << 3) | (lw >> 29);
    // the 29 bits as a float from two exact halves (FP32 instructions only)
    const unsigned L = lw & 0x1fffffffu;
    const float fr = fmaf(__uint_as_float(0x4B000000u | (L >> 23)) - 8388608.0f, 8388608.0f,
                          __uint_as_float(0x4B000000u | (L & 0x7fffffu)) - 8388608.0f);
    const int ef = (int)(mag >> 20) - 948;   // biased FP32 exponent of 2^(E - 52)
    float l = ef >= 1 ? fr * __uint_as_float((unsigned)ef << 23)
                      : (fr * __uint_as_float((unsigned)(ef + 64) << 23)) * 0x1p-64f;
    if (mag < (897u << 20)) {
        hb = 0;
        l = 0.0f;
    } else if (mag >= (1151u << 20)) {
        hb = (mag > 0x7ff00000u || (mag == 0x7ff00000u && lw)) ? 0x7fc00000u : 0x7f800000u;
        l = 0.0f;
    }
    // normalised (exact): hi becomes the nearest float, |lo| <= ulp(hi) / 2,
    // as the double-word algorithms' bounds assume of their operands
    return fast_two_sum(__uint_as_float(sg | hb), __uint_as_float(__float_as_uint(l) ^ sg));
}

// a0 b0 + a1 b1 + a2 b2 for double-word operands: Dot2 on the high parts
// (exact products by two_prod, exact sums by two_sum, their errors summed in
// one float s), the cross terms ah bl + al bh added to s, al bl (below
// u^2 |a b|) dropped, and the pair (sum, s) renormalised.  The error is at
// most about (gamma_3^2 + 3u^2) sum |a_i b_i| ~ 12u^2 of the terms' magnitudes,
// however much they cancel: 37 operations, against 67 for three dw_mul and
// two dw_add.
__device__ __forceinline__ dw dw_dot3c(dw a0, dw b0, dw a1, dw b1, dw a2, dw b2)
{
    const dw p0 = two_prod(a0.hi, b0.hi), p1 = two_prod(a1.hi, b1.hi), p2 = two_prod(a2.hi, b2.hi);
    float s = p0.lo + fmaf(a0.hi, b0.lo, a0.lo * b0.hi);
    const dw t1 = two_sum(p0.hi, p1.hi);
    s += t1.lo + (p1.lo + fmaf(a1.hi, b1.lo, a1.lo * b1.hi));
    const dw t2 = two_sum(t1.hi, p2.hi);
    s += t2.lo + (p2.lo + fmaf(a2.hi, b2.lo, a2.lo * b2.hi));
    return two_sum(t2.hi, s);
}

// x + y + z of double-word values: Sum2 on the high parts with the low parts
// added to the compensation; error about 4u^2 (|x| + |y| + |z|)
__device__ __forceinline__ dw dw_sum3(dw x, dw y, dw z)
{
    const dw t1 = two_sum(x.hi, y.hi);
    float c = t1.lo + (x.lo + y.lo);
    const dw t2 = two_sum(t1.hi, z.hi);
    c += t2.lo + z.lo;
    return two_sum(t2.hi, c);
}

// a b - c d for double-word operands (a cross-product component), in the
// manner of dw_dot3c: exact high products and difference, the errors and the
// cross terms in one float; error below 8u^2 (|a b| + |c d|)
__device__ __forceinline__ dw dw_diff2(dw a, dw b, dw c, dw d)
{
    const dw p = two_prod(a.hi, b.hi), q = two_prod(c.hi, d.hi);
    const dw t = two_sum(p.hi, -q.hi);
    const float s = ((p.lo - q.lo) + (fmaf(a.hi, b.lo, a.lo * b.hi) - fmaf(c.hi, d.lo, c.lo * d.hi))) + t.lo;
    return two_sum(t.hi, s);
}

// 1 / x for a double-word x of normal magnitude: the FP32 quotient r0 and one
// Newton step r0 + r0 (1 - x r0), whose residual is formed exactly up to
// x.lo r0 (x.hi r0 by two_prod, 1 - its high part exact as it lies within
// 2u of 1); relative error below 8u^2 (the residual's two roundings, the
// correction's, and the step's quadratic term; tests/test_dw_arith.py)
__device__ __forceinline__ dw dw_recip(dw x)
{
    const float r0 = 1.0f / x.hi;
    const dw p = two_prod(x.hi, r0);
    const float e = ((1.0f - p.hi) - p.lo) - x.lo * r0;
    return fast_two_sum(r0, r0 * e);
}

__device__ __forceinline__ dw dw_of2(float2 v) { return {v.x, v.y}; }

// hi + lo rounded to FP64 (one FP64 addition; both conversions are exact)
__device__ __forceinline__ double f64_of(dw x) { return f64_of(x.hi) + f64_of(x.lo); }

// A running sum in Sum2's manner (Ogita, Rump, Oishi 2005): the high parts
// summed with two_sum, the rounding errors and the low parts in the
// compensation.  For the mixed step's node sums over a support list (a few
// dozen terms): error at most ~n^2 u^2 of the terms' magnitudes, ~1e-12 in
// the worst case, 1e-14 typically; 7 FP32 operations per FP32 term, 8 and a
// split per FP64 term, against one FP64 addition.
struct dw_sum {
    float s = 0.0f, c = 0.0f;
    __device__ __forceinline__ void add(dw x)
    {
        const dw t = two_sum(s, x.hi);
        s = t.hi;
        c += t.lo + x.lo;
    }
    __device__ __forceinline__ void add(float x)
    {
        const dw t = two_sum(s, x);
        s = t.hi;
        c += t.lo;
    }
    __device__ __forceinline__ double value() const { return f64_of(two_sum(s, c)); }
};

}  // namespace des
