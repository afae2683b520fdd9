// IEEE double comparisons, minimum and maximum evaluated on the integer
// pipes from the bit patterns. On GB300 every FP64 instruction -- compares
// and min/max included -- occupies an SMSP's FP64 pipe for 64 cycles per
// warp, while the integer pipes are idle; the secant pass makes ~30 such
// decisions. Each helper returns exactly what the IEEE comparison returns for
// every input, NaN and signed zeros included (IEEE ordering of doubles is the
// ordering of their sign-magnitude bit patterns, with NaN unordered and
// +0 == -0).
#pragma once

#include <cuda_runtime.h>

namespace tr {

constexpr long long kInfBits = 0x7ff0000000000000ll;

__device__ __forceinline__ long long dbits(double x) { return __double_as_longlong(x); }

// x > 0
__device__ __forceinline__ bool fp_gt0(double x)
{
    const long long b = dbits(x);
    return b > 0 && b <= kInfBits;
}

// x < 0
__device__ __forceinline__ bool fp_lt0(double x)
{
    const unsigned long long b = (unsigned long long)dbits(x);
    return b > 0x8000000000000000ull && b <= 0xfff0000000000000ull;
}

// x == 0 (either sign)
__device__ __forceinline__ bool fp_eq0(double x) { return ((unsigned long long)dbits(x) << 1) == 0; }

// x > c for a constant or value c > 0 that is not NaN
__device__ __forceinline__ bool fp_gt_pos(double x, double c)
{
    const long long b = dbits(x);
    return b > dbits(c) && b <= kInfBits;
}

// x >= c for c >= +0 (not NaN, not -0); x >= +0 is true for x = -0 as well
__device__ __forceinline__ bool fp_ge_nonneg(double x, double c)
{
    const long long b = dbits(x);
    if (((unsigned long long)b << 1) == 0) return dbits(c) == 0;  // x = +-0: only c = 0 qualifies
    return b >= dbits(c) && b <= kInfBits;
}

// x < c for a constant or value c > 0 that is not NaN
__device__ __forceinline__ bool fp_lt_pos(double x, double c)
{
    const long long b = dbits(x);
    // sign set: -0 and negative numbers are below c, a negative NaN is not
    return b < 0 ? (unsigned long long)b <= 0xfff0000000000000ull : b < dbits(c);
}

// |a| > b for any a, b (false when either is NaN)
__device__ __forceinline__ bool fp_abs_gt(double a, double b)
{
    const long long ma = dbits(a) & 0x7fffffffffffffffll;
    const long long bb = dbits(b);
    const long long mb = bb & 0x7fffffffffffffffll;
    if (ma > kInfBits || mb > kInfBits) return false;
    if (bb < 0) return ma != 0 || mb != 0;  // b <= -0: |a| > b unless both are zeros
    return ma > mb;
}

// fmax(x, 0.0) and fmax(0.0, x): the positive value, otherwise +0 (NaN -> +0,
// as IEEE maxNum returns the non-NaN operand)
__device__ __forceinline__ double fp_max0(double x) { return fp_gt0(x) ? x : 0.0; }

// fmin(c, x) for c > 0 not NaN and x >= +0 or NaN (a NaN x gives c), and
// fmax(c, x) for c > 0 not NaN and any x (x <= c or NaN gives c)
__device__ __forceinline__ double fp_min_pos(double c, double x)
{
    const long long b = dbits(x);
    return (b >= 0 && b < dbits(c)) ? x : c;
}
__device__ __forceinline__ double fp_max_pos(double c, double x) { return fp_gt_pos(x, c) ? x : c; }

// 2.0 * a * b * c * d as the reference writes it, (((2a) b) c) d, given the
// undoubled chain g1 = a b, g2 = g1 c, g = g2 d (all positive). Doubling
// commutes with rounding while a product stays in the normal range, so when
// g1, g2 and g are at least 2^-1021 and 2g is finite the result is exactly
// 2g, formed by raising g's exponent on the integer pipe; otherwise it is
// evaluated as written.
__device__ __forceinline__ double twice_chain(double g1, double g2, double g, double a, double b, double c, double d)
{
    const unsigned e1 = (unsigned)((unsigned long long)dbits(g1) >> 52) & 0x7ffu;
    const unsigned e2 = (unsigned)((unsigned long long)dbits(g2) >> 52) & 0x7ffu;
    const unsigned e3 = (unsigned)((unsigned long long)dbits(g) >> 52) & 0x7ffu;
    // exponents 2..0x7fd: the exact products are normal and their doubles finite
    if (e1 - 2u < 0x7fcu && e2 - 2u < 0x7fcu && e3 - 2u < 0x7fcu)
        return __longlong_as_double(dbits(g) + (1ll << 52));
    return 2.0 * a * b * c * d;
}

}  // namespace tr

namespace tr {

// Correctly rounded quotients that share one reciprocal.
//
// With y = RN(1/b) (CUDA's correctly rounded __drcp_rn), each quotient costs
// one product and four FMAs instead of a full division: q0 = RN(a y) is within
// 2 ulp of a/b; one correction q1 = RN(q0 + RN(a - b q0) y) is faithful; then
// the residual a - b q1 is exact and q2 = RN(q1 + (a - b q1) y) is the
// correctly rounded a/b (Markstein's theorem, P. Markstein, "Computation of
// elementary functions on the IBM RISC System/6000 processor", IBM J. Res.
// Dev. 34(1), 1990; also Muller et al., Handbook of Floating-Point
// Arithmetic, the FMA-based division section). The theorem needs normal
// operands and a normal quotient away from overflow: operands whose exponents
// are far from that range, zeros, infinities and NaNs take the IEEE division.
struct SharedRcp {
    double b, y;
    bool ok;  // b normal, |b| in [2^-500, 2^501)
};

__device__ __forceinline__ int dexp(double x) { return (int)(((unsigned long long)dbits(x) >> 52) & 0x7ff); }

__device__ __forceinline__ SharedRcp shared_rcp(double b)
{
    SharedRcp r;
    r.b = b;
    const int eb = dexp(b);
    r.ok = eb >= 1023 - 500 && eb <= 1023 + 500;
    r.y = r.ok ? __drcp_rn(b) : 0.0;
    return r;
}

__device__ __forceinline__ double shared_div(double a, const SharedRcp& d)
{
    const int ea = dexp(a);
    // a normal and |a|, |b| in [2^-500, 2^501): |a/b| is far inside the normal
    // range; else the IEEE division
    if (!d.ok || ea < 1023 - 500 || ea > 1023 + 500) return a / d.b;
    double q = a * d.y;
    double r = __fma_rn(-d.b, q, a);
    q = __fma_rn(r, d.y, q);
    r = __fma_rn(-d.b, q, a);
    return __fma_rn(r, d.y, q);
}

// RN(a / b) > c -- the IEEE quotient compared with c -- for any a, b > 0 and
// c > 0 (neither NaN), mostly without the division. RN(a/b) > c exactly when
// a/b lies above the midpoint m = c + u between c and the next double
// (u = ulp(c)/2, a power of two), up to the tie a/b = m. With x = a - c b and
// y = u b (exact for b and c normal, y normal): a/b > m <=> x > y. The FMA
// gives e = RN(x) with one rounding, and rounding is monotone with y
// representable, so e > y implies x > y and e < y implies x < y. Only e == y
// (a tie, or x within half an ulp of y), NaN and operands outside the normal
// range take the division.
__device__ __forceinline__ bool quot_gt_pos(double a, double b, double c)
{
    const int eb = dexp(b), ec = dexp(c);
    const int k = ec - 1023 - 53;  // u = 2^k
    if ((unsigned)(eb - 1) < 0x7feu && (unsigned)(ec - 1) < 0x7feu && (unsigned)(eb + k - 1) < 0x7feu) {
        const double y = __longlong_as_double(dbits(b) + ((long long)k << 52));
        const double e = __fma_rn(-c, b, a);
        if (fp_gt_pos(e, y)) return true;
        if (fp_lt_pos(e, y)) return false;
    }
    return fp_gt_pos(a / b, c);
}

// |x| on the integer pipe
__device__ __forceinline__ double fp_abs(double x) { return __longlong_as_double(dbits(x) & 0x7fffffffffffffffll); }

// x is finite (not infinite, not NaN)
__device__ __forceinline__ bool fp_finite(double x) { return (dbits(x) & kInfBits) != kInfBits; }

// 0.5 * x: for an exponent field of 2..0x7fe the product is x with the field
// lowered by one, exactly (the result stays normal); zeros, subnormals,
// the smallest normals, infinities and NaN take the multiplication.
__device__ __forceinline__ double fp_half(double x)
{
    const unsigned e = (unsigned)((unsigned long long)dbits(x) >> 52) & 0x7ffu;
    return (e - 2u < 0x7fdu) ? __longlong_as_double(dbits(x) - (1ll << 52)) : 0.5 * x;
}

}  // namespace tr
