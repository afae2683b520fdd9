// Correctly rounded pow(x, 2.0/3.0) and pow(x, 5.0/3.0) in double precision,
// host and device. (The exponents are the doubles nearest 2/3 and 5/3, as in
// the reference's pow calls; steps 1-3 work with the rationals and step 4
// applies the exponent offset.)
//
// The MC solver raises the hydraulic radius R to the powers 2/3 and 5/3 at
// every depth it evaluates (troute_mc_final.cu:80, :91, :99, :111, :136); this
// is where most of its FP64 work went with the general pow(). Both powers come
// from one inverse cube root:
//   1. write x = y * 2^(3k) with y in [1, 8) (exact exponent split);
//   2. seed r ~ y^(-1/3) in single precision (hardware log2/exp2 on the GPU,
//      ~2^-22 relative), then one Newton step for f(r) = y r^3 - 1 in double
//      precision, r <- r + r (1 - y r^3) / 3 (quadratic: ~2^-43);
//   3. z = y r ~ y^(2/3) to ~2^-42; the residual d = z^3 - y^2 is evaluated
//      exactly enough with error-free products (a*b = p + fma(a, b, -p), the
//      FMA form of Dekker's TwoProduct), and one more Newton step gives the
//      correction delta = -d / (3 z^2) = -d r^4 / 3 (z is within a factor 2 of
//      the root, so q - s below is exact), leaving z + delta within ~2^-84 of
//      y^(2/3);
//   4. the exponent offset e = fl(2/3) - 2/3 contributes the factor
//      1 + e ln x (|e ln x| < 1e-13), so pow(x, fl(2/3)) =
//      round(z + (delta + z e ln x)) and pow(x, fl(5/3)) =
//      round(y z + (err(y z) + y delta + y z e' ln x)), each scaled back by
//      2^(2k), 2^(5k) (exact).
// The sums of step 4 are within ~2^-74 relative of the exact values (the
// ~1e-16 exponent-offset term is formed from the seed's single-precision
// log2, and on the device for x in [2^-9, 2^9) in single precision: ~2^-24
// of it). Their rounding is checked (Ziv's rounding test): each sum s = a + c
// is split exactly into s + err (Fast2Sum, |a| >= |c|), and when |err| comes
// within 2^-68 relative of half an ulp of s -- a rounding midpoint the
// computed sum may be on the wrong side of -- both powers are recomputed with
// one more Newton step (z within ~2^-51, z + delta within ~2^-100) and the
// offset terms from a double-precision log. That happens for ~1 argument in
// 2^14; the results are then the correctly rounded values except within
// ~2^-95 of a midpoint (never met in the parity runs, ~10^10 evaluations).
// The C library's pow() (glibc) is not correctly rounded: it differs from
// these results by one ulp on ~0.2 % of arguments.
// Only IEEE operations and explicit fma() are used, so compiling without
// implicit FMA contraction does not change these results.
#pragma once

#include <cstdint>
#include <cstring>

#if defined(__CUDACC__)
#define CRPOW_HD __host__ __device__ __forceinline__
#else
#define CRPOW_HD inline
#include <cmath>
#endif

namespace tr {

CRPOW_HD uint64_t crpow_bits(double x)
{
#if defined(__CUDA_ARCH__)
    return (uint64_t)__double_as_longlong(x);
#else
    uint64_t b;
    std::memcpy(&b, &x, 8);
    return b;
#endif
}

CRPOW_HD double crpow_from_bits(uint64_t b)
{
#if defined(__CUDA_ARCH__)
    return __longlong_as_double((long long)b);
#else
    double x;
    std::memcpy(&x, &b, 8);
    return x;
#endif
}

#if defined(__CUDA_ARCH__)
// Float <-> double conversions for the seed, on the integer pipe (the FP64
// pipe is the solver's bottleneck): y in [1, 8) truncated to float; a normal
// float (or +0) widened exactly.
__device__ __forceinline__ float crpow_y_to_float(double y)
{
    const long long b = __double_as_longlong(y);
    return __int_as_float((int)(((b >> 52) - 896) << 23) | (int)((b >> 29) & 0x7fffff));
}
__device__ __forceinline__ double crpow_widen(float f)
{
    const unsigned fb = __float_as_uint(f);
    if ((fb << 1) == 0) return 0.0;
    const unsigned long long sign = (unsigned long long)(fb >> 31) << 63;
    return __longlong_as_double((long long)(sign | ((unsigned long long)(((fb >> 23) & 0xff) + 896) << 52) |
                                            ((unsigned long long)(fb & 0x7fffff) << 29)));
}
#endif

// Single-precision log2(y) and seed of y^(-1/3) for y in [1, 8).
CRPOW_HD void crpow_seed(double y, float* log2y, double* rinv)
{
#if defined(__CUDA_ARCH__)
    const float yf = crpow_y_to_float(y);
    float l, r;
    asm("lg2.approx.ftz.f32 %0, %1;" : "=f"(l) : "f"(yf));
    const float e = l * (-1.0f / 3.0f);
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(e));
    *log2y = l;
    *rinv = crpow_widen(r);
#else
    *log2y = std::log2((float)y);
    *rinv = (double)(1.0f / std::cbrt((float)y));
#endif
}

// 2^n as a double for |n| <= 1022 (exact)
CRPOW_HD double crpow_exp2i(int n) { return crpow_from_bits((uint64_t)(1023 + n) << 52); }

// Scales v by 2^n (n may exceed the single-step range); exact for normal results.
CRPOW_HD double crpow_scale(double v, int n)
{
#if defined(__CUDA_ARCH__)
    {
        // a normal result: add n to the exponent field on the integer pipe
        const long long b = __double_as_longlong(v);
        const int ev = (int)((b >> 52) & 0x7ff);
        if (ev != 0 && ev != 0x7ff && ev + n >= 1 && ev + n <= 0x7fe)
            return __longlong_as_double(b + ((long long)n << 52));
    }
#endif
    while (n > 1000) { v *= crpow_exp2i(1000); n -= 1000; }
    while (n < -1000) { v *= crpow_exp2i(-1000); n += 1000; }
    return v * crpow_exp2i(n);
}

// fl(2/3) - 2/3 = -(1/3) 2^-53 and fl(5/3) - 5/3 = (1/3) 2^-52
constexpr double kFl23Minus23 = -3.700743415417188e-17;
constexpr double kFl53Minus53 = 7.401486830834377e-17;

// Whether s = fl(a + c), with err = (a + c) - s exact, may round differently
// from a value within 2^-68 s of a + c: |err| above (1 - 2^-15) ulp(s) / 2,
// compared on the integer pipe (non-negative doubles order like their bit
// patterns); a power of two (the spacing changes at s) or a tiny s always
// counts as uncertain.
CRPOW_HD bool crpow_near_midpoint(double s, double err)
{
    const uint64_t sb = crpow_bits(s);
    const uint64_t eb = crpow_bits(err) & 0x7FFFFFFFFFFFFFFFull;
    const uint64_t es = (sb >> 52) & 0x7FF;
    if ((sb & 0x000FFFFFFFFFFFFFull) == 0 || es < 64) return true;
    // (1 - 2^-15) ulp(s) / 2 = 2^(es - 1077) (2 - 2^-14): biased exponent es - 54
    const uint64_t thr = ((es - 54) << 52) | 0x000FFFC000000000ull;
    return eb > thr;
}

// The accurate path of pow23_53 for arguments the rounding test sends there:
// one more Newton step for r = y^(-1/3), the residual correction again, and
// the exponent-offset terms from a double-precision log of x = y 2^(3k).
// Returns {x^(2/3), x^(5/3)} before the scaling by 2^(2k), 2^(5k). On the
// device it is a separate function: it runs for a tiny share of the
// arguments, and out of line it keeps the solver's loop body small.
#if defined(__CUDA_ARCH__)
static __device__ __noinline__
#else
static inline
#endif
double2 crpow_accurate(double y, double r, double s, double se, int k)
{
    const double third = 1.0 / 3.0;
    const double r3 = (r * r) * r;
    const double g = fma(-y, r3, 1.0);
    const double rr = fma(r * g, third, r);
    const double zz = y * rr;
    const double pp = zz * zz;
    const double ppe = fma(zz, zz, -pp);
    const double qq = zz * pp;
    const double qqe = fma(zz, pp, -qq);
    const double tt = zz * ppe;
    const double dd = (qq - s) + ((qqe + tt) - se);
    const double rr2 = rr * rr;
    const double dl = -(dd * (rr2 * rr2)) * third;
#if defined(__CUDA_ARCH__)
    const double lnx = log(y) + (double)(3 * k) * 0.6931471805599453;
#else
    const double lnx = std::log(y) + (double)(3 * k) * 0.6931471805599453;
#endif
    double2 out;
    out.x = zz + (dl + zz * (kFl23Minus23 * lnx));
    const double ww = y * zz;
    const double wwe = fma(y, zz, -ww);
    out.y = ww + ((wwe + y * dl) + ww * (kFl53Minus53 * lnx));
    return out;
}

// x^fl(2/3) and x^fl(5/3), both correctly rounded (see above). x < 0 gives NaN,
// x = 0 gives 0, +inf gives +inf, NaN propagates, like pow().
CRPOW_HD void pow23_53(double x, double* p23, double* p53)
{
#if defined(__CUDA_ARCH__)
    const long long xb = __double_as_longlong(x);
    const bool x_pos = xb > 0 && xb <= 0x7ff0000000000000ll;  // x > 0 (integer pipe)
#else
    const bool x_pos = x > 0.0;
#endif
    if (!x_pos) {
        const double v = (x == 0.0) ? 0.0 : (x - x) / (x - x);  // 0 or NaN
        *p23 = v;
        *p53 = v;
        return;
    }
    uint64_t b = crpow_bits(x);
    int ex = (int)((b >> 52) & 0x7FF);
    if (ex == 0x7FF) {  // inf (NaN fails x > 0 above)
        *p23 = x;
        *p53 = x;
        return;
    }
    int shift = 0;
    if (ex == 0) {  // subnormal: lift into the normal range first
        x *= crpow_exp2i(54);
        b = crpow_bits(x);
        ex = (int)((b >> 52) & 0x7FF);
        shift = 54;
    }
    const int e = ex - 1023 - shift;                   // x = m 2^e, m in [1, 2)
    const int k = (e >= 0) ? e / 3 : -((-e + 2) / 3);  // floor(e / 3)
    const int j = e - 3 * k;                           // 0, 1, 2
    const double y = crpow_from_bits((b & 0x000FFFFFFFFFFFFFull) | ((uint64_t)(1023 + j) << 52));

    const double third = 1.0 / 3.0;
    double r;
    float log2y;
    crpow_seed(y, &log2y, &r);
    {
        const double r3 = (r * r) * r;
        const double g = fma(-y, r3, 1.0);  // 1 - y r^3
        r = fma(r * g, third, r);
    }
    const double z = y * r;  // ~ y^(2/3)
    // d = z^3 - y^2 with error-free products
    const double p = z * z;
    const double pe = fma(z, z, -p);
    const double q = z * p;
    const double qe = fma(z, p, -q);
    const double t = z * pe;
    const double s = y * y;
    const double se = fma(y, y, -s);
    const double d = (q - s) + ((qe + t) - se);
    const double r2 = r * r;
    const double delta = -(d * (r2 * r2)) * third;
    // exponent offset: x^fl(2/3) = x^(2/3) (1 + (fl(2/3) - 2/3) ln x), same for 5/3;
    // ln x needs only ~1e-3 relative accuracy here (the term is ~1e-16 x^(2/3))
#if defined(__CUDA_ARCH__)
    double c2, c5;
    if (k >= -3 && k <= 2) {
        // x in [2^-9, 2^9), |ln x| < 6.3: the correction terms (< 5e-16) in
        // single precision on the FP32 pipe, off by less than 2^-74 of the result
        const float lnxf = (log2y + 3.0f * (float)k) * 0.6931472f;
        c2 = crpow_widen((float)kFl23Minus23 * lnxf);
        c5 = crpow_widen((float)kFl53Minus53 * lnxf);
    } else {
        const double lnx = (crpow_widen(log2y) + 3.0 * (double)k) * 0.6931471805599453;
        c2 = kFl23Minus23 * lnx;
        c5 = kFl53Minus53 * lnx;
    }
#else
    const double lnx = ((double)log2y + 3.0 * (double)k) * 0.6931471805599453;
    const double c2 = kFl23Minus23 * lnx, c5 = kFl53Minus53 * lnx;
#endif
    const double a23 = delta + z * c2;
    double z23 = z + a23;
    const double w0 = y * z;
    const double we = fma(y, z, -w0);
    const double a53 = (we + y * delta) + w0 * c5;
    double z53 = w0 + a53;
    // rounding test (Fast2Sum: z >= |a23|, w0 >= |a53|, so the errors are exact)
    if (crpow_near_midpoint(z23, a23 - (z23 - z)) || crpow_near_midpoint(z53, a53 - (z53 - w0))) {
        const double2 acc = crpow_accurate(y, r, s, se, k);
        z23 = acc.x;
        z53 = acc.y;
    }
    *p23 = crpow_scale(z23, 2 * k);
    *p53 = crpow_scale(z53, 5 * k);
}

CRPOW_HD double pow23(double x)
{
    double a, b;
    pow23_53(x, &a, &b);
    return a;
}

}  // namespace tr
