// fast_exp.h -- exp(x) in FP64 by a table-driven method (shared by device and host code).
//
// Method: P. T. P. Tang, "Table-driven implementation of the exponential function in IEEE
// floating-point arithmetic", ACM TOMS 15(2):144-157, 1989, with N = 64 table entries:
//   x = (64 m + j) ln2/64 + r,  |r| <= ln2/128,
//   exp(x) = 2^m * 2^(j/64) * (1 + p(r)),  p(r) = r + r^2 (1/2 + r/6 + r^2/24 + r^3/120 + r^4/720).
// The reduction uses a two-part ln2/64 (the leading part has 32 significant bits, so k*L1 is
// exact for every reachable k) and fused multiply-adds; the scale by 2^m is an integer add to
// the exponent field.  Cost: 11 FP64 operations (1 mul + 10 fma/add), no division.  The table
// 2^(j/64) holds correctly rounded doubles; callers pass it in (kernels keep it in shared
// memory, where lane-divergent indices do not serialise as constant-memory reads would).
// Accuracy: within about 1 ulp of the exact value on [-745.13, 709.78]; +inf above, 0 below.
#pragma once
#ifndef __CUDACC_RTC__
#include <cstdint>
#include <cstring>
#else
typedef long long int64_t;
typedef unsigned int uint32_t;
#endif

#ifndef GDTK_HD
#ifdef __CUDACC__
#define GDTK_HD __host__ __device__ __forceinline__
#else
#define GDTK_HD inline
#endif
#endif

namespace gdtk {

// 2^(j/64), j = 0..63, correctly rounded.
#define GDTK_EXP2_TABLE_INIT { \
    0x1.0000000000000p+0, 0x1.02c9a3e778061p+0, 0x1.059b0d3158574p+0, 0x1.0874518759bc8p+0, \
    0x1.0b5586cf9890fp+0, 0x1.0e3ec32d3d1a2p+0, 0x1.11301d0125b51p+0, 0x1.1429aaea92de0p+0, \
    0x1.172b83c7d517bp+0, 0x1.1a35beb6fcb75p+0, 0x1.1d4873168b9aap+0, 0x1.2063b88628cd6p+0, \
    0x1.2387a6e756238p+0, 0x1.26b4565e27cddp+0, 0x1.29e9df51fdee1p+0, 0x1.2d285a6e4030bp+0, \
    0x1.306fe0a31b715p+0, 0x1.33c08b26416ffp+0, 0x1.371a7373aa9cbp+0, 0x1.3a7db34e59ff7p+0, \
    0x1.3dea64c123422p+0, 0x1.4160a21f72e2ap+0, 0x1.44e086061892dp+0, 0x1.486a2b5c13cd0p+0, \
    0x1.4bfdad5362a27p+0, 0x1.4f9b2769d2ca7p+0, 0x1.5342b569d4f82p+0, 0x1.56f4736b527dap+0, \
    0x1.5ab07dd485429p+0, 0x1.5e76f15ad2148p+0, 0x1.6247eb03a5585p+0, 0x1.6623882552225p+0, \
    0x1.6a09e667f3bcdp+0, 0x1.6dfb23c651a2fp+0, 0x1.71f75e8ec5f74p+0, 0x1.75feb564267c9p+0, \
    0x1.7a11473eb0187p+0, 0x1.7e2f336cf4e62p+0, 0x1.82589994cce13p+0, 0x1.868d99b4492edp+0, \
    0x1.8ace5422aa0dbp+0, 0x1.8f1ae99157736p+0, 0x1.93737b0cdc5e5p+0, 0x1.97d829fde4e50p+0, \
    0x1.9c49182a3f090p+0, 0x1.a0c667b5de565p+0, 0x1.a5503b23e255dp+0, 0x1.a9e6b5579fdbfp+0, \
    0x1.ae89f995ad3adp+0, 0x1.b33a2b84f15fbp+0, 0x1.b7f76f2fb5e47p+0, 0x1.bcc1e904bc1d2p+0, \
    0x1.c199bdd85529cp+0, 0x1.c67f12e57d14bp+0, 0x1.cb720dcef9069p+0, 0x1.d072d4a07897cp+0, \
    0x1.d5818dcfba487p+0, 0x1.da9e603db3285p+0, 0x1.dfc97337b9b5fp+0, 0x1.e502ee78b3ff6p+0, \
    0x1.ea4afa2a490dap+0, 0x1.efa1bee615a27p+0, 0x1.f50765b6e4540p+0, 0x1.fa7c1819e90d8p+0, \
}

GDTK_HD int64_t gdtk_bits(double x) {
#ifdef __CUDA_ARCH__
    return __double_as_longlong(x);
#else
    int64_t b;
    std::memcpy(&b, &x, 8);
    return b;
#endif

}

GDTK_HD double gdtk_from_bits(int64_t b) {
#ifdef __CUDA_ARCH__
    return __longlong_as_double(b);
#else
    double x;
    std::memcpy(&x, &b, 8);
    return x;
#endif
}

GDTK_HD double gdtk_fma(double a, double b, double c) {
#ifdef __CUDA_ARCH__
    return __fma_rn(a, b, c);
#else
    return __builtin_fma(a, b, c);
#endif
}

GDTK_HD double gdtk_exp(double x, const double* tab) {
    const double INV_L = 0x1.71547652b82fep+6;   // 64 / ln 2
    const double L1 = 0x1.62e42fee00000p-7;      // ln2/64, leading 32 bits
    const double L2 = 0x1.a39ef35793c76p-39;     // ln2/64 - L1
    const double SHIFT = 0x1.8p52;               // round-to-integer shift
    // |x| < 512 (biased exponent below 1032), tested on the bits: the result is normal and the
    // scaling below needs no range check.  NaN, infinities and the range ends take the compares.
    const bool inner = ((gdtk_bits(x) >> 52) & 0x7ff) < 1032;
    if (!inner) {
        if (!(x > -745.1332191019412)) return x != x ? x : 0.0;
        if (x > 709.782712893384) return x * 0x1p1023;   // +inf
    }
    double t = gdtk_fma(x, INV_L, SHIFT);
    int k = (int)(uint32_t)(gdtk_bits(t) & 0xffffffff);
    double kd = t - SHIFT;
    double r = gdtk_fma(-kd, L1, x);
    r = gdtk_fma(-kd, L2, r);
    double r2 = r * r;
    double q = gdtk_fma(1.0 / 720.0, r, 1.0 / 120.0);
    q = gdtk_fma(q, r, 1.0 / 24.0);
    q = gdtk_fma(q, r, 1.0 / 6.0);
    q = gdtk_fma(q, r, 0.5);
    double p = gdtk_fma(r2, q, r);
    double T = tab[k & 63];
    double y = gdtk_fma(T, p, T);
    int m = k >> 6;
    if (inner || (m >= -1020 && m <= 1022)) return gdtk_from_bits(gdtk_bits(y) + ((int64_t)m << 52));
    // near the ends of the range: scale in two exact-power steps (the second may round
    // into the subnormal range, as the true result does)
    int m1 = m / 2, m2 = m - m1;
    double s1 = gdtk_from_bits((int64_t)(1023 + m1) << 52);
    double s2 = gdtk_from_bits((int64_t)(1023 + m2) << 52);
    return (y * s1) * s2;
}

#ifdef __CUDA_ARCH__
static __device__ __noinline__ double gdtk_div_ieee(double a, double b) { return a / b; }
#endif

// a / b in FP64 in a few instructions: the hardware's approximate reciprocal y0
// (rcp.approx.ftz.f64), one cubically convergent Newton-Raphson step y = y0 (1 + e + e^2),
// e = 1 - b y0, then one correction of the quotient, q = a y + (a - b a y) y, whose remainder
// term is exact in a fused multiply-add (P. Markstein, "Computation of elementary functions on
// the IBM RISC System/6000 processor", IBM J. Res. Develop. 34(1):111-119, 1990).  The result is
// within 1 ulp of the correctly rounded quotient (almost always equal to it) when b and the
// quotient lie in [2^-999, 2^1001); outside that range, and for zero, infinite or NaN operands,
// the IEEE division runs instead (one shared out-of-line copy).  Five FMA/multiplies, no branch
// in the common case; the inline IEEE division is many times larger, and this kernel's loop is
// limited by instruction fetch.
GDTK_HD double gdtk_div(double a, double b) {
#ifdef __CUDA_ARCH__
    double y;
    asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(y) : "d"(b));
    const double e = __fma_rn(-b, y, 1.0);
    y = __fma_rn(y, __fma_rn(e, e, e), y);
    const double q = a * y;
    const double res = __fma_rn(__fma_rn(-b, q, a), y, q);
    const unsigned eb = (unsigned)(__double_as_longlong(b) >> 52) & 0x7ffu;
    const unsigned eq = (unsigned)(__double_as_longlong(res) >> 52) & 0x7ffu;
    if (eb - 24u < 2000u) {
        if (eq - 24u < 2000u) return res;
        if (a == 0.0) return q;   // a signed zero, as a / b
    }
    return gdtk_div_ieee(a, b);
#else
    return a / b;
#endif
}

// a / b within 2 ulp, one FMA cheaper than gdtk_div: the same reciprocal y (the approximation refined by
// one cubically convergent Newton-Raphson step, within about 1 ulp of 1/b) times a, without the
// quotient correction.  The same range rules and IEEE fallback as gdtk_div.  The chemistry kernel's
// divisions need no more: its results are compared with the reference at 1e-8, not bitwise.
GDTK_HD double gdtk_div_nr(double a, double b) {
#ifdef __CUDA_ARCH__
    double y;
    asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(y) : "d"(b));
    const double e = __fma_rn(-b, y, 1.0);
    y = __fma_rn(y, __fma_rn(e, e, e), y);
    const double q = a * y;
    const unsigned eb = (unsigned)(__double_as_longlong(b) >> 52) & 0x7ffu;
    const unsigned eq = (unsigned)(__double_as_longlong(q) >> 52) & 0x7ffu;
    if (eb - 24u < 2000u) {
        if (eq - 24u < 2000u) return q;
        if (a == 0.0) return q;
    }
    return gdtk_div_ieee(a, b);
#else
    return a / b;
#endif
}

}  // namespace gdtk
