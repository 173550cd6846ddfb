// lp_math.h -- the double-precision exp, log and chi-squared CDF of label
// propagation, written with IEEE-754 basic operations only (+ - * /, and
// frexp/ldexp, which are exact), so that a host build without contraction of
// a*b+c (-ffp-contract=off) and a device build without it (-fmad=false) give
// bit-identical results.  Label propagation picks, per contig, the label
// with the largest chi-squared CDF and breaks exact ties by a fixed order, so
// the device and the host checkers must agree to the last bit.
//
// Methods (all standard, written here from the mathematics):
//  * exp: Cody-Waite reduction z = k ln2 + r with ln2 split into a 32-bit
//    head (k * head exact) and a tail; e^r by the Taylor series to degree 13
//    (|r| <= ln2/2, truncation below 4e-18); scaling by 2^k with ldexp.
//  * log: x = m 2^e with m in [sqrt(1/2), sqrt(2)); log m = 2 atanh(s),
//    s = (m-1)/(m+1), by the odd series of atanh to s^23 (|s| <= 0.172).
//  * the chi-squared CDF with 2c degrees of freedom at x is the regularised
//    lower incomplete gamma P(c, y), y = x/2, for integer c (lpm::chi2_cdf in
//    double; lpf::chi2_cdf, the one label propagation uses, in float-float
//    with the same series, below):
//      y <  c:  P = pois(c; y) * sum_k y^k / ((c+1)...(c+k))
//      y >= c:  P = 1 - pois(c-1; y) * sum_{i<c} (c-1)!/i! y^(i-c+1)
//    with pois(j; y) = exp(-y + j log y - log j!) and log j! summed in order;
//    the series' divisions are multiplications by reciprocals (1/(c+k) and
//    1/y), which a device table can supply without changing a bit.
//    This replaces boost::math::cdf(chi_squared(2c), x), which the reference
//    calls (cuda/Cuda2.cu:611-616); Boost is not used here.
#pragma once

#include <cmath>
#include <cstdint>

#if defined(__CUDACC__)
#define LP_HD __host__ __device__ __forceinline__
#else
#define LP_HD inline
#endif

namespace lpm {

constexpr double kLn2Hi = 0x1.62e42fee00000p-1;  // ln 2 to 32 fraction bits
constexpr double kLn2Lo = 0x1.a39ef35793c76p-33; // ln 2 - kLn2Hi
constexpr double kInvLn2 = 0x1.71547652b82fep+0;
constexpr double kSqrtHalf = 0x1.6a09e667f3bcdp-1;

LP_HD double exp(double z) {
    if (z != z) return z;
    if (z > 709.0) return INFINITY;
    if (z < -745.5) return 0.0;
    const double kd = floor(z * kInvLn2 + 0.5);
    const double r = (z - kd * kLn2Hi) - kd * kLn2Lo;
    double p = 1.0 / 6227020800.0;  // 1/13!
    p = p * r + 1.0 / 479001600.0;
    p = p * r + 1.0 / 39916800.0;
    p = p * r + 1.0 / 3628800.0;
    p = p * r + 1.0 / 362880.0;
    p = p * r + 1.0 / 40320.0;
    p = p * r + 1.0 / 5040.0;
    p = p * r + 1.0 / 720.0;
    p = p * r + 1.0 / 120.0;
    p = p * r + 1.0 / 24.0;
    p = p * r + 1.0 / 6.0;
    p = p * r + 0.5;
    p = p * r + 1.0;
    p = p * r + 1.0;
    const int k = (int)kd;
    // two steps keep the intermediate normal when 2^k alone is subnormal
    if (k < -1000) return ldexp(ldexp(p, k + 64), -64);
    return ldexp(p, k);
}

LP_HD double log(double x) {
    if (x != x || x < 0) return NAN;
    if (x == 0) return -INFINITY;
    if (x == INFINITY) return x;
    int e = 0;
    double m = frexp(x, &e);  // [0.5, 1)
    if (m < kSqrtHalf) {
        m = m * 2.0;
        e -= 1;
    }
    const double s = (m - 1.0) / (m + 1.0);
    const double s2 = s * s;
    double q = 1.0 / 23.0;
    q = q * s2 + 1.0 / 21.0;
    q = q * s2 + 1.0 / 19.0;
    q = q * s2 + 1.0 / 17.0;
    q = q * s2 + 1.0 / 15.0;
    q = q * s2 + 1.0 / 13.0;
    q = q * s2 + 1.0 / 11.0;
    q = q * s2 + 1.0 / 9.0;
    q = q * s2 + 1.0 / 7.0;
    q = q * s2 + 1.0 / 5.0;
    q = q * s2 + 1.0 / 3.0;
    const double t = s + (s * s2) * q;
    const double de = (double)e;
    return de * kLn2Hi + (de * kLn2Lo + 2.0 * t);
}

// log(j!) for j = 0..count-1 into out, summed in increasing j
LP_HD void log_factorials(double* out, uint32_t count) {
    double acc = 0.0;
    for (uint32_t j = 0; j < count; ++j) {
        if (j >= 2) acc = acc + lpm::log((double)j);
        out[j] = acc;
    }
}

// 1/j, from recip[j] when the table holds it (recip[j] = 1.0 / j, so the
// value is the same either way; the table only spares the division)
LP_HD double inv(uint32_t j, const double* recip, uint32_t nrecip) {
    return (recip && j < nrecip) ? recip[j] : 1.0 / (double)j;
}

// recip[j] = 1.0 / j for 1 <= j < count (recip[0] = 0)
LP_HD void reciprocals(double* out, uint32_t count) {
    for (uint32_t j = 0; j < count; ++j) out[j] = j ? 1.0 / (double)j : 0.0;
}

// chi-squared CDF with dof = 2c degrees of freedom at x (c >= 1 an
// integer); logfact[j] = log(j!) for j <= c; recip (optional, nrecip
// entries) as in inv().  Each series step multiplies by a reciprocal.
LP_HD double chi2_cdf(double dof, double x, const double* logfact, const double* recip = nullptr,
                      uint32_t nrecip = 0) {
    const uint32_t c = (uint32_t)(dof * 0.5);
    const double y = x * 0.5;
    if (!(y > 0)) return 0.0;
    if (y == INFINITY) return 1.0;
    const double ly = lpm::log(y);
    if (y < (double)c) {
        const double lp = (-y + (double)c * ly) - logfact[c];
        double t = 1.0, v = 1.0;
        for (uint32_t k = 1; k < 1000000u; ++k) {
            t = (t * y) * inv(c + k, recip, nrecip);
            v = v + t;
            if (t < v * 1e-17) break;
        }
        return lpm::exp(lp) * v;
    }
    const double lq = (-y + (double)(c - 1) * ly) - logfact[c - 1];
    const double iy = 1.0 / y;
    double u = 1.0, w = 1.0;
    for (uint32_t i = c - 1; i >= 1; --i) {
        u = (u * (double)i) * iy;
        w = w + u;
        if (u < w * 1e-17) break;
    }
    return 1.0 - lpm::exp(lq) * w;
}

}  // namespace lpm

// ---------------------------------------------------------------------------
// The chi-squared CDF in float-float arithmetic: pairs of FP32 values
// (hi + lo, ~48 bits), with the error-free transforms of Knuth (TwoSum),
// Dekker (Fast2Sum) and an FMA product, as in the double-double algorithms
// of Hida, Li and Bailey at float width.  FP32 +, -, *, / and fmaf are
// correctly rounded on the host and the device alike, so without
// contraction the two give the same bits -- and GB300 runs FP32 far faster
// than FP64, which bounds the label sweeps.  The CDF's input (the sum of
// the label's log(1 - sSCR), which the reference forms in double) and its
// output are doubles.
namespace lpf {

struct F2 {
    float hi, lo;
};

LP_HD F2 make(float h, float l) {
    F2 r;
    r.hi = h;
    r.lo = l;
    return r;
}
LP_HD F2 fast_two_sum(float a, float b) {  // |a| >= |b|
    const float s = a + b;
    return make(s, b - (s - a));
}
LP_HD F2 two_sum(float a, float b) {
    const float s = a + b;
    const float bb = s - a;
    return make(s, (a - (s - bb)) + (b - bb));
}
LP_HD F2 add(F2 x, F2 y) {
    const F2 s = two_sum(x.hi, y.hi);
    return fast_two_sum(s.hi, s.lo + (x.lo + y.lo));
}
LP_HD F2 neg(F2 x) { return make(-x.hi, -x.lo); }
LP_HD F2 mul(F2 x, F2 y) {
    const float p = x.hi * y.hi;
    const float e = fmaf(x.hi, y.hi, -p);
    return fast_two_sum(p, e + (x.hi * y.lo + x.lo * y.hi));
}
LP_HD F2 mul_f(F2 x, float b) {
    const float p = x.hi * b;
    const float e = fmaf(x.hi, b, -p);
    return fast_two_sum(p, e + x.lo * b);
}
LP_HD F2 from_double(double d) {
    const float h = (float)d;
    return make(h, (float)(d - (double)h));
}
LP_HD double to_double(F2 x) { return (double)x.hi + (double)x.lo; }
// 1 / x: a float seed and one Newton step in float-float
LP_HD F2 recip(F2 x) {
    const float r = 1.0f / x.hi;
    const F2 e = add(make(1.0f, 0.0f), neg(mul_f(x, r)));  // 1 - x r
    return add(make(r, 0.0f), mul_f(e, r));
}

// ln 2 and 1 / ln 2 as float-float pairs (from the double constants above)
LP_HD F2 ln2() { return make(0x1.62e430p-1f, -0x1.05c610p-29f); }

// log of a positive finite double
LP_HD F2 log(double x) {
    int e = 0;
    double m = frexp(x, &e);
    if (m < lpm::kSqrtHalf) {
        m = m * 2.0;
        e -= 1;
    }
    const F2 mf = from_double(m);
    const F2 s = mul(add(mf, make(-1.0f, 0.0f)), lpf::recip(add(mf, make(1.0f, 0.0f))));
    const F2 s2 = mul(s, s);
    // atanh series: s (1 + s^2/3 + s^4/5 + ... + s^22/23), |s| <= 0.172
    F2 q = from_double(1.0 / 23.0);
    for (int k = 10; k >= 1; --k) q = add(mul(q, s2), from_double(1.0 / (2 * k + 1)));
    q = add(mul(q, s2), make(1.0f, 0.0f));
    const F2 t = mul(s, q);
    return add(mul_f(ln2(), (float)e), mul_f(t, 2.0f));
}

// exp of a float-float value
LP_HD F2 exp(F2 x) {
    // (below e^-87 the result would leave the float's normal range: 0)
    if (!(x.hi > -87.0f)) return make(0.0f, 0.0f);
    if (x.hi > 88.0f) return make(INFINITY, 0.0f);
    const float k = floorf(x.hi * 1.44269504f + 0.5f);
    const F2 r = add(x, neg(mul_f(ln2(), k)));  // |r| <= ~0.35
    // Taylor series to degree 14 (truncation < 1e-17 for |r| <= 0.35)
    F2 p = from_double(1.0 / 87178291200.0);  // 1/14!
    double f = 87178291200.0;
    for (int n = 13; n >= 1; --n) {
        f = f / (n + 1);
        p = add(mul(p, r), from_double(1.0 / f));
    }
    p = add(mul(p, r), make(1.0f, 0.0f));
    const int ki = (int)k;
    return make(ldexpf(p.hi, ki), ldexpf(p.lo, ki));
}

// log(j!) for j = 0..count-1, summed in increasing j
LP_HD void log_factorials(F2* out, uint32_t count) {
    F2 acc = make(0.0f, 0.0f);
    for (uint32_t j = 0; j < count; ++j) {
        if (j >= 2) acc = add(acc, lpf::log((double)j));
        out[j] = acc;
    }
}

// 1 / j as float-float: from recip[j] when the table holds it (the table
// holds the same value), else formed here
LP_HD F2 inv(uint32_t j, const F2* recip, uint32_t nrecip) {
    return (recip && j < nrecip) ? recip[j] : from_double(1.0 / (double)j);
}
LP_HD void reciprocals(F2* out, uint32_t count) {
    for (uint32_t j = 0; j < count; ++j) out[j] = j ? from_double(1.0 / (double)j) : make(0.0f, 0.0f);
}

// chi-squared CDF with dof = 2c degrees of freedom at x (c >= 1 an integer),
// the same series as lpm::chi2_cdf in float-float; logfact[j] = log(j!) for
// j <= c; recip (optional) as in inv().
LP_HD double chi2_cdf(double dof, double x, const F2* logfact, const F2* recip = nullptr, uint32_t nrecip = 0) {
    const uint32_t c = (uint32_t)(dof * 0.5);
    const double yd = x * 0.5;
    if (!(yd > 0)) return 0.0;
    if (yd == INFINITY) return 1.0;
    const F2 y = from_double(yd);
    const F2 ly = lpf::log(yd);
    if (yd < (double)c) {
        const F2 lp = add(add(mul_f(ly, (float)c), neg(y)), neg(logfact[c]));
        F2 t = make(1.0f, 0.0f), v = make(1.0f, 0.0f);
        for (uint32_t k = 1; k < 1000000u; ++k) {
            t = mul(mul(t, y), inv(c + k, recip, nrecip));
            v = add(v, t);
            if (t.hi < v.hi * 1e-17f) break;
        }
        return to_double(mul(lpf::exp(lp), v));
    }
    const F2 lq = add(add(mul_f(ly, (float)(c - 1)), neg(y)), neg(logfact[c - 1]));
    const F2 iy = lpf::recip(y);
    F2 u = make(1.0f, 0.0f), w = make(1.0f, 0.0f);
    for (uint32_t i = c - 1; i >= 1; --i) {
        u = mul(mul_f(u, (float)i), iy);
        w = add(w, u);
        if (u.hi < w.hi * 1e-17f) break;
    }
    return to_double(add(make(1.0f, 0.0f), neg(mul(lpf::exp(lq), w))));
}

}  // namespace lpf
