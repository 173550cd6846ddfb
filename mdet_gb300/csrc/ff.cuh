// ff.cuh -- float-float ("double-single") arithmetic for the exact stage.
//
// GB300 runs FP64 at a small fraction of its FP32 rate, so the exact pair
// scoring carries its double-precision quantities as unevaluated sums of two
// floats (hi + lo, |lo| <= ulp(hi)/2), about 48 significant bits.  The
// error-free transformations are Knuth's TwoSum, Dekker's Fast2Sum and the
// FMA-based TwoProd (Dekker 1971; Ogita, Rump & Oishi 2005); the compound
// operations follow the double-double algorithms of Hida, Li & Bailey (QD
// library, 2001) at float width.  exp() is this project's own: Cody-Waite
// reduction by ln 2, a 2^-4 argument scaling, a Taylor polynomial of degree 7
// evaluated in float-float, and four squarings; log() is one Newton step
// y + a e^-y - 1 from logf's value.
#pragma once

#include <cuda_runtime.h>
#include <math.h>

struct ff {
    float hi, lo;
};

__device__ __forceinline__ ff ff_make(float hi, float lo) {
    ff r;
    r.hi = hi;
    r.lo = lo;
    return r;
}

// TwoSum: s + e == a + b exactly
__device__ __forceinline__ ff two_sum(float a, float b) {
    const float s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
    return ff_make(s, e);
}

// Fast2Sum (|a| >= |b|)
__device__ __forceinline__ ff quick_two_sum(float a, float b) {
    const float s = __fadd_rn(a, b);
    const float e = __fsub_rn(b, __fsub_rn(s, a));
    return ff_make(s, e);
}

// TwoProd: p + e == a * b exactly
__device__ __forceinline__ ff two_prod(float a, float b) {
    const float p = __fmul_rn(a, b);
    const float e = __fmaf_rn(a, b, -p);
    return ff_make(p, e);
}

__device__ __forceinline__ ff ff_from_double(double d) {
    const float hi = __double2float_rn(d);
    const float lo = __double2float_rn(d - (double)hi);
    return ff_make(hi, lo);
}

__device__ __forceinline__ double ff_to_double(ff a) { return (double)a.hi + (double)a.lo; }

__device__ __forceinline__ ff ff_neg(ff a) { return ff_make(-a.hi, -a.lo); }

// accurate addition (both parts through TwoSum)
__device__ __forceinline__ ff ff_add(ff a, ff b) {
    ff s = two_sum(a.hi, b.hi);
    const ff t = two_sum(a.lo, b.lo);
    s.lo = __fadd_rn(s.lo, t.hi);
    s = quick_two_sum(s.hi, s.lo);
    s.lo = __fadd_rn(s.lo, t.lo);
    return quick_two_sum(s.hi, s.lo);
}

__device__ __forceinline__ ff ff_add_f(ff a, float b) {
    ff s = two_sum(a.hi, b);
    s.lo = __fadd_rn(s.lo, a.lo);
    return quick_two_sum(s.hi, s.lo);
}

__device__ __forceinline__ ff ff_mul(ff a, ff b) {
    ff p = two_prod(a.hi, b.hi);
    p.lo = __fmaf_rn(a.hi, b.lo, p.lo);
    p.lo = __fmaf_rn(a.lo, b.hi, p.lo);
    return quick_two_sum(p.hi, p.lo);
}

__device__ __forceinline__ ff ff_mul_f(ff a, float b) {
    ff p = two_prod(a.hi, b);
    p.lo = __fmaf_rn(a.lo, b, p.lo);
    return quick_two_sum(p.hi, p.lo);
}

// a > b, a <= b on the represented values (false when either is NaN)
__device__ __forceinline__ bool ff_gt(ff a, ff b) { return a.hi > b.hi || (a.hi == b.hi && a.lo > b.lo); }
__device__ __forceinline__ bool ff_le(ff a, ff b) { return a.hi < b.hi || (a.hi == b.hi && a.lo <= b.lo); }

// sqrt of a >= 0: one Newton correction of the float root
__device__ __forceinline__ ff ff_sqrt(ff a) {
    if (!(a.hi > 0.f)) return ff_make(a.hi == 0.f ? 0.f : __int_as_float(0x7fffffff), 0.f);
    const float y = __fsqrt_rn(a.hi);
    const ff y2 = two_prod(y, y);
    const float rem = __fadd_rn(__fsub_rn(__fsub_rn(a.hi, y2.hi), y2.lo), a.lo);
    return quick_two_sum(y, __fmul_rn(rem, __fdividef(0.5f, y)));
}

// 1 / a: one Newton correction of the float reciprocal
__device__ __forceinline__ ff ff_recip(ff a) {
    const float q = __frcp_rn(a.hi);
    // r = 1 - a*q in float-float
    const ff aq = ff_mul_f(a, q);
    const ff r = ff_add_f(ff_neg(aq), 1.f);
    return quick_two_sum(q, __fmul_rn(r.hi, q));
}

// e^a for |a| < 80
__device__ __forceinline__ ff ff_exp(ff a) {
    const ff kLn2 = ff_make(0x1.62e430p-1f, -0x1.05c610p-29f);  // ln 2
    const float k = rintf(__fmul_rn(a.hi, 1.44269504f));
    // r = a - k ln2 (k ln2 formed exactly as a float-float product)
    const ff kl = ff_mul_f(kLn2, k);
    ff r = ff_add(a, ff_neg(kl));
    r.hi = __fmul_rn(r.hi, 0.0625f);  // exact scaling by 2^-4
    r.lo = __fmul_rn(r.lo, 0.0625f);
    // Taylor coefficients 1/j!, j = 7 .. 2, as float-float
    const ff c7 = ff_make(0x1.a01a02p-13f, -0x1.7f97fap-39f);
    const ff c6 = ff_make(0x1.6c16c2p-10f, -0x1.27d27ep-35f);
    const ff c5 = ff_make(0x1.111112p-7f, -0x1.dddddep-32f);
    const ff c4 = ff_make(0x1.555556p-5f, -0x1.555556p-30f);
    const ff c3 = ff_make(0x1.555556p-3f, -0x1.555556p-28f);
    ff p = c7;
    p = ff_add(ff_mul(p, r), c6);
    p = ff_add(ff_mul(p, r), c5);
    p = ff_add(ff_mul(p, r), c4);
    p = ff_add(ff_mul(p, r), c3);
    p = ff_add_f(ff_mul(p, r), 0.5f);
    p = ff_add_f(ff_mul(p, r), 1.f);
    p = ff_add_f(ff_mul(p, r), 1.f);
#pragma unroll
    for (int i = 0; i < 4; ++i) p = ff_mul(p, p);
    const float sc = __int_as_float(((int)k + 127) << 23);  // 2^k, |k| <= 116
    return ff_make(__fmul_rn(p.hi, sc), __fmul_rn(p.lo, sc));
}

// log a for 1e-30 < a < 1e30: logf's value y (error ~1e-7) and one Newton
// step y + a e^-y - 1, which squares that error; ~1e-14 absolute.
__device__ __forceinline__ ff ff_log(ff a) {
    const ff y = ff_make(logf(a.hi), 0.f);
    const ff r = ff_add_f(ff_mul(a, ff_exp(ff_neg(y))), -1.f);
    return ff_add(y, r);
}
