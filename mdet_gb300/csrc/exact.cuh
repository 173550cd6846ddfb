// exact.cuh -- exact scoring of one contig pair on the device: the
// reference's distance terms and the MetaBAT2 logistic model
// (cuda/Cuda2.cu:192-241), shared by the graph, the max-probability sample
// and the labelling of training pairs for the learned proposal.
#pragma once

#include "ff.cuh"
#include "graph.cuh"

namespace mdet_exact {

constexpr double kLn9 = 2.1972245773362196;

__device__ __forceinline__ unsigned long long dkey(double v) {
    unsigned long long b = (unsigned long long)__double_as_longlong(v);
    return (b & 0x8000000000000000ull) ? ~b : (b | 0x8000000000000000ull);
}
__device__ __forceinline__ double dkey_inv(unsigned long long k) {
    unsigned long long b = (k & 0x8000000000000000ull) ? (k & 0x7fffffffffffffffull) : ~k;
    return __longlong_as_double((long long)b);
}

// s + c accumulates t with the rounding error of each addition kept in c
// (TwoSum, error-free)
__device__ __forceinline__ void two_sum_acc(float& s, float& c, float t) {
    const float sum = __fadd_rn(s, t);
    const float bp = __fsub_rn(sum, s);
    const float err = __fadd_rn(__fsub_rn(s, __fsub_rn(sum, bp)), __fsub_rn(t, bp));
    s = sum;
    c = __fadd_rn(c, err);
}

// d in the reference's terms float((a_k-b_k)^2) (cuda/Cuda2.cu:194-196).
// The reference adds them in FP64; FP64 throughput is scarce on this part, so
// two FP32 chains with error-free TwoSum compensation carry the sum instead
// (relative error ~1e-14, the same order as the FP64 accumulation); the sum
// and its root are kept in float-float.
__device__ __forceinline__ ff exact_dist(const float* __restrict__ a, const float* __restrict__ b) {
    const float4* ra = reinterpret_cast<const float4*>(a);
    const float4* rb = reinterpret_cast<const float4*>(b);
    float s0 = 0.f, c0 = 0.f, s1 = 0.f, c1 = 0.f;
#pragma unroll 2
    for (int q = 0; q < MDET_NTNF / 4; ++q) {
        float4 x = __ldg(ra + q), y = __ldg(rb + q);
        float d0 = __fsub_rn(x.x, y.x), d1 = __fsub_rn(x.y, y.y), d2 = __fsub_rn(x.z, y.z), d3 = __fsub_rn(x.w, y.w);
        two_sum_acc(s0, c0, __fmul_rn(d0, d0));
        two_sum_acc(s1, c1, __fmul_rn(d1, d1));
        two_sum_acc(s0, c0, __fmul_rn(d2, d2));
        two_sum_acc(s1, c1, __fmul_rn(d3, d3));
    }
    const ff s = two_sum(s0, s1);
    const ff d2 = quick_two_sum(s.hi, __fadd_rn(__fadd_rn(c0, c1), s.lo));
    return ff_sqrt(d2);
}

__device__ __forceinline__ ff horner_h(const ff* h, ff t) {
    ff acc = h[5];
    acc = ff_add(ff_mul(acc, t), h[4]);
    acc = ff_add(ff_mul(acc, t), h[3]);
    acc = ff_add(ff_mul(acc, t), h[2]);
    acc = ff_add(ff_mul(acc, t), h[1]);
    return ff_mul(acc, t);
}

// pre-probability of contigs i, j at distance d (cuda/Cuda2.cu:199-241), in
// float-float.  need_model2: also evaluate the second model when the first
// is at or below log(9).
__device__ __forceinline__ ff pre_prob(const PartsFF& pi, const PartsFF& pj, ff d, const ModelHFF& H,
                                       bool need_model2) {
    const ff kLn9ff = ff_make(0x1.193ea8p+1f, -0x1.54bf3ep-25f);
    const bool imin = ff_le(pi.ls, pj.ls);
    const PartsFF& pmin = imin ? pi : pj;
    const PartsFF& pmax = imin ? pj : pi;
    const ff t = ff_mul(pmin.ls, pmax.ls);  // fixed operand order: the same bits for (i, j) and (j, i)
    ff b = ff_add(ff_add(pmin.f[0], pmax.g[0]), horner_h(H.h[0], t));
    ff c = ff_add(ff_add(pmin.f[1], pmax.g[1]), horner_h(H.h[1], t));
    ff pre = ff_neg(ff_add(b, ff_mul(c, d)));
    if (ff_le(pre, kLn9ff)) {
        if (!need_model2) return pre;
        b = ff_add(ff_add(pmin.f[2], pmax.g[2]), horner_h(H.h[2], t));
        c = ff_add(ff_add(pmin.f[3], pmax.g[3]), horner_h(H.h[3], t));
        pre = ff_neg(ff_add(b, ff_mul(c, d)));
        if (ff_gt(pre, kLn9ff)) pre = kLn9ff;
    }
    return pre;
}

// sTNF = 1 - 1/(1 + e^pre) (cuda/Cuda2.cu:255), returned in double
__device__ __forceinline__ double sim_of(ff pre) {
    if (pre.hi > 80.f) return 1.0;
    if (!(pre.hi > -80.f)) return 0.0;
    const ff s = ff_recip(ff_add_f(ff_exp(pre), 1.f));
    return 1.0 - ff_to_double(s);
}

}  // namespace mdet_exact
