// exact.cuh -- exact scoring of one contig pair on the device: the
// reference's distance terms and the MetaBAT2 logistic model
// (cuda/Cuda2.cu:192-241), shared by the graph, the max-probability sample
// and the labelling of training pairs for the learned proposal.
#pragma once

#include "graph.cuh"

namespace mdet_exact {

constexpr double kLn9 = 2.1972245773362196;

__device__ __forceinline__ double horner_h(const double* h, double t) {
    return t * fma(t, fma(t, fma(t, fma(t, h[5], h[4]), h[3]), h[2]), h[1]);
}

__device__ __forceinline__ unsigned long long dkey(double v) {
    unsigned long long b = (unsigned long long)__double_as_longlong(v);
    return (b & 0x8000000000000000ull) ? ~b : (b | 0x8000000000000000ull);
}
__device__ __forceinline__ double dkey_inv(unsigned long long k) {
    unsigned long long b = (k & 0x8000000000000000ull) ? (k & 0x7fffffffffffffffull) : ~k;
    return __longlong_as_double((long long)b);
}

// d in the reference's terms float((a_k-b_k)^2) (cuda/Cuda2.cu:194-196).
// The reference adds them in FP64; FP64 throughput is scarce on this part, so
// two FP32 chains with error-free TwoSum compensation carry the sum instead
// (relative error ~1e-14, the same order as the FP64 accumulation), and only
// the final combine and sqrt run in FP64.
__device__ __forceinline__ void two_sum_acc(float& s, float& c, float t) {
    const float sum = __fadd_rn(s, t);
    const float bp = __fsub_rn(sum, s);
    const float err = __fadd_rn(__fsub_rn(s, __fsub_rn(sum, bp)), __fsub_rn(t, bp));
    s = sum;
    c = __fadd_rn(c, err);
}

__device__ __forceinline__ double exact_dist(const float* __restrict__ a, const float* __restrict__ b) {
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
    return sqrt(((double)s0 + (double)s1) + ((double)c0 + (double)c1));
}

// pre-probability of sorted contigs i, j at distance d.  need_model2: also
// evaluate the second model when the first is at or below log(9).
__device__ __forceinline__ double pre_prob(const ModelParts& pi, const ModelParts& pj, double li, double lj, double d,
                                           const ModelH& H, bool need_model2) {
    const bool imin = li <= lj;
    const ModelParts& pmin = imin ? pi : pj;
    const ModelParts& pmax = imin ? pj : pi;
    const double t = li * lj;
    double b = pmin.f[0] + pmax.g[0] + horner_h(H.h[0], t);
    double c = pmin.f[1] + pmax.g[1] + horner_h(H.h[1], t);
    double pre = -(b + c * d);
    if (pre <= kLn9) {
        if (!need_model2) return pre;
        b = pmin.f[2] + pmax.g[2] + horner_h(H.h[2], t);
        c = pmin.f[3] + pmax.g[3] + horner_h(H.h[3], t);
        pre = -(b + c * d);
        if (pre > kLn9) pre = kLn9;
    }
    return pre;
}


}  // namespace mdet_exact
