// abundance.cu -- the coverage side of the graph: the pair gate of the
// abundance form (is_nz, cuda/Cuda2.cu:845-856, applied at 925) and the
// sTNF -> sSCR conversion of the edges (cuda/Cuda2.cu:1921-1971 with
// cal_abd_dist2 / cal_abd_dist 667-719, cal_abd_corr 1219-1245 and the ranks
// of cuda/ranker.h:56-80).
//
// Layout: the context keeps the reference's ABD (mean depth) and ABD_VAR
// (variance) as n x nabd row-major FP64 matrices in the original contig order,
// plus one byte per contig that says whether none of its depths exceeds 1,
// and, formed once when the depths are set, each contig's per-sample variance,
// clamped mean and CDF scale and its correlation deviations (k_abd_prep).
// sSCR runs one thread per edge over its nabd samples -- the crossing points
// of the two normal densities in float-float (abd_dist2_ff; in FP64 as the
// reference forms them where the variances are close), the four normal CDFs
// per sample in float-float from this project's erfc table, the
// correlation's cross sum --
// then three radix sorts (the abundance
// similarities, sTNF and the depth correlations) turn values into ranks and
// the ranks into quantiles of the similarity distribution.
//
// This unit is compiled without FMA contraction: sums and products round
// separately, as in the reference, so the depth correlations -- whose ranks
// pick quantiles -- come out bit-identical to a host evaluation.
#include <cub/cub.cuh>

#include "erfc_table.cuh"
#include "graph.cuh"

namespace {

// erfc in float-float from this project's own table (erfc_table.cuh,
// generated by gen_erfc_table.py): degree-13 interpolants on 26 pieces of
// [0, 6.5], absolute error ~5e-16 before the float-float evaluation; 0
// beyond 6.5 (erfc < 4e-20 there); erfc(-z) = 2 - erfc(z).  The FP32 pipes
// run this far faster than the FP64 pipe runs the double erfc.  Kept out of
// line: the score kernel calls it from eight places, and eight inlined
// copies stall the kernel on instruction fetch.
__device__ __noinline__ ff erfc_ff(ff z) {
    const bool neg = z.hi < 0.f;
    if (neg) z = ff_neg(z);
    ff r;
    if (!(z.hi < 6.5f)) {
        r = ff_make(0.f, 0.f);  // NaN arguments land here too
        if (z.hi != z.hi) return z;
    } else {
        const int p = min((int)(z.hi * 4.f), MDET_ERFC_PIECES - 1);
        // u = (z - centre) * 8, exact scaling of an exact difference
        ff u = ff_add_f(z, -((float)p + 0.5f) * 0.25f);
        u.hi *= 8.f;
        u.lo *= 8.f;
        const float(*c)[2] = kErfcTable[p];
        r = ff_make(__ldg(&c[MDET_ERFC_DEG][0]), __ldg(&c[MDET_ERFC_DEG][1]));
#pragma unroll
        for (int j = MDET_ERFC_DEG - 1; j >= 0; --j)
            r = ff_add(ff_mul(r, u), ff_make(__ldg(&c[j][0]), __ldg(&c[j][1])));
    }
    return neg ? ff_add_f(ff_neg(r), 2.f) : r;
}

// 1 / (sd * sqrt(2)) in float-float: the per-(contig, sample) factor of the
// normal CDF below.
__device__ __forceinline__ ff cdf_scale(double sd) {
    return ff_recip(ff_mul(ff_from_double(sd), ff_make(0x1.6a09e6p+0f, 0x1.9fcef4p-26f)));  // sqrt(2)
}

// Boost's normal CDF, erfc(-(x - mean) / (sd * sqrt(2))) / 2 (the function
// the reference calls), with x - mean formed in FP64 as the reference forms
// it and the rest in float-float (isd = cdf_scale(sd)); returned in double.
__device__ __forceinline__ double normal_cdf_ff(double mean, ff isd, double x) {
    const ff diff = ff_from_double(x - mean);
    const ff z = ff_mul(diff, isd);
    return ff_to_double(erfc_ff(ff_neg(z))) * 0.5;
}

// What the scoring needs of one contig's depths, formed once when the depths
// are set (everything here depends on one contig alone, so per edge it would
// be formed again for every edge the contig is in):
//   vv[i]   = s * s, s = sqrt(max(var[i], 1)) (the variance the crossing
//             points use) and isd[i] = cdf_scale(s), per sample;
//   dev[i]  = the deviation of depth i + 1 from the running mean of depths
//             0..i, i < nabd - 1, and dev[nabd - 1] = sqrt of the running
//             sum of squared deviations times i / (i + 1): the one-row steps
//             of cal_abd_corr, in its order.  The edge's correlation is then
//             (sum (dev1[i] * dev2[i]) * ratio[i]) / (sx1 * sx2): the
//             reference's operations on the reference's values.
//   ratio[i] = (i + 1) / (i + 2.0), as the reference forms it;
//   m3[i]   = the clamped mean max(abd[i], 1e-6) as three floats whose sum is
//             exactly that double (hi, mid, low), vf[i] = vv[i] in
//             float-float: the inputs of the float-float crossing points.
__global__ void k_abd_prep(const double* __restrict__ abd, const double* __restrict__ var, uint64_t n, uint32_t nabd,
                           double* __restrict__ vv, float2* __restrict__ isd, double* __restrict__ dev,
                           double* __restrict__ ratio, float4* __restrict__ m3, float2* __restrict__ vf) {
    const uint64_t t0 = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (t0 + 1 < nabd) ratio[t0] = (t0 + 1) / (t0 + 2.0);
    for (uint64_t r = t0; r < n; r += (uint64_t)gridDim.x * blockDim.x) {
        const double* a = abd + r * nabd;
        const double* w = var + r * nabd;
        double sxx = 0., mx = 0.;
        for (uint32_t i = 0; i < nabd; ++i) {
            const double u = w[i];
            const double sd = sqrt(u < 1 ? 1. : u);
            vv[r * nabd + i] = sd * sd;
            const ff f = cdf_scale(sd);
            isd[r * nabd + i] = make_float2(f.hi, f.lo);
            const ff fv = ff_from_double(sd * sd);
            vf[r * nabd + i] = make_float2(fv.hi, fv.lo);
            const double x = a[i];
            // the clamped mean as three floats that sum to it exactly
            const double mc = x < 1e-6 ? 1e-6 : x;
            const float mh = __double2float_rn(mc);
            const double r1 = mc - (double)mh;
            const float ml = __double2float_rn(r1);
            m3[r * nabd + i] = make_float4(mh, ml, __double2float_rn(r1 - (double)ml), 0.f);
            if (i == 0) {
                mx = x;
            } else {
                const double q = i / (i + 1.0);
                const double dx = x - mx;
                sxx += dx * dx * q;
                mx += dx / (i + 1.0);
                dev[r * nabd + i - 1] = dx;
            }
        }
        dev[r * nabd + nabd - 1] = sqrt(sxx);
    }
}

__global__ void k_abd_low(const double* __restrict__ abd, uint64_t n, uint32_t nabd, uint8_t* __restrict__ low) {
    for (uint64_t r = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; r < n; r += (uint64_t)gridDim.x * blockDim.x) {
        bool any = false;
        for (uint32_t i = 0; i < nabd; ++i) any = any || abd[r * nabd + i] > 1.;
        low[r] = any ? 0 : 1;
    }
}

__global__ void k_low_sorted(const uint32_t* __restrict__ perm, const uint8_t* __restrict__ low, uint64_t n,
                             uint8_t* __restrict__ out) {
    for (uint64_t s = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; s < n; s += (uint64_t)gridDim.x * blockDim.x)
        out[s] = low[perm[s]];
}


// Overlap of two normal densities from their crossing points k1 <= k2, the
// narrower distribution evaluated first (cal_abd_dist2), the FP64 form: the
// crossing points, whose numerator cancels when the variances are close, in
// FP64 in the reference's order; the four CDF values in float-float.  Used
// where abd_dist2_ff declines.
__device__ __noinline__ double abd_dist2(double m1, double v1, ff f1, double m2, double v2, ff f2) {
    double k1, k2;
    if (fabs(v2 - v1) < 1e-4) {
        k1 = k2 = (m1 + m2) / 2;
    } else {
        const double t = sqrt(v1 * v2 * ((m1 - m2) * (m1 - m2) - 2 * (v1 - v2) * log(sqrt(v2 / v1))));
        k1 = (t - m1 * v2 + m2 * v1) / (v1 - v2);
        k2 = (t + m1 * v2 - m2 * v1) / (v2 - v1);
    }
    if (k1 > k2) {
        const double x = k1;
        k1 = k2;
        k2 = x;
    }
    double ma = m1, mb = m2;
    ff fa = f1, fb = f2;
    if (v1 > v2) {
        ma = m2;
        fa = f2;
        mb = m1;
        fb = f1;
    }
    if (k1 == k2) return fabs(normal_cdf_ff(ma, fa, k1) - normal_cdf_ff(mb, fb, k1));
    return fabs(normal_cdf_ff(ma, fa, k2) - normal_cdf_ff(ma, fa, k1) + normal_cdf_ff(mb, fb, k1) - normal_cdf_ff(mb, fb, k2));
}

// k - m in float-float, m given exactly as three floats: error ~2^-48 of
// the result.
__device__ __forceinline__ ff ff_sub_m3(ff k, float4 m) {
    ff s = two_sum(k.hi, -m.x);
    s = ff_add_f(s, k.lo);
    s = ff_add_f(s, -m.y);
    return ff_add_f(s, -m.z);
}

// twice the normal CDF at k (erfc of the scaled difference), in double
__device__ __forceinline__ double cdf2_at(ff k, float4 m, ff isd) {
    return ff_to_double(erfc_ff(ff_neg(ff_mul(ff_sub_m3(k, m), isd))));
}

// cal_abd_dist2 with the crossing points in float-float.  At the crossing
// points the two densities are equal, so the overlap is stationary in k1
// and k2: an error e in either moves it by O((e / sd)^2).  Where the
// variances differ by at least 1e-3 of the larger one, the crossing points'
// cancellation is bounded by that ratio, and float-float places them within
// ~1e-9 sd of the true points (the reference's FP64 points are nearer
// still), so the overlap agrees with the reference's to ~1e-18 -- far inside
// the CDFs' own error.  The CDF arguments are formed from the three-float
// means to float-float accuracy, and the four CDF values are combined in
// FP64 in the reference's order, as in the FP64 path: the combination needs
// FP64, since for far-apart distributions 1 - d is small and must keep its
// relative accuracy.  Returns -1 where the FP64 path decides instead: closer
// variances, values out of the float-float range, crossing points that do
// not separate.
__device__ __forceinline__ double abd_dist2_ff(float4 mm1, float4 mm2, ff vf1, ff vf2, ff f1, ff f2) {
    // in FP32: variances (>= 1) this far apart also pass the reference's own
    // |v2 - v1| >= 1e-4 test, and their order is that of the FP64 values
    if (!(fabsf(vf1.hi - vf2.hi) >= 1e-3f * fmaxf(vf1.hi, vf2.hi))) return -1.;
    const ff q = ff_mul(vf2, ff_recip(vf1));
    if (!(q.hi > 1e-30f && q.hi < 1e30f && vf1.hi < 1e15f && vf2.hi < 1e15f && mm1.x < 1e15f && mm2.x < 1e15f))
        return -1.;
    const ff m1 = ff_make(mm1.x, mm1.y), m2 = ff_make(mm2.x, mm2.y);
    const ff L = ff_log(q);  // 2 log(sqrt(v2 / v1))
    const ff dm = ff_add(m1, ff_neg(m2));
    const ff dv = ff_add(vf1, ff_neg(vf2));
    // t = sqrt(v1 v2 ((m1 - m2)^2 - 2 (v1 - v2) log(sqrt(v2 / v1))))
    const ff A = ff_add(ff_mul(dm, dm), ff_neg(ff_mul(dv, L)));
    const ff t = ff_sqrt(ff_mul(ff_mul(vf1, vf2), A));
    const ff c = ff_add(ff_mul(m1, vf2), ff_neg(ff_mul(m2, vf1)));  // m1 v2 - m2 v1
    const ff idv = ff_recip(dv);
    ff k1 = ff_mul(ff_add(t, ff_neg(c)), idv);  // (t - m1 v2 + m2 v1) / (v1 - v2)
    ff k2 = ff_mul(ff_add(t, c), ff_neg(idv));  // (t + m1 v2 - m2 v1) / (v2 - v1)
    if (!(fabsf(k1.hi) < 1e30f && fabsf(k2.hi) < 1e30f &&
          fabsf(k1.hi - k2.hi) > 0x1p-30f * (fabsf(k1.hi) + fabsf(k2.hi))))
        return -1.;
    if (ff_gt(k1, k2)) {
        const ff x = k1;
        k1 = k2;
        k2 = x;
    }
    float4 ma = mm1, mb = mm2;
    ff fa = f1, fb = f2;
    if (vf1.hi > vf2.hi) {
        ma = mm2;
        fa = f2;
        mb = mm1;
        fb = f1;
    }
    // the reference's sum of the four halved values, halved once at the end
    // (scaling by 1/2 commutes with every rounding here)
    return fabs(cdf2_at(k2, ma, fa) - cdf2_at(k1, ma, fa) + cdf2_at(k1, mb, fb) - cdf2_at(k2, mb, fb)) * 0.5;
}

struct ScoreArgs {
    const uint64_t* from;
    const uint64_t* to;
    uint64_t ne, n;
    const double* abd;
    const double* vv;     // per contig and sample (k_abd_prep)
    const float2* isd;
    const float4* m3;
    const float2* vf;
    const double* dev;
    const double* ratio;
    uint32_t nabd;
    double min_cv;
    bool corr;
    double* raw;     // mean abundance similarity per edge
    uint32_t* nnz;   // samples where either depth exceeds min_cv
    double* cor;     // depth correlation per edge (corr only)
    uint32_t* idx;   // 0 .. ne-1, the values of the rank sorts
    unsigned long long* bad;  // edges with an index out of range or no covered sample
};

// One thread per edge: r1 = to[e], r2 = from[e] (the reference's order).
__global__ void k_abd_score(ScoreArgs p) {
    for (uint64_t e = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; e < p.ne;
         e += (uint64_t)gridDim.x * blockDim.x) {
        p.idx[e] = (uint32_t)e;
        const uint64_t r1 = p.to[e], r2 = p.from[e];
        if (r1 >= p.n || r2 >= p.n) {
            atomicAdd(p.bad, 1ull);
            p.raw[e] = 0.;
            p.nnz[e] = 0;
            if (p.corr) p.cor[e] = 0.;
            continue;
        }
        const double* a1 = p.abd + r1 * p.nabd;
        const double* a2 = p.abd + r2 * p.nabd;
        const double* q1 = p.vv + r1 * p.nabd;
        const double* q2 = p.vv + r2 * p.nabd;
        const float2* f1 = p.isd + r1 * p.nabd;
        const float2* f2 = p.isd + r2 * p.nabd;
        const double* d1 = p.dev + r1 * p.nabd;
        const double* d2 = p.dev + r2 * p.nabd;
        double sum = 0.;
        uint32_t k = 0;
        // the cross sum of the Pearson correlation (cal_abd_corr), from the
        // rows' own deviations
        double sxy = 0.;
        for (uint32_t i = 0; i < p.nabd; ++i) {
            const double x = a1[i], y = a2[i];
            // cal_abd_dist for sample i
            if (x > p.min_cv || y > p.min_cv) {
                double d = 0.;
                const double m1 = x < 1e-6 ? 1e-6 : x, m2 = y < 1e-6 ? 1e-6 : y;
                if (m1 != m2) {
                    const float2 g1 = f1[i], g2 = f2[i];
                    const float2 w1 = p.vf[r1 * p.nabd + i], w2 = p.vf[r2 * p.nabd + i];
                    d = abd_dist2_ff(p.m3[r1 * p.nabd + i], p.m3[r2 * p.nabd + i], ff_make(w1.x, w1.y),
                                     ff_make(w2.x, w2.y), ff_make(g1.x, g1.y), ff_make(g2.x, g2.y));
                    if (d < 0.) d = abd_dist2(m1, q1[i], ff_make(g1.x, g1.y), m2, q2[i], ff_make(g2.x, g2.y));
                }
                d = d < 1e-6 ? 1e-6 : d;  // std::min(std::max(d, 1e-6), 1 - 1e-6), NaN kept
                d = (1. - 1e-6) < d ? 1. - 1e-6 : d;
                sum += 1. - d;
                ++k;
            }
            if (i > 0) sxy += d1[i - 1] * d2[i - 1] * __ldg(p.ratio + i - 1);
        }
        if (k == 0) atomicAdd(p.bad, 1ull);
        p.raw[e] = sum / (double)k;
        p.nnz[e] = k;
        if (p.corr) p.cor[e] = sxy / (d1[p.nabd - 1] * d2[p.nabd - 1]);
    }
}

// Sorted position p starts its run of equal keys: p, else 0 (a max-scan then
// gives every position the start of its run).
__global__ void k_run_heads(const double* __restrict__ keys, uint64_t ne, uint32_t* __restrict__ head) {
    for (uint64_t q = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; q < ne; q += (uint64_t)gridDim.x * blockDim.x)
        head[q] = (q == 0 || keys[q] != keys[q - 1]) ? (uint32_t)q : 0u;
}

// Ranks from the run starts: ascending sort -> the run's first rank ("min");
// descending sort -> the run's last rank in ascending order ("max").
__global__ void k_run_ranks(const uint32_t* __restrict__ order, const uint32_t* __restrict__ start, uint64_t ne,
                            bool descending, uint32_t* __restrict__ rank) {
    for (uint64_t q = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; q < ne; q += (uint64_t)gridDim.x * blockDim.x)
        rank[order[q]] = descending ? (uint32_t)(ne - start[q]) : start[q] + 1u;
}

// The weighted geometric mean pow(raw, 1 - w) * pow(t, w), w = 1 / (1 + nnz)
// (times the correlation's quantile, square-rooted, with enough samples),
// as exp((1 - w) log raw + w log t) in float-float: ff_log and ff_exp are
// good to ~1e-14, so sSCR is within ~1e-13 relative of the reference's FP64
// pows (the values lie in [1e-6, 1]: every similarity term is at least
// 1e-6).  The three FP64 pows cost ~250 FP64 operations an edge.
__global__ void k_sscr(const double* __restrict__ raw, const uint32_t* __restrict__ nnz,
                       const uint32_t* __restrict__ rt, const uint32_t* __restrict__ rc,
                       const double* __restrict__ distr, uint64_t ne, bool corr, double* __restrict__ out) {
    for (uint64_t e = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; e < ne; e += (uint64_t)gridDim.x * blockDim.x) {
        const ff t = ff_from_double(distr[rt[e] - 1]);
        const ff w = ff_recip(ff_make((float)(1 + nnz[e]), 0.f));
        const ff l = ff_add(ff_mul(ff_add_f(ff_neg(w), 1.f), ff_log(ff_from_double(raw[e]))), ff_mul(w, ff_log(t)));
        const ff sc = ff_exp(l);
        out[e] = ff_to_double(corr ? ff_sqrt(ff_mul(sc, ff_from_double(distr[rc[e] - 1]))) : sc);
    }
}

struct MaxOp {
    __device__ __forceinline__ uint32_t operator()(uint32_t a, uint32_t b) const { return a > b ? a : b; }
};

unsigned grid_for(mdet_ctx* ctx, uint64_t items, unsigned block) {
    const uint64_t want = (items + block - 1) / block, cap = (uint64_t)ctx->num_sms * 16;
    return (unsigned)(want < 1 ? 1 : (want < cap ? want : cap));
}

// ranks of keys[0..ne) into rank (ascending "min" or, descending, "max")
int rank_runs(mdet_ctx* ctx, const double* keys, const uint32_t* idx, uint64_t ne, bool descending, double* ks,
              uint32_t* os, uint32_t* head, uint32_t* start, uint32_t* rank, void* tmp, size_t tmpb) {
    cudaStream_t s = ctx->stream;
    size_t tb = tmpb;
    if (descending)
        MDET_CUDA(ctx, cub::DeviceRadixSort::SortPairsDescending(tmp, tb, keys, ks, idx, os, (int)ne, 0, 64, s));
    else
        MDET_CUDA(ctx, cub::DeviceRadixSort::SortPairs(tmp, tb, keys, ks, idx, os, (int)ne, 0, 64, s));
    k_run_heads<<<grid_for(ctx, ne, 256), 256, 0, s>>>(ks, ne, head);
    MDET_LAUNCHED(ctx, "k_run_heads");
    tb = tmpb;
    MDET_CUDA(ctx, cub::DeviceScan::InclusiveScan(tmp, tb, head, start, MaxOp(), (int)ne, s));
    k_run_ranks<<<grid_for(ctx, ne, 256), 256, 0, s>>>(os, start, ne, descending, rank);
    MDET_LAUNCHED(ctx, "k_run_ranks");
    return MDET_OK;
}

int sscr_core(mdet_ctx* ctx, const uint64_t* from, const uint64_t* to, const double* stnf, uint64_t ne,
              double min_cv, uint32_t min_sample, double* out) {
    cudaStream_t s = ctx->stream;
    if (ne == 0) return MDET_OK;
    if (ctx->abd_nabd == 0) {  // no abundance: sSCR = sTNF
        MDET_CUDA(ctx, cudaMemcpyAsync(out, stnf, ne * 8, cudaMemcpyDeviceToDevice, s));
        return MDET_OK;
    }
    if (ne >= (1ull << 31)) return ctx_fail(ctx, MDET_ERR_INVALID, "too many edges (%llu)", (unsigned long long)ne);
    const bool corr = ctx->abd_nabd >= min_sample;
    double* raw = (double*)ctx_scratch(ctx, "abd.raw", ne * 8);
    uint32_t* nnz = (uint32_t*)ctx_scratch(ctx, "abd.nnz", ne * 4);
    double* cor = (double*)ctx_scratch(ctx, "abd.cor", ne * 8);
    uint32_t* idx = (uint32_t*)ctx_scratch(ctx, "abd.idx", ne * 4);
    double* ks = (double*)ctx_scratch(ctx, "abd.ks", ne * 8);
    uint32_t* os = (uint32_t*)ctx_scratch(ctx, "abd.os", ne * 4);
    uint32_t* head = (uint32_t*)ctx_scratch(ctx, "abd.head", ne * 4);
    uint32_t* start = (uint32_t*)ctx_scratch(ctx, "abd.start", ne * 4);
    uint32_t* rt = (uint32_t*)ctx_scratch(ctx, "abd.rt", ne * 4);
    uint32_t* rc = (uint32_t*)ctx_scratch(ctx, "abd.rc", ne * 4);
    double* distr = (double*)ctx_scratch(ctx, "abd.distr", ne * 8);
    unsigned long long* bad = (unsigned long long*)ctx_scratch(ctx, "abd.bad", 8);
    if (!raw || !nnz || !cor || !idx || !ks || !os || !head || !start || !rt || !rc || !distr || !bad)
        return MDET_ERR_NOMEM;
    size_t t1 = 0, t2 = 0, t3 = 0, t4 = 0;
    MDET_CUDA(ctx, cub::DeviceRadixSort::SortKeys(nullptr, t1, raw, distr, (int)ne, 0, 64, s));
    MDET_CUDA(ctx, cub::DeviceRadixSort::SortPairs(nullptr, t2, stnf, ks, idx, os, (int)ne, 0, 64, s));
    MDET_CUDA(ctx, cub::DeviceRadixSort::SortPairsDescending(nullptr, t3, cor, ks, idx, os, (int)ne, 0, 64, s));
    MDET_CUDA(ctx, cub::DeviceScan::InclusiveScan(nullptr, t4, head, start, MaxOp(), (int)ne, s));
    const size_t tmpb = std::max(std::max(t1, t2), std::max(t3, t4));
    void* tmp = ctx_scratch(ctx, "abd.cubtmp", tmpb);
    if (!tmp) return MDET_ERR_NOMEM;
    MDET_CUDA(ctx, cudaMemsetAsync(bad, 0, 8, s));

    ScoreArgs p;
    p.from = from;
    p.to = to;
    p.ne = ne;
    p.n = ctx->abd_n;
    p.abd = (const double*)ctx->bufs["abd.m"].p;
    p.vv = (const double*)ctx->bufs["abd.vv"].p;
    p.isd = (const float2*)ctx->bufs["abd.isd"].p;
    p.dev = (const double*)ctx->bufs["abd.dev"].p;
    p.ratio = (const double*)ctx->bufs["abd.ratio"].p;
    p.m3 = (const float4*)ctx->bufs["abd.m3"].p;
    p.vf = (const float2*)ctx->bufs["abd.vf"].p;
    p.nabd = ctx->abd_nabd;
    p.min_cv = min_cv;
    p.corr = corr;
    p.raw = raw;
    p.nnz = nnz;
    p.cor = cor;
    p.idx = idx;
    p.bad = bad;
    ctx_timer_begin(ctx, "k_abd_score");
    k_abd_score<<<grid_for(ctx, ne, 128), 128, 0, s>>>(p);
    ctx_timer_end(ctx, "k_abd_score");
    MDET_LAUNCHED(ctx, "k_abd_score");

    // the abundance similarities in ascending order (partial_sort_copy)
    ctx_timer_begin(ctx, "abd_ranks");
    size_t tb = tmpb;
    MDET_CUDA(ctx, cub::DeviceRadixSort::SortKeys(tmp, tb, raw, distr, (int)ne, 0, 64, s));
    MDET_TRY(rank_runs(ctx, stnf, idx, ne, false, ks, os, head, start, rt, tmp, tmpb));
    if (corr) MDET_TRY(rank_runs(ctx, cor, idx, ne, true, ks, os, head, start, rc, tmp, tmpb));
    ctx_timer_end(ctx, "abd_ranks");
    ctx_timer_begin(ctx, "k_sscr");
    k_sscr<<<grid_for(ctx, ne, 256), 256, 0, s>>>(raw, nnz, rt, rc, distr, ne, corr, out);
    ctx_timer_end(ctx, "k_sscr");
    MDET_LAUNCHED(ctx, "k_sscr");

    unsigned long long nbad = 0;
    MDET_CUDA(ctx, cudaMemcpyAsync(&nbad, bad, 8, cudaMemcpyDeviceToHost, s));
    MDET_CUDA(ctx, cudaStreamSynchronize(s));
    if (nbad)
        return ctx_fail(ctx, MDET_ERR_INVALID,
                        "%llu edges have a contig index out of range or no sample with depth above min_cv",
                        (unsigned long long)nbad);
    return MDET_OK;
}

}  // namespace

int abd_gate(mdet_ctx* ctx, GraphPrep& g) {
    g.low = nullptr;
    if (ctx->abd_nabd == 0) return MDET_OK;
    if (ctx->abd_n != g.n)
        return ctx_fail(ctx, MDET_ERR_INVALID, "the abundance set on the context covers %llu contigs, the graph %llu",
                        (unsigned long long)ctx->abd_n, (unsigned long long)g.n);
    uint8_t* low_s = (uint8_t*)ctx_scratch(ctx, "abd.lows", g.n);
    if (!low_s) return MDET_ERR_NOMEM;
    k_low_sorted<<<grid_for(ctx, g.n, 256), 256, 0, ctx->stream>>>(g.perm, (const uint8_t*)ctx->bufs["abd.low"].p,
                                                                    g.n, low_s);
    MDET_LAUNCHED(ctx, "k_low_sorted");
    g.low = low_s;
    return MDET_OK;
}

extern "C" {

int mdet_ctx_set_abundance(mdet_ctx* ctx, const double* abd, const double* abd_var, uint64_t n, uint32_t nabd) {
    if (!ctx) return MDET_ERR_INVALID;
    MDET_CUDA(ctx, cudaSetDevice(ctx->device));
    if (nabd == 0 || n == 0 || !abd) {
        ctx->abd_n = 0;
        ctx->abd_nabd = 0;
        return MDET_OK;
    }
    if (!abd_var) return ctx_fail(ctx, MDET_ERR_INVALID, "null variance matrix");
    if (n >= (1ull << 31)) return ctx_fail(ctx, MDET_ERR_INVALID, "too many contigs");
    cudaStream_t s = ctx->stream;
    double* dm = (double*)ctx_scratch(ctx, "abd.m", n * nabd * 8);
    double* dv = (double*)ctx_scratch(ctx, "abd.v", n * nabd * 8);
    uint8_t* low = (uint8_t*)ctx_scratch(ctx, "abd.low", n);
    double* vv = (double*)ctx_scratch(ctx, "abd.vv", n * nabd * 8);
    float2* isd = (float2*)ctx_scratch(ctx, "abd.isd", n * nabd * 8);
    double* dev = (double*)ctx_scratch(ctx, "abd.dev", n * nabd * 8);
    double* ratio = (double*)ctx_scratch(ctx, "abd.ratio", nabd * 8);
    float4* m3 = (float4*)ctx_scratch(ctx, "abd.m3", n * nabd * 16);
    float2* vf = (float2*)ctx_scratch(ctx, "abd.vf", n * nabd * 8);
    if (!dm || !dv || !low || !vv || !isd || !dev || !ratio || !m3 || !vf) return MDET_ERR_NOMEM;
    MDET_CUDA(ctx, cudaMemcpyAsync(dm, abd, n * nabd * 8, cudaMemcpyHostToDevice, s));
    MDET_CUDA(ctx, cudaMemcpyAsync(dv, abd_var, n * nabd * 8, cudaMemcpyHostToDevice, s));
    k_abd_low<<<grid_for(ctx, n, 256), 256, 0, s>>>(dm, n, nabd, low);
    MDET_LAUNCHED(ctx, "k_abd_low");
    k_abd_prep<<<std::max<unsigned>(grid_for(ctx, n, 256), (nabd + 255) / 256), 256, 0, s>>>(dm, dv, n, nabd, vv,
                                                                                            isd, dev, ratio, m3, vf);
    MDET_LAUNCHED(ctx, "k_abd_prep");
    MDET_CUDA(ctx, cudaStreamSynchronize(s));
    ctx->abd_n = n;
    ctx->abd_nabd = nabd;
    return MDET_OK;
}

int mdet_edges_sscr_dev(mdet_ctx* ctx, const uint64_t* d_from, const uint64_t* d_to, const double* d_stnf,
                        uint64_t n_edges, double min_cv, uint32_t min_sample, double* d_sscr) {
    if (!ctx) return MDET_ERR_INVALID;
    MDET_CUDA(ctx, cudaSetDevice(ctx->device));
    ctx->launches = 0;
    if (n_edges && (!d_from || !d_to || !d_stnf || !d_sscr)) return ctx_fail(ctx, MDET_ERR_INVALID, "null pointer");
    return sscr_core(ctx, d_from, d_to, d_stnf, n_edges, min_cv, min_sample, d_sscr);
}

int mdet_edges_sscr(mdet_ctx* ctx, const uint64_t* from, const uint64_t* to, const double* stnf, uint64_t n_edges,
                    double min_cv, uint32_t min_sample, double* sscr) {
    if (!ctx) return MDET_ERR_INVALID;
    MDET_CUDA(ctx, cudaSetDevice(ctx->device));
    ctx->launches = 0;
    if (n_edges == 0) return MDET_OK;
    if (!from || !to || !stnf || !sscr) return ctx_fail(ctx, MDET_ERR_INVALID, "null pointer");
    cudaStream_t s = ctx->stream;
    uint64_t* df = (uint64_t*)ctx_scratch(ctx, "io.efrom", n_edges * 8);
    uint64_t* dt = (uint64_t*)ctx_scratch(ctx, "io.eto", n_edges * 8);
    double* ds = (double*)ctx_scratch(ctx, "io.estnf", n_edges * 8);
    double* dout = (double*)ctx_scratch(ctx, "io.esscr", n_edges * 8);
    if (!df || !dt || !ds || !dout) return MDET_ERR_NOMEM;
    MDET_CUDA(ctx, cudaMemcpyAsync(df, from, n_edges * 8, cudaMemcpyHostToDevice, s));
    MDET_CUDA(ctx, cudaMemcpyAsync(dt, to, n_edges * 8, cudaMemcpyHostToDevice, s));
    MDET_CUDA(ctx, cudaMemcpyAsync(ds, stnf, n_edges * 8, cudaMemcpyHostToDevice, s));
    MDET_TRY(sscr_core(ctx, df, dt, ds, n_edges, min_cv, min_sample, dout));
    MDET_CUDA(ctx, cudaMemcpyAsync(sscr, dout, n_edges * 8, cudaMemcpyDeviceToHost, s));
    MDET_CUDA(ctx, cudaStreamSynchronize(s));
    return MDET_OK;
}

}  // extern "C"
