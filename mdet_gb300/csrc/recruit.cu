// recruit.cu -- dissolving small bins and recruiting leftover and small
// contigs on the GPU (cuda/Cuda2.cu:2064-2283, after label propagation).
//
// The reference groups the large contigs into bins by label (members in
// ascending index), dissolves every bin whose sizes sum below minClsSize
// into "leftovers", replaces each depth row by its average ranks
// (cuda/ranker.h), and gives every bin with at least ten members the mean
// pairwise depth correlation of its members (cal_abd_corr,
// cuda/Cuda2.cu:1219-1245).  A leftover -- and, against the small contigs'
// own ranked depths, a small contig -- joins a bin when its mean correlation
// with the bin's first ten members and then with all members reaches the
// bin's mean; a contig that two bins accept joins none (the reference stops
// at the second, whatever order it visits the bins in, so the outcome does
// not depend on that order).  The recruits are kept when their bases stay
// under 10 % of the binned bases (leftovers) or 15 % of the small contigs'
// total (small contigs).
//
// GB300 form: the grouping, dissolving and the two gates are O(n) host work.
// On the device, each depth row is ranked and its deviations from its running
// mean taken once (k_corr_rows); a correlation is then one cross sum.  The
// bins' means are first estimated in FP32 with a proven error bound; an FP32
// prefilter drops the (contig, bin) pairs the reference's first-ten test
// provably rejects; the rest get the reference's test in FP64, term by term
// in member order.  A test whose value lands within the bound of its bin's
// estimate is decided again with a finer estimate (the FP64 terms in a fixed
// tree) and at last with the bin's exact mean (the reference's terms in the
// reference's order), so every decision is the reference's.  The unit is
// compiled without FMA contraction: every FP64 correlation and sum is
// bit-identical to a host evaluation, and the FP32 estimates use explicit
// FMAs that the bounds count.
#include <algorithm>
#include <cstdlib>
#include <utility>
#include <vector>

#include "common.cuh"

namespace {

constexpr uint32_t kMaxSamples = 256;  // depth columns a row may have
constexpr uint32_t kMinCS = 10;        // members a bin needs to recruit (the reference's minCS)
constexpr uint64_t kTermCap = 1ull << 28;  // pairwise terms held at once for the bins' means (2 GiB)

// Average ranks of each row in place (rank(rowMat, rowMat) with method
// "average", cuda/ranker.h): 1-based ascending ranks, a run of equal values
// getting the mean of its ranks, formed in float.  Thread per row; the row
// is sorted by insertion (rows are short).
__global__ void k_rank_rows(float* __restrict__ m, uint64_t rows, uint32_t nabd) {
    const uint64_t r = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (r >= rows) return;
    float v[kMaxSamples];
    uint16_t ord[kMaxSamples];
    float* row = m + r * nabd;
    for (uint32_t i = 0; i < nabd; ++i) {
        v[i] = row[i];
        ord[i] = (uint16_t)i;
    }
    for (uint32_t i = 1; i < nabd; ++i) {  // stable insertion sort of the indices by value
        const uint16_t o = ord[i];
        const float x = v[o];
        uint32_t j = i;
        while (j > 0 && x < v[ord[j - 1]]) {
            ord[j] = ord[j - 1];
            --j;
        }
        ord[j] = o;
    }
    for (uint32_t c = 0; c < nabd;) {
        uint32_t k = 1;
        while (c + k < nabd && v[ord[c]] == v[ord[c + k]]) ++k;
        const float rk = (float)(2 * c + k - 1) / 2 + 1;
        for (uint32_t q = 0; q < k; ++q) row[ord[c + q]] = rk;
        c += k;
    }
}

// The reference's correlation (cal_abd_corr) runs the two rows' means and
// squared deviations side by side, but only its cross term mixes them: the
// deviation dx_i of row x at column i from its running mean, and the sum of
// dx_i^2 i/(i+1), depend on x alone.  k_corr_rows takes those steps once per
// row, in the reference's operation order, and keeps dx_1..dx_m (m = nabd-1)
// and sqrt(sum); a correlation is then
//   r = (sum over i of (dx_i * dy_i) * ratio_i) / (sx * sy),
// the cross sum in column order from 0.0 -- the reference's operations on
// the reference's values (IEEE products commute), so the same bits.
//
// Next to the FP64 rows it keeps FP32 copies for the estimates: xf (dx_i,
// then 1 / sx) for a row in the contig role and xw (dx_i * ratio_i rounded
// to FP32, then 1 / sx) for a row in the member role.
__global__ void k_corr_rows(const float* __restrict__ m, uint64_t rows, uint32_t nabd, uint64_t row0,
                            double* __restrict__ d64, float* __restrict__ xf, float* __restrict__ xw) {
    const uint64_t r = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (r >= rows) return;
    const float* row = m + r * nabd;
    const uint64_t o = (row0 + r) * nabd;
    double sxx = 0.0, mx = row[0];
    for (uint32_t i = 1; i < nabd; ++i) {
        const double ratio = i / (i + 1.0);
        const double dx = row[i] - mx;
        sxx += dx * dx * ratio;
        mx += dx / (i + 1.0);
        d64[o + i - 1] = dx;
        xf[o + i - 1] = (float)dx;
        xw[o + i - 1] = (float)dx * (float)ratio;
    }
    const double sx = sqrt(sxx);
    d64[o + nabd - 1] = sx;
    const float inv = 1.0f / (float)sx;
    xf[o + nabd - 1] = inv;
    xw[o + nabd - 1] = inv;
}

// ratio_i = i / (i + 1.0) for i = 1..m, as the reference forms it.
__device__ __forceinline__ void load_ratios(double* ratio, uint32_t m) {
    for (uint32_t i = threadIdx.x; i < m; i += blockDim.x) ratio[i] = (i + 1) / (i + 2.0);
    __syncthreads();
}

// One correlation from two prepared FP64 rows (see k_corr_rows).
__device__ __forceinline__ double corr64(const double* __restrict__ x, const double* __restrict__ y,
                                         const double* __restrict__ ratio, uint32_t m) {
    double sxy = 0.0;
    for (uint32_t i = 0; i < m; ++i) sxy += x[i] * y[i] * ratio[i];
    return sxy / (x[m] * y[m]);
}

// FP32 correlation of a member row (xw form) with a row in the contig role
// (xf form).
__device__ __forceinline__ float corr32(const float* __restrict__ x, const float* __restrict__ y, uint32_t m) {
    float s = 0.f;
    for (uint32_t i = 0; i < m; ++i) s = __fmaf_rn(x[i], y[i], s);
    return s * (x[m] * y[m]);
}

// Error bounds.  u = 2^-24.  For rows whose 1 / sx, 1 / sy are at most
// 1 / kMinDev (every product then stays far from FP32's range limits; depth
// rows are rank vectors, so sx is 0 or well above kMinDev), an FP32
// correlation is within (m + 10.2) * 1.02 u of the exact real value rho of
// the FP64 rows: (m + 4) u from the conversions, the products dx*ratio and
// the fused dot product (|sum dx dy ratio| <= sx sy by Cauchy-Schwarz), 6 u
// from the two rounded inverses and the two products.  The reference's FP64
// correlation is within (m + 4) 2^-53 of rho.
//
// The prefilter: the FP32 sum of ten such terms is within 91 u of theirs
// and the division by ten adds 1.01 u, so an FP32 first-ten mean is within
// (1.02 m + 20.5) u of the reference's.  A pair whose FP32 mean is below the
// bin's threshold less delta = 4 (m + 32) u is one the reference's
// first-ten test rejects.
//
// A bin's mean, estimated from FP32 terms added in FP32 runs of eight, the
// runs in FP64 (per-thread sums and a fixed tree), is within
// (1.03 m + 18.5) u + (2 T + 64) 2^-53 of the
// reference's (T terms; the reference's ordered FP64 sum is within T 2^-53
// of exact per term, the tree within (T + 64) 2^-53), so within
// eps1 = 2.5 (m + 9) u + (4 T + 128) 2^-52; estimated from the FP64 terms
// themselves in a fixed tree, within eps2 = (4 T + 128) 2^-52.  A test
// whose value is at least eps from the estimate decides as the
// reference's; one within eps of it is decided again with the next
// estimate, and at last against the bin's exact mean (the reference's terms
// in the reference's order).
constexpr float kMinDev = 0x1p-20f;

double prefilter_delta(uint32_t nabd) { return 4.0 * (nabd - 1 + 32) * 0x1p-24; }

__device__ __forceinline__ double mean_eps(uint32_t m, uint64_t terms, bool fp32, double scale) {
    return scale * ((fp32 ? 2.5 * (m + 9) * 0x1p-24 : 0.0) + (4.0 * terms + 128.0) * 0x1p-52);
}

// The largest float at or below x (NaN stays NaN: the prefilter then never
// skips).
__device__ __forceinline__ float float_below(double x) {
    float f = (float)x;
    if ((double)f > x) f = nextafterf(f, -INFINITY);
    return f;
}

// The scored bins' member rows, column-major per bin (element q of the
// bin's member k at o * nabd + q * cs + k, o the bin's first member): the
// lanes of a warp on consecutive members then read consecutive words.
__global__ void k_bin_gather(const float* __restrict__ xf, const double* __restrict__ d64, uint32_t nabd,
                             const uint64_t* __restrict__ off, const uint32_t* __restrict__ mem, uint32_t nbins,
                             float* __restrict__ gf, double* __restrict__ g64) {
    for (uint32_t b = blockIdx.x; b < nbins; b += gridDim.x) {
        const uint64_t o = off[b], cs = off[b + 1] - o, base = o * nabd;
        for (uint64_t k = threadIdx.x; k < cs; k += blockDim.x) {
            const uint64_t r = (uint64_t)mem[o + k] * nabd;
            for (uint32_t q = 0; q < nabd; ++q) {
                gf[base + q * cs + k] = xf[r + q];
                g64[base + q * cs + k] = d64[r + q];
            }
        }
    }
}

// corr32 and corr64 with the second row column-major (stride cs).
__device__ __forceinline__ float corr32_col(const float* __restrict__ x, const float* __restrict__ y, uint64_t cs,
                                            uint32_t m) {
    float s = 0.f;
    for (uint32_t i = 0; i < m; ++i) s = __fmaf_rn(x[i], y[i * cs], s);
    return s * (x[m] * y[m * cs]);
}

__device__ __forceinline__ double corr64_col(const double* __restrict__ x, uint64_t cs, const double* __restrict__ y,
                                             const double* __restrict__ ratio, uint32_t m) {
    double sxy = 0.0;
    for (uint32_t i = 0; i < m; ++i) sxy += x[i * cs] * y[i] * ratio[i];
    return sxy / (x[m * cs] * y[m]);
}

// Estimated mean pairwise correlation of each scored bin: a block per bin;
// its warps take the rows i in turn, the lanes the terms (i, j) from the
// column-major rows; each thread adds its terms in FP32 runs of at most
// eight, the runs in FP64, and the block adds the threads' sums in a fixed
// tree (a run of eight adds at most 7.2 u per term to the estimate's error,
// inside eps1).  deg[b] = 1 when a member's 1 / sx is above 1 / kMinDev
// (the bound does not cover it: the bin then gets its exact mean).
__global__ void __launch_bounds__(256) k_bin_mean32(const float* __restrict__ xw, const float* __restrict__ gf,
                                                    uint32_t nabd, const uint64_t* __restrict__ off,
                                                    const uint32_t* __restrict__ mem, uint32_t nbins,
                                                    double* __restrict__ est, uint8_t* __restrict__ deg) {
    __shared__ double wsum[8];
    const uint32_t m = nabd - 1;
    const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
    for (uint32_t b = blockIdx.x; b < nbins; b += gridDim.x) {
        const uint64_t o = off[b], cs = off[b + 1] - o;
        const float* g = gf + o * nabd;
        int bad = 0;
        for (uint64_t k = threadIdx.x; k < cs; k += blockDim.x) bad |= !(g[m * cs + k] <= 1.0f / kMinDev);
        double pd = 0.0;
        float pf = 0.f;
        uint32_t run = 0;
        for (uint64_t i = warp; i + 1 < cs; i += nw) {
            const float* x = xw + (uint64_t)mem[o + i] * nabd;
            for (uint64_t j = i + 1 + lane; j < cs; j += 32) {
                pf += corr32_col(x, g + j, cs, m);
                if (++run == 8) {
                    pd += (double)pf;
                    pf = 0.f;
                    run = 0;
                }
            }
        }
        bad = __syncthreads_or(bad);
        double part = pd + (double)pf;
        for (int d = 16; d > 0; d >>= 1) part += __shfl_down_sync(0xffffffffu, part, d);
        if (lane == 0) wsum[warp] = part;
        __syncthreads();
        if (threadIdx.x == 0) {
            double t = 0.0;
            for (uint32_t w = 0; w < nw; ++w) t += wsum[w];
            est[b] = t / (double)(cs * (cs - 1) / 2);
            deg[b] = bad ? 1 : 0;
        }
        __syncthreads();
    }
}

// The reference's mean pairwise correlation of bins (cls_corr), exact: the
// terms (i, j) added in the order (0,1), (0,2), ..., (1,2), ... of the
// reference's double loop, for the bins of a list (positions [p0, p1)).
//
// A warp per bin: for member i the lanes compute the terms of 32
// consecutive j and every lane adds them in order.
__global__ void k_bin_corr(const double* __restrict__ d64, uint32_t nabd, const uint64_t* __restrict__ off,
                           const uint32_t* __restrict__ mem, const uint32_t* __restrict__ bins, uint32_t p0,
                           uint32_t p1, double* __restrict__ out) {
    __shared__ double ratio[kMaxSamples];
    const uint32_t m = nabd - 1;
    load_ratios(ratio, m);
    const uint32_t warps = (gridDim.x * blockDim.x) >> 5;
    const uint32_t lane = threadIdx.x & 31;
    for (uint32_t p = p0 + ((blockIdx.x * blockDim.x + threadIdx.x) >> 5); p < p1; p += warps) {
        const uint32_t b = bins[p];
        const uint64_t o = off[b], cs = off[b + 1] - off[b];
        double sum = 0.0;
        for (uint64_t i = 0; i < cs; ++i) {
            const double* xi = d64 + (uint64_t)mem[o + i] * nabd;
            for (uint64_t j0 = i + 1; j0 < cs; j0 += 32) {
                const uint64_t j = j0 + lane;
                const double t = j < cs ? corr64(xi, d64 + (uint64_t)mem[o + j] * nabd, ratio, m) : 0.0;
                const uint32_t cnt = (uint32_t)min((uint64_t)32, cs - j0);
                for (uint32_t q = 0; q < cnt; ++q) sum += __shfl_sync(0xffffffffu, t, q);
            }
        }
        if (lane == 0) out[b] = sum / (double)(cs * (cs - 1) / 2);
    }
}

// The same in two steps, for list positions whose terms fit a buffer: every
// term at its place in the reference's order (toff: each position's first
// term; rows of a bin of cs members start at i (2 cs - i - 1) / 2), all
// lanes busy on the FP64 correlations; then a thread per bin adds its terms
// in that order.  The adds are one dependent chain per bin, so a lane per
// bin keeps the FP64 pipe's issue slots for useful work, where a warp per
// bin would spend a warp instruction on each.
__global__ void k_bin_terms(const double* __restrict__ d64, uint32_t nabd, const uint64_t* __restrict__ off,
                            const uint32_t* __restrict__ mem, const uint32_t* __restrict__ bins,
                            const uint64_t* __restrict__ toff, uint32_t p0, uint32_t p1, double* __restrict__ term) {
    __shared__ double ratio[kMaxSamples];
    const uint32_t m = nabd - 1;
    load_ratios(ratio, m);
    const uint64_t t0 = toff[p0], nt = toff[p1] - t0;
    for (uint64_t g = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; g < nt;
         g += (uint64_t)gridDim.x * blockDim.x) {
        uint32_t lo = p0, hi = p1;  // the position: the last with toff <= t0 + g
        while (hi - lo > 1) {
            const uint32_t mid = (lo + hi) >> 1;
            if (toff[mid] <= t0 + g) lo = mid;
            else hi = mid;
        }
        const uint32_t b = bins[lo];
        const uint64_t o = off[b], cs = off[b + 1] - o, k = t0 + g - toff[lo];
        uint64_t ri = 0, rh = cs - 1;  // the row: the last i with i (2 cs - i - 1) / 2 <= k
        while (rh - ri > 1) {
            const uint64_t mid = (ri + rh) >> 1;
            if (mid * (2 * cs - mid - 1) / 2 <= k) ri = mid;
            else rh = mid;
        }
        const uint64_t j = ri + 1 + (k - ri * (2 * cs - ri - 1) / 2);
        term[g] = corr64(d64 + (uint64_t)mem[o + ri] * nabd, d64 + (uint64_t)mem[o + j] * nabd, ratio, m);
    }
}

__global__ void k_bin_sum(const double* __restrict__ term, const uint64_t* __restrict__ off,
                          const uint32_t* __restrict__ bins, const uint64_t* __restrict__ toff, uint32_t p0,
                          uint32_t p1, double* __restrict__ out) {
    const uint32_t p = p0 + blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= p1) return;
    const double* t = term + (toff[p] - toff[p0]);
    const uint64_t nt = toff[p + 1] - toff[p];
    // the next block of 16 terms is loaded while the previous one is added
    // (two register blocks in turn): the chain's adds stay in order, the
    // loads run ahead of them
    constexpr int kB = 16;
    double sum = 0.0, a[kB], c[kB];
    uint64_t k = 0;
    if (nt >= kB) {
#pragma unroll
        for (int q = 0; q < kB; ++q) a[q] = __ldcs(t + q);
        k = kB;
        for (;;) {
            const bool more_c = k + kB <= nt;
            if (more_c) {
#pragma unroll
                for (int q = 0; q < kB; ++q) c[q] = __ldcs(t + k + q);
                k += kB;
            }
#pragma unroll
            for (int q = 0; q < kB; ++q) sum += a[q];
            if (!more_c) break;
            const bool more_a = k + kB <= nt;
            if (more_a) {
#pragma unroll
                for (int q = 0; q < kB; ++q) a[q] = __ldcs(t + k + q);
                k += kB;
            }
#pragma unroll
            for (int q = 0; q < kB; ++q) sum += c[q];
            if (!more_a) break;
        }
    }
    for (; k < nt; ++k) sum += t[k];
    const uint32_t b = bins[p];
    const uint64_t cs = off[b + 1] - off[b];
    out[b] = sum / (double)(cs * (cs - 1) / 2);
}

// The second estimate of list positions [p0, p1): a block per position
// adds the bin's FP64 terms in a fixed tree (per-thread runs, then warps).
__global__ void __launch_bounds__(256) k_bin_tree(const double* __restrict__ term, const uint64_t* __restrict__ off,
                                                  const uint32_t* __restrict__ bins, const uint64_t* __restrict__ toff,
                                                  uint32_t p0, uint32_t p1, double* __restrict__ est) {
    __shared__ double wsum[8];
    const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
    for (uint32_t p = p0 + blockIdx.x; p < p1; p += gridDim.x) {
        const double* t = term + (toff[p] - toff[p0]);
        const uint64_t nt = toff[p + 1] - toff[p];
        double a0 = 0.0, a1 = 0.0;
        uint64_t k = threadIdx.x;
        for (; k + blockDim.x < nt; k += 2 * blockDim.x) {
            a0 += t[k];
            a1 += t[k + blockDim.x];
        }
        if (k < nt) a0 += t[k];
        double part = a0 + a1;
        for (int d = 16; d > 0; d >>= 1) part += __shfl_down_sync(0xffffffffu, part, d);
        if (lane == 0) wsum[warp] = part;
        __syncthreads();
        if (threadIdx.x == 0) {
            double sum = 0.0;
            for (uint32_t w = 0; w < nw; ++w) sum += wsum[w];
            const uint32_t b = bins[p];
            const uint64_t cs = off[b + 1] - off[b];
            est[b] = sum / (double)(cs * (cs - 1) / 2);
        }
        __syncthreads();
    }
}

// Per bin: the test interval [lo, hi) and the prefilter threshold, from
// the bin's best mean so far (tier[b]: 0 the FP32-term estimate, 1 the
// FP64-term estimate, 2 the exact mean, which decides every test as the
// reference's: lo = hi = the mean).
__global__ void k_bin_bounds(const double* __restrict__ est1, const double* __restrict__ est2,
                             const double* __restrict__ exact, const uint8_t* __restrict__ tier,
                             const uint64_t* __restrict__ off, uint32_t nbins, uint32_t nabd, double delta,
                             double scale, double* __restrict__ lo, double* __restrict__ hi,
                             float* __restrict__ thr) {
    const uint32_t b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= nbins) return;
    if (tier[b] == 2) {
        lo[b] = hi[b] = exact[b];
        thr[b] = float_below(exact[b] - delta);
    } else {
        const uint64_t cs = off[b + 1] - off[b];
        const double v = tier[b] == 0 ? est1[b] : est2[b];
        const double e = mean_eps(nabd - 1, cs * (cs - 1) / 2, tier[b] == 0, scale);
        lo[b] = v - e;
        hi[b] = v + e;
        thr[b] = float_below(v - e - delta);
    }
}

// A thread per contig over a chunk of bins (blockIdx.y); the lanes of a
// warp are consecutive contigs on the same bin, so a member row is one
// broadcast load.  MR > 0 keeps the contig's row in registers (m <= MR).
template <int MR>
__global__ void __launch_bounds__(256) k_recruit_filter(const float* __restrict__ xf, const float* __restrict__ xw,
                                                        uint32_t nabd, const uint32_t* __restrict__ left, uint64_t nl,
                                                        uint64_t n, uint64_t ncand, const uint64_t* __restrict__ off,
                                                        const uint32_t* __restrict__ mem, uint32_t nbins,
                                                        uint32_t chunk, const float* __restrict__ thr,
                                                        uint2* __restrict__ pass, uint64_t cap,
                                                        unsigned long long* __restrict__ npass) {
    const uint64_t cand = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (cand >= ncand) return;
    const uint32_t m = nabd - 1;
    const float* y = xf + (cand < nl ? (uint64_t)left[cand] : n + (cand - nl)) * nabd;
    float yr[MR > 0 ? MR : 1];
    if (MR > 0) {
#pragma unroll
        for (int i = 0; i < MR; ++i) yr[i] = i < (int)m ? y[i] : 0.f;
    }
    const float iy = y[m];
    const bool ok_y = iy <= 1.0f / kMinDev;
    const uint32_t b0 = blockIdx.y * chunk, b1 = min(nbins, b0 + chunk);
    for (uint32_t b = b0; b < b1; ++b) {
        const uint64_t o = off[b];
        bool maybe = !ok_y;
        float c = 0.f;
        for (uint32_t k = 0; k < kMinCS && !maybe; ++k) {
            const float* x = xw + (uint64_t)mem[o + k] * nabd;
            float s = 0.f;
            if (MR > 0) {
#pragma unroll
                for (int i = 0; i < MR; ++i)
                    if (i < (int)m) s = __fmaf_rn(x[i], yr[i], s);
            } else {
                for (uint32_t i = 0; i < m; ++i) s = __fmaf_rn(x[i], y[i], s);
            }
            const float ix = x[m];
            if (!(ix <= 1.0f / kMinDev)) maybe = true;
            c += s * (ix * iy);
        }
        if (maybe || !(c / kMinCS < thr[b])) {
            const unsigned long long k = atomicAdd(npass, 1ull);
            if (k < cap) pass[k] = make_uint2((uint32_t)cand, b);
        }
    }
}

// The reference's two-step test for the pairs the prefilter kept: a warp
// per (contig, bin); the lanes compute FP64 member correlations side by
// side and every lane adds them in member order (the first ten, the early
// stop, the rest, the division), as the reference's.  The two comparisons
// with the bin's mean use [lo, hi): a value below lo is below the mean, one
// at or above hi at or above it; a value inside (only for a bin without its
// exact mean) leaves the pair undecided -- it goes to the list amb and the
// bin is marked in need.  qcount counts the bins that accept a contig, qbin
// holds one of them (meaningful when qcount == 1).
__global__ void k_recruit_exact(const double* __restrict__ d64, const double* __restrict__ g64, uint32_t nabd,
                                const uint32_t* __restrict__ left, uint64_t nl, uint64_t n,
                                const uint64_t* __restrict__ off, const double* __restrict__ lo,
                                const double* __restrict__ hi, const uint2* __restrict__ pass, uint64_t npass,
                                uint32_t* __restrict__ qcount, uint32_t* __restrict__ qbin, uint2* __restrict__ amb,
                                unsigned long long* __restrict__ namb, uint8_t* __restrict__ need) {
    __shared__ double ratio[kMaxSamples];
    const uint32_t m = nabd - 1;
    load_ratios(ratio, m);
    const uint64_t warps = (gridDim.x * (uint64_t)blockDim.x) >> 5;
    const uint32_t lane = threadIdx.x & 31;
    for (uint64_t p = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5; p < npass; p += warps) {
        const uint2 pr = pass[p];
        const uint64_t cand = pr.x;
        const uint32_t b = pr.y;
        const double* y = d64 + (cand < nl ? (uint64_t)left[cand] : n + (cand - nl)) * nabd;
        const uint64_t o = off[b], cs = off[b + 1] - off[b];
        const double* g = g64 + o * nabd;
        const double l = lo[b], h = hi[b];
        double t = lane < kMinCS ? corr64_col(g + lane, cs, y, ratio, m) : 0.0;
        double c = 0.0;
        for (uint32_t q = 0; q < kMinCS; ++q) c += __shfl_sync(0xffffffffu, t, q);
        const double v = c / kMinCS;
        bool undecided = false;
        if (v < l) continue;  // the reference's early stop on the first ten members
        if (v < h) {
            undecided = true;
        } else {
            for (uint64_t i0 = kMinCS; i0 < cs; i0 += 32) {
                const uint64_t i = i0 + lane;
                t = i < cs ? corr64_col(g + i, cs, y, ratio, m) : 0.0;
                const uint32_t cnt = (uint32_t)min((uint64_t)32, cs - i0);
                for (uint32_t q = 0; q < cnt; ++q) c += __shfl_sync(0xffffffffu, t, q);
            }
            c /= cs;
            if (c >= h) {
                if (lane == 0) {
                    atomicAdd(&qcount[cand], 1u);
                    qbin[cand] = b;
                }
                continue;
            }
            undecided = c >= l;  // NaN and c < l: rejected
        }
        if (undecided && lane == 0) {
            amb[atomicAdd(namb, 1ull)] = pr;
            need[b] = 1;
        }
    }
}

// The contigs grouped by label: labels ascending, each group's members
// ascending (what iterating a std::map<label, vector> filled in index order
// gives), by an open-addressing table of the distinct labels, a sort of
// those, and a counting sort of the contigs.
void group_by_label(const int64_t* label, uint64_t n, std::vector<int64_t>& glabel, std::vector<uint64_t>& goff,
                    std::vector<uint32_t>& gmem) {
    uint64_t cap = 1024;
    std::vector<int64_t> key(cap);
    std::vector<uint32_t> slot(cap, UINT32_MAX);
    std::vector<int64_t> seen;  // distinct labels, first-seen order
    std::vector<uint32_t> id(n);
    auto home = [](int64_t k, uint64_t mask) {  // splitmix64's finaliser
        uint64_t x = (uint64_t)k;
        x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
        x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
        return (x ^ (x >> 31)) & mask;
    };
    for (uint64_t i = 0; i < n; ++i) {
        uint64_t h = home(label[i], cap - 1);
        while (slot[h] != UINT32_MAX && key[h] != label[i]) h = (h + 1) & (cap - 1);
        if (slot[h] == UINT32_MAX) {
            slot[h] = (uint32_t)seen.size();
            key[h] = label[i];
            seen.push_back(label[i]);
            if (seen.size() * 2 > cap) {  // grow: rehash the distinct labels
                cap *= 2;
                key.assign(cap, 0);
                slot.assign(cap, UINT32_MAX);
                for (uint32_t d = 0; d < seen.size(); ++d) {
                    uint64_t g = home(seen[d], cap - 1);
                    while (slot[g] != UINT32_MAX) g = (g + 1) & (cap - 1);
                    slot[g] = d;
                    key[g] = seen[d];
                }
                h = home(label[i], cap - 1);
                while (key[h] != label[i] || slot[h] == UINT32_MAX) h = (h + 1) & (cap - 1);
            }
        }
        id[i] = slot[h];
    }
    const uint32_t k = (uint32_t)seen.size();
    std::vector<std::pair<int64_t, uint32_t>> ord(k);
    for (uint32_t d = 0; d < k; ++d) ord[d] = {seen[d], d};
    std::sort(ord.begin(), ord.end());
    std::vector<uint32_t> rank(k);
    glabel.resize(k);
    for (uint32_t r = 0; r < k; ++r) {
        rank[ord[r].second] = r;
        glabel[r] = ord[r].first;
    }
    goff.assign(k + 1, 0);
    for (uint64_t i = 0; i < n; ++i) ++goff[rank[id[i]] + 1];
    for (uint32_t r = 0; r < k; ++r) goff[r + 1] += goff[r];
    std::vector<uint64_t> at(goff.begin(), goff.end() - 1);
    gmem.resize(n);
    for (uint64_t i = 0; i < n; ++i) gmem[at[rank[id[i]]]++] = (uint32_t)i;
}

int grid_for(mdet_ctx* ctx, uint64_t threads, int block) {
    const uint64_t blocks = (threads + block - 1) / block;
    return (int)std::min<uint64_t>(blocks, (uint64_t)ctx->num_sms * 32);
}

}  // namespace

extern "C" int mdet_recruit(mdet_ctx* ctx, const float* abd, const float* small_abd, uint64_t n, uint64_t n_small,
                            uint32_t nabd, const int64_t* label, const uint64_t* sizes, const uint64_t* small_sizes,
                            uint64_t min_cls_size, uint64_t small_total, int64_t* out, int64_t* small_out,
                            mdet_recruit_stats* st) {
    if (!ctx) return MDET_ERR_INVALID;
    MDET_CUDA(ctx, cudaSetDevice(ctx->device));
    ctx->launches = 0;
    if (st) memset(st, 0, sizeof(*st));
    if (n && (!abd || !label || !sizes || !out)) return ctx_fail(ctx, MDET_ERR_INVALID, "null pointer");
    if (n_small && (!small_abd || !small_sizes || !small_out)) return ctx_fail(ctx, MDET_ERR_INVALID, "null pointer");
    if (nabd == 0 || nabd > kMaxSamples)
        return ctx_fail(ctx, MDET_ERR_INVALID, "%u depth columns (1..%u supported)", nabd, kMaxSamples);
    if (n >= 0xFFFFFFFFull || n_small >= 0xFFFFFFFFull || n + n_small >= 0xFFFFFFFFull)
        return ctx_fail(ctx, MDET_ERR_INVALID, "too many contigs");
    // bins by label in ascending label order, members ascending (the
    // reference's std::map of vectors); dissolve those under min_cls_size
    std::vector<int64_t> glabel;
    std::vector<uint64_t> goff;
    std::vector<uint32_t> gmem;
    group_by_label(label, n, glabel, goff, gmem);
    std::vector<uint32_t> leftovers;
    for (uint64_t i = 0; i < n; ++i) out[i] = -1;
    for (uint64_t i = 0; i < n_small; ++i) small_out[i] = -1;
    uint64_t binned = 0, kept = 0;
    std::vector<int64_t> bin_label;
    std::vector<uint64_t> boff{0};
    std::vector<uint32_t> bmem;
    for (size_t g = 0; g < glabel.size(); ++g) {
        const uint32_t* m0 = gmem.data() + goff[g];
        const uint64_t cs = goff[g + 1] - goff[g];
        uint64_t sz = 0;
        for (uint64_t k = 0; k < cs; ++k) sz += sizes[m0[k]];
        if (sz < min_cls_size) {
            leftovers.insert(leftovers.end(), m0, m0 + cs);
            continue;
        }
        ++kept;
        binned += sz;
        for (uint64_t k = 0; k < cs; ++k) out[m0[k]] = glabel[g];
        if (cs >= kMinCS) {
            bin_label.push_back(glabel[g]);
            bmem.insert(bmem.end(), m0, m0 + cs);
            boff.push_back(bmem.size());
        }
    }
    const uint32_t nb = (uint32_t)bin_label.size();
    const uint64_t nl = leftovers.size();
    if (st) {
        st->n_bins = kept;
        st->n_bins_scored = nb;
        st->n_leftovers = nl;
        st->binned_bases = binned;
    }
    if (nl == 0 && n_small == 0) return MDET_OK;
    cudaStream_t s = ctx->stream;
    const uint64_t rows = n + n_small, ncand = nl + n_small;
    float* d_abd = (float*)ctx_scratch(ctx, "rc.abd", n * nabd * 4);
    float* d_sabd = (float*)ctx_scratch(ctx, "rc.sabd", std::max<uint64_t>(n_small, 1) * nabd * 4);
    double* d_d64 = (double*)ctx_scratch(ctx, "rc.d64", rows * nabd * 8);
    float* d_xf = (float*)ctx_scratch(ctx, "rc.xf", rows * nabd * 4);
    float* d_xw = (float*)ctx_scratch(ctx, "rc.xw", rows * nabd * 4);
    uint64_t* d_off = (uint64_t*)ctx_scratch(ctx, "rc.off", (nb + 1) * 8);
    uint32_t* d_mem = (uint32_t*)ctx_scratch(ctx, "rc.mem", std::max<size_t>(bmem.size(), 1) * 4);
    uint32_t* d_left = (uint32_t*)ctx_scratch(ctx, "rc.left", std::max<uint64_t>(nl, 1) * 4);
    double* d_bc = (double*)ctx_scratch(ctx, "rc.bcorr", std::max<uint32_t>(nb, 1) * 8);
    float* d_thr = (float*)ctx_scratch(ctx, "rc.thr", std::max<uint32_t>(nb, 1) * 4);
    uint32_t* d_qc = (uint32_t*)ctx_scratch(ctx, "rc.qc", std::max<uint64_t>(ncand, 1) * 4);
    uint32_t* d_qb = (uint32_t*)ctx_scratch(ctx, "rc.qb", std::max<uint64_t>(ncand, 1) * 4);
    unsigned long long* d_np = (unsigned long long*)ctx_scratch(ctx, "rc.npass", 8);
    if (!d_abd || !d_sabd || !d_d64 || !d_xf || !d_xw || !d_off || !d_mem || !d_left || !d_bc || !d_thr || !d_qc ||
        !d_qb || !d_np)
        return MDET_ERR_NOMEM;
    MDET_CUDA(ctx, cudaMemcpyAsync(d_abd, abd, n * nabd * 4, cudaMemcpyHostToDevice, s));
    if (n_small) MDET_CUDA(ctx, cudaMemcpyAsync(d_sabd, small_abd, n_small * nabd * 4, cudaMemcpyHostToDevice, s));
    MDET_CUDA(ctx, cudaMemcpyAsync(d_off, boff.data(), (nb + 1) * 8, cudaMemcpyHostToDevice, s));
    if (!bmem.empty()) MDET_CUDA(ctx, cudaMemcpyAsync(d_mem, bmem.data(), bmem.size() * 4, cudaMemcpyHostToDevice, s));
    if (nl) MDET_CUDA(ctx, cudaMemcpyAsync(d_left, leftovers.data(), nl * 4, cudaMemcpyHostToDevice, s));
    MDET_CUDA(ctx, cudaMemsetAsync(d_qc, 0, std::max<uint64_t>(ncand, 1) * 4, s));
    ctx_timer_begin(ctx, "k_rank_rows");
    k_rank_rows<<<(unsigned)((n + 127) / 128), 128, 0, s>>>(d_abd, n, nabd);
    MDET_LAUNCHED(ctx, "k_rank_rows");
    k_corr_rows<<<(unsigned)((n + 127) / 128), 128, 0, s>>>(d_abd, n, nabd, 0, d_d64, d_xf, d_xw);
    MDET_LAUNCHED(ctx, "k_corr_rows");
    if (n_small) {
        k_rank_rows<<<(unsigned)((n_small + 127) / 128), 128, 0, s>>>(d_sabd, n_small, nabd);
        MDET_LAUNCHED(ctx, "k_rank_rows");
        k_corr_rows<<<(unsigned)((n_small + 127) / 128), 128, 0, s>>>(d_sabd, n_small, nabd, n, d_d64, d_xf, d_xw);
        MDET_LAUNCHED(ctx, "k_corr_rows");
    }
    ctx_timer_end(ctx, "k_rank_rows");
    uint64_t npass = 0;
    if (nb) {
        double* d_est = (double*)ctx_scratch(ctx, "rc.est", nb * 8);
        double* d_est2 = (double*)ctx_scratch(ctx, "rc.est2", nb * 8);
        double* d_lo = (double*)ctx_scratch(ctx, "rc.lo", nb * 8);
        double* d_hi = (double*)ctx_scratch(ctx, "rc.hi", nb * 8);
        uint8_t* d_deg = (uint8_t*)ctx_scratch(ctx, "rc.deg", nb);
        uint8_t* d_tier = (uint8_t*)ctx_scratch(ctx, "rc.tier", nb);
        uint8_t* d_need = (uint8_t*)ctx_scratch(ctx, "rc.need", nb);
        uint32_t* d_bins = (uint32_t*)ctx_scratch(ctx, "rc.bins", nb * 4);
        uint64_t* d_toff = (uint64_t*)ctx_scratch(ctx, "rc.toff", (nb + 1) * 8);
        float* d_gf = (float*)ctx_scratch(ctx, "rc.gf", bmem.size() * nabd * 4);
        double* d_g64 = (double*)ctx_scratch(ctx, "rc.g64", bmem.size() * nabd * 8);
        if (!d_est || !d_est2 || !d_lo || !d_hi || !d_deg || !d_tier || !d_need || !d_bins || !d_toff || !d_gf ||
            !d_g64)
            return MDET_ERR_NOMEM;
        // MDET_RECRUIT_EPS_SCALE (>= 1) widens the estimates' intervals and
        // MDET_RECRUIT_TERM_CAP (terms) lowers the term buffer: the tests use
        // them to run the refining paths on small inputs
        double eps_scale = 1.0;
        if (const char* ev = getenv("MDET_RECRUIT_EPS_SCALE")) eps_scale = std::max(1.0, strtod(ev, nullptr));
        uint64_t tcap_max = kTermCap;
        if (const char* ev = getenv("MDET_RECRUIT_TERM_CAP"))
            if (const uint64_t v = strtoull(ev, nullptr, 10)) tcap_max = std::min<uint64_t>(v, kTermCap);
        std::vector<uint8_t> tier(nb, 0);
        uint64_t bins_exact = 0;
        // a list of bins to tier t: their FP64 terms, by runs of list
        // positions that fit the term buffer, added in a fixed tree (t = 1) or
        // in the reference's order (t = 2); a bin larger than the buffer goes
        // to its exact mean by a warp alone
        auto refine = [&](const std::vector<uint32_t>& bl, uint8_t t) -> int {
            if (bl.empty()) return MDET_OK;
            const uint32_t nbl = (uint32_t)bl.size();
            std::vector<uint64_t> toff(nbl + 1, 0);
            for (uint32_t p = 0; p < nbl; ++p) {
                const uint64_t cs = boff[bl[p] + 1] - boff[bl[p]];
                toff[p + 1] = toff[p] + cs * (cs - 1) / 2;
            }
            const uint64_t tcap = std::min<uint64_t>(toff[nbl], tcap_max);
            double* d_term = (double*)ctx_scratch(ctx, "rc.term", tcap * 8);
            if (!d_term) return MDET_ERR_NOMEM;
            MDET_CUDA(ctx, cudaMemcpyAsync(d_bins, bl.data(), nbl * 4, cudaMemcpyHostToDevice, s));
            MDET_CUDA(ctx, cudaMemcpyAsync(d_toff, toff.data(), (nbl + 1) * 8, cudaMemcpyHostToDevice, s));
            for (uint32_t p = 0; p < nbl;) {
                if (toff[p + 1] - toff[p] > tcap) {
                    k_bin_corr<<<1, 32, 0, s>>>(d_d64, nabd, d_off, d_mem, d_bins, p, p + 1, d_bc);
                    MDET_LAUNCHED(ctx, "k_bin_corr");
                    tier[bl[p]] = 2;
                    ++bins_exact;
                    ++p;
                    continue;
                }
                uint32_t e = p + 1;
                while (e < nbl && toff[e + 1] - toff[p] <= tcap) ++e;
                k_bin_terms<<<grid_for(ctx, toff[e] - toff[p], 256), 256, 0, s>>>(d_d64, nabd, d_off, d_mem, d_bins,
                                                                                d_toff, p, e, d_term);
                MDET_LAUNCHED(ctx, "k_bin_terms");
                if (t == 2) {
                    k_bin_sum<<<(e - p + 31) / 32, 32, 0, s>>>(d_term, d_off, d_bins, d_toff, p, e, d_bc);
                    MDET_LAUNCHED(ctx, "k_bin_sum");
                    bins_exact += e - p;
                } else {
                    k_bin_tree<<<std::min<uint32_t>(e - p, (uint32_t)ctx->num_sms * 8), 256, 0, s>>>(
                        d_term, d_off, d_bins, d_toff, p, e, d_est2);
                    MDET_LAUNCHED(ctx, "k_bin_tree");
                }
                for (uint32_t q = p; q < e; ++q) tier[bl[q]] = t;
                p = e;
            }
            // the term buffer and the list are reused by the next call
            MDET_CUDA(ctx, cudaStreamSynchronize(s));
            return MDET_OK;
        };
        const double delta = prefilter_delta(nabd);
        auto bounds = [&]() -> int {
            MDET_CUDA(ctx, cudaMemcpyAsync(d_tier, tier.data(), nb, cudaMemcpyHostToDevice, s));
            k_bin_bounds<<<(nb + 255) / 256, 256, 0, s>>>(d_est, d_est2, d_bc, d_tier, d_off, nb, nabd, delta,
                                                          eps_scale, d_lo, d_hi, d_thr);
            MDET_LAUNCHED(ctx, "k_bin_bounds");
            return MDET_OK;
        };
        // the bins' first estimates; exact means for bins the bound does not
        // cover
        ctx_timer_begin(ctx, "k_bin_corr");
        k_bin_gather<<<std::min<uint32_t>(nb, (uint32_t)ctx->num_sms * 8), 256, 0, s>>>(d_xf, d_d64, nabd, d_off,
                                                                                          d_mem, nb, d_gf, d_g64);
        MDET_LAUNCHED(ctx, "k_bin_gather");
        k_bin_mean32<<<std::min<uint32_t>(nb, (uint32_t)ctx->num_sms * 8), 256, 0, s>>>(d_xw, d_gf, nabd, d_off,
                                                                                          d_mem, nb, d_est, d_deg);
        MDET_LAUNCHED(ctx, "k_bin_mean32");
        std::vector<uint8_t> flag(nb);
        MDET_CUDA(ctx, cudaMemcpyAsync(flag.data(), d_deg, nb, cudaMemcpyDeviceToHost, s));
        MDET_CUDA(ctx, cudaStreamSynchronize(s));
        std::vector<uint32_t> bl;
        for (uint32_t b = 0; b < nb; ++b)
            if (flag[b]) bl.push_back(b);
        MDET_TRY(refine(bl, 2));
        MDET_TRY(bounds());
        ctx_timer_end(ctx, "k_bin_corr");
        // the prefilter: blocks of 256 contigs by chunks of bins, about two
        // waves of resident threads in all
        const uint64_t bx = (ncand + 255) / 256;
        const uint64_t want = (uint64_t)ctx->num_sms * 2048 * 2 / 256;
        const uint32_t chunks =
            (uint32_t)std::min<uint64_t>(std::min<uint64_t>(std::max<uint64_t>(want / bx, 1), nb), 65535);
        const uint32_t chunk = (nb + chunks - 1) / chunks;
        const dim3 grid((unsigned)bx, (nb + chunk - 1) / chunk);
        uint64_t cap = std::min<uint64_t>(ncand * nb, std::max<uint64_t>(ncand * 8, 1u << 22));
        ctx_timer_begin(ctx, "k_recruit_filter");
        for (int pass_no = 0; pass_no < 2; ++pass_no) {
            uint2* d_pass = (uint2*)ctx_scratch(ctx, "rc.pass", cap * 8);
            if (!d_pass) return MDET_ERR_NOMEM;
            MDET_CUDA(ctx, cudaMemsetAsync(d_np, 0, 8, s));
            const uint32_t m = nabd - 1;
            if (m <= 16)
                k_recruit_filter<16><<<grid, 256, 0, s>>>(d_xf, d_xw, nabd, d_left, nl, n, ncand, d_off, d_mem, nb,
                                                          chunk, d_thr, d_pass, cap, d_np);
            else if (m <= 32)
                k_recruit_filter<32><<<grid, 256, 0, s>>>(d_xf, d_xw, nabd, d_left, nl, n, ncand, d_off, d_mem, nb,
                                                          chunk, d_thr, d_pass, cap, d_np);
            else
                k_recruit_filter<0><<<grid, 256, 0, s>>>(d_xf, d_xw, nabd, d_left, nl, n, ncand, d_off, d_mem, nb,
                                                         chunk, d_thr, d_pass, cap, d_np);
            MDET_LAUNCHED(ctx, "k_recruit_filter");
            MDET_CUDA(ctx, cudaMemcpyAsync(&npass, d_np, 8, cudaMemcpyDeviceToHost, s));
            MDET_CUDA(ctx, cudaStreamSynchronize(s));
            if (npass <= cap) break;
            cap = npass;  // the list overflowed: once more with room for all of it
        }
        ctx_timer_end(ctx, "k_recruit_filter");
        if (npass > cap) return ctx_fail(ctx, MDET_ERR_INTERNAL, "prefilter list overflow");
        uint64_t undecided = 0;
        if (npass) {
            // the tests; those within eps of a bin's estimate again with the
            // bin's next estimate, and at last with its exact mean
            uint2* d_list[2] = {(uint2*)ctx_scratch(ctx, "rc.pass", cap * 8), nullptr};
            uint2* d_amb[2] = {(uint2*)ctx_scratch(ctx, "rc.amb", npass * 8),
                               (uint2*)ctx_scratch(ctx, "rc.amb2", npass * 8)};
            if (!d_list[0] || !d_amb[0] || !d_amb[1]) return MDET_ERR_NOMEM;
            const uint2* cur = d_list[0];
            uint64_t ncur = npass;
            ctx_timer_begin(ctx, "k_recruit");
            for (uint8_t round = 0; ncur; ++round) {
                uint2* next = d_amb[round & 1];
                MDET_CUDA(ctx, cudaMemsetAsync(d_np, 0, 8, s));
                MDET_CUDA(ctx, cudaMemsetAsync(d_need, 0, nb, s));
                k_recruit_exact<<<grid_for(ctx, ncur * 32, 256), 256, 0, s>>>(d_d64, d_g64, nabd, d_left, nl, n,
                                                                              d_off, d_lo, d_hi, cur, ncur, d_qc,
                                                                              d_qb, next, d_np, d_need);
                MDET_LAUNCHED(ctx, "k_recruit_exact");
                uint64_t namb = 0;
                MDET_CUDA(ctx, cudaMemcpyAsync(&namb, d_np, 8, cudaMemcpyDeviceToHost, s));
                MDET_CUDA(ctx, cudaStreamSynchronize(s));
                if (!namb) break;
                if (round == 2) return ctx_fail(ctx, MDET_ERR_INTERNAL, "recruit tests left undecided");
                if (round == 0) undecided = namb;
                MDET_CUDA(ctx, cudaMemcpyAsync(flag.data(), d_need, nb, cudaMemcpyDeviceToHost, s));
                MDET_CUDA(ctx, cudaStreamSynchronize(s));
                bl.clear();
                for (uint32_t b = 0; b < nb; ++b)
                    if (flag[b] && tier[b] < 2) bl.push_back(b);
                MDET_TRY(refine(bl, round == 0 ? 1 : 2));
                MDET_TRY(bounds());
                cur = next;
                ncur = namb;
            }
            ctx_timer_end(ctx, "k_recruit");
        }
        if (st) {
            st->pairs_tested = ncand * nb;
            st->pairs_exact = npass;
            st->pairs_undecided = undecided;
            st->bins_exact = bins_exact;
        }
    }
    std::vector<uint32_t> qc(ncand), qb(ncand);
    if (ncand) {
        MDET_CUDA(ctx, cudaMemcpyAsync(qc.data(), d_qc, ncand * 4, cudaMemcpyDeviceToHost, s));
        MDET_CUDA(ctx, cudaMemcpyAsync(qb.data(), d_qb, ncand * 4, cudaMemcpyDeviceToHost, s));
    }
    MDET_CUDA(ctx, cudaStreamSynchronize(s));
    // the gates: leftovers under 10 % of the binned bases, small contigs
    // under 15 % of small_total (0 rejects them, as the reference's
    // totalSize1 does outside verbose runs)
    unsigned long long added = 0, matched = 0;
    for (uint64_t l = 0; l < nl; ++l)
        if (qc[l] == 1) {
            added += sizes[leftovers[l]];
            ++matched;
        }
    const bool take_left = added > 0 && (double)added / binned < .10;
    if (take_left)
        for (uint64_t l = 0; l < nl; ++l)
            if (qc[l] == 1) out[leftovers[l]] = bin_label[qb[l]];
    if (st) {
        st->n_leftovers_matched = matched;
        st->leftover_bases = added;
        st->leftovers_accepted = take_left ? 1 : 0;
    }
    added = matched = 0;
    for (uint64_t k = 0; k < n_small; ++k)
        if (qc[nl + k] == 1) {
            added += small_sizes[k];
            ++matched;
        }
    const bool take_small = added > 0 && (double)added / small_total < .15;
    if (take_small)
        for (uint64_t k = 0; k < n_small; ++k)
            if (qc[nl + k] == 1) small_out[k] = bin_label[qb[nl + k]];
    if (st) {
        st->n_small_matched = matched;
        st->small_bases = added;
        st->small_accepted = take_small ? 1 : 0;
    }
    return MDET_OK;
}
