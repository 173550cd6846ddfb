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
// GB300 form: the grouping, dissolving and the two gates are O(n) host work;
// the ranks, the per-bin means (a warp per bin, its terms computed by the
// lanes and summed by one lane in the reference's order, so the double sum
// rounds exactly as the reference's) and the per-(contig, bin) tests (a
// thread per pair, sums in member order) run on the device.  The unit is
// compiled without FMA contraction, so every correlation and every sum is
// bit-identical to a host evaluation and the >= tests decide the same way.
#include <map>
#include <vector>

#include "common.cuh"

namespace {

constexpr uint32_t kMaxSamples = 256;  // depth columns a row may have
constexpr uint32_t kMinCS = 10;        // members a bin needs to recruit (the reference's minCS)

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

// cal_abd_corr: Pearson correlation of two depth rows with running means
// and co-moments, in the reference's operation order (no FMA contraction).
__device__ double corr_rows(const float* __restrict__ x, const float* __restrict__ y, uint32_t nabd) {
    double sxx = 0.0, syy = 0.0, sxy = 0.0, mx = 0.0, my = 0.0;
    for (uint32_t i = 0; i < nabd; ++i) {
        const double a = x[i], b = y[i];
        if (i == 0) {
            mx = a;
            my = b;
            continue;
        }
        const double ratio = i / (i + 1.0);
        const double dx = a - mx, dy = b - my;
        sxx += dx * dx * ratio;
        syy += dy * dy * ratio;
        sxy += dx * dy * ratio;
        mx += dx / (i + 1.0);
        my += dy / (i + 1.0);
    }
    return sxy / (sqrt(sxx) * sqrt(syy));
}

// Mean pairwise correlation of each scored bin (cls_corr): a warp per bin;
// for member i the lanes compute the terms (i, j) for 32 consecutive j and
// lane 0 adds them in order, so the sum runs (0,1), (0,2), ..., (1,2), ...
// exactly as the reference's double loop.
__global__ void k_bin_corr(const float* __restrict__ abd, uint32_t nabd, const uint64_t* __restrict__ off,
                           const uint32_t* __restrict__ mem, uint32_t nbins, double* __restrict__ out) {
    const uint32_t warps = (gridDim.x * blockDim.x) >> 5;
    const uint32_t lane = threadIdx.x & 31;
    for (uint32_t b = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; b < nbins; b += warps) {
        const uint64_t o = off[b], cs = off[b + 1] - off[b];
        double sum = 0.0;
        for (uint64_t i = 0; i < cs; ++i) {
            const float* xi = abd + (uint64_t)mem[o + i] * nabd;
            for (uint64_t j0 = i + 1; j0 < cs; j0 += 32) {
                const uint64_t j = j0 + lane;
                const double t = j < cs ? corr_rows(xi, abd + (uint64_t)mem[o + j] * nabd, nabd) : 0.0;
                const uint32_t cnt = (uint32_t)min((uint64_t)32, cs - j0);
                for (uint32_t q = 0; q < cnt; ++q) {
                    const double tq = __shfl_sync(0xffffffffu, t, q);
                    if (lane == 0) sum += tq;
                }
            }
        }
        if (lane == 0) out[b] = sum / (double)(cs * (cs - 1) / 2);
    }
}

// One thread per (candidate, scored bin): the reference's two-step test.
// Candidates [0, nl) are leftovers (rows of abd), [nl, nl + ns) small
// contigs (rows of sabd).  qcount counts the bins that accept a candidate,
// qbin holds one of them (meaningful when qcount == 1).
__global__ void k_recruit(const float* __restrict__ abd, const float* __restrict__ sabd, uint32_t nabd,
                          const uint32_t* __restrict__ left, uint64_t nl, uint64_t ns,
                          const uint64_t* __restrict__ off, const uint32_t* __restrict__ mem, uint32_t nbins,
                          const double* __restrict__ bcorr, uint32_t* __restrict__ qcount,
                          uint32_t* __restrict__ qbin) {
    const uint64_t total = (nl + ns) * (uint64_t)nbins;
    for (uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; t < total;
         t += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t cand = t / nbins;
        const uint32_t b = (uint32_t)(t % nbins);
        const float* y = cand < nl ? abd + (uint64_t)left[cand] * nabd : sabd + (cand - nl) * nabd;
        const uint64_t o = off[b], cs = off[b + 1] - off[b];
        const double th = bcorr[b];
        double c = 0.0;
        uint64_t i = 0;
        for (; i < kMinCS; ++i) c += corr_rows(abd + (uint64_t)mem[o + i] * nabd, y, nabd);
        if (c / kMinCS < th) continue;  // the reference's early stop on the first ten members
        for (; i < cs; ++i) c += corr_rows(abd + (uint64_t)mem[o + i] * nabd, y, nabd);
        c /= cs;
        if (c >= th) {
            atomicAdd(&qcount[cand], 1u);
            qbin[cand] = b;
        }
    }
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
    if (n >= 0xFFFFFFFFull || n_small >= 0xFFFFFFFFull) return ctx_fail(ctx, MDET_ERR_INVALID, "too many contigs");
    // bins by label, members ascending; dissolve those under min_cls_size
    std::map<int64_t, std::vector<uint32_t>> cls;
    for (uint64_t i = 0; i < n; ++i) cls[label[i]].push_back((uint32_t)i);
    std::vector<uint32_t> leftovers;
    for (auto it = cls.begin(); it != cls.end();) {
        uint64_t s = 0;
        for (uint32_t m : it->second) s += sizes[m];
        if (s < min_cls_size) {
            leftovers.insert(leftovers.end(), it->second.begin(), it->second.end());
            it = cls.erase(it);
        } else {
            ++it;
        }
    }
    for (uint64_t i = 0; i < n; ++i) out[i] = -1;
    for (uint64_t i = 0; i < n_small; ++i) small_out[i] = -1;
    uint64_t binned = 0;
    std::vector<int64_t> bin_label;
    std::vector<uint64_t> boff{0};
    std::vector<uint32_t> bmem;
    for (auto& kv : cls) {
        for (uint32_t m : kv.second) {
            out[m] = kv.first;
            binned += sizes[m];
        }
        if (kv.second.size() >= kMinCS) {
            bin_label.push_back(kv.first);
            bmem.insert(bmem.end(), kv.second.begin(), kv.second.end());
            boff.push_back(bmem.size());
        }
    }
    const uint32_t nb = (uint32_t)bin_label.size();
    const uint64_t nl = leftovers.size();
    if (st) {
        st->n_bins = cls.size();
        st->n_bins_scored = nb;
        st->n_leftovers = nl;
        st->binned_bases = binned;
    }
    if (nl == 0 && n_small == 0) return MDET_OK;
    cudaStream_t s = ctx->stream;
    float* d_abd = (float*)ctx_scratch(ctx, "rc.abd", n * nabd * 4);
    float* d_sabd = (float*)ctx_scratch(ctx, "rc.sabd", std::max<uint64_t>(n_small, 1) * nabd * 4);
    uint64_t* d_off = (uint64_t*)ctx_scratch(ctx, "rc.off", (nb + 1) * 8);
    uint32_t* d_mem = (uint32_t*)ctx_scratch(ctx, "rc.mem", std::max<size_t>(bmem.size(), 1) * 4);
    uint32_t* d_left = (uint32_t*)ctx_scratch(ctx, "rc.left", std::max<uint64_t>(nl, 1) * 4);
    double* d_bc = (double*)ctx_scratch(ctx, "rc.bcorr", std::max<uint32_t>(nb, 1) * 8);
    uint32_t* d_qc = (uint32_t*)ctx_scratch(ctx, "rc.qc", std::max<uint64_t>(nl + n_small, 1) * 4);
    uint32_t* d_qb = (uint32_t*)ctx_scratch(ctx, "rc.qb", std::max<uint64_t>(nl + n_small, 1) * 4);
    if (!d_abd || !d_sabd || !d_off || !d_mem || !d_left || !d_bc || !d_qc || !d_qb) return MDET_ERR_NOMEM;
    MDET_CUDA(ctx, cudaMemcpyAsync(d_abd, abd, n * nabd * 4, cudaMemcpyHostToDevice, s));
    if (n_small) MDET_CUDA(ctx, cudaMemcpyAsync(d_sabd, small_abd, n_small * nabd * 4, cudaMemcpyHostToDevice, s));
    MDET_CUDA(ctx, cudaMemcpyAsync(d_off, boff.data(), (nb + 1) * 8, cudaMemcpyHostToDevice, s));
    if (!bmem.empty()) MDET_CUDA(ctx, cudaMemcpyAsync(d_mem, bmem.data(), bmem.size() * 4, cudaMemcpyHostToDevice, s));
    if (nl) MDET_CUDA(ctx, cudaMemcpyAsync(d_left, leftovers.data(), nl * 4, cudaMemcpyHostToDevice, s));
    MDET_CUDA(ctx, cudaMemsetAsync(d_qc, 0, std::max<uint64_t>(nl + n_small, 1) * 4, s));
    ctx_timer_begin(ctx, "k_rank_rows");
    k_rank_rows<<<(unsigned)((n + 127) / 128), 128, 0, s>>>(d_abd, n, nabd);
    MDET_LAUNCHED(ctx, "k_rank_rows");
    if (n_small) {
        k_rank_rows<<<(unsigned)((n_small + 127) / 128), 128, 0, s>>>(d_sabd, n_small, nabd);
        MDET_LAUNCHED(ctx, "k_rank_rows");
    }
    ctx_timer_end(ctx, "k_rank_rows");
    if (nb) {
        ctx_timer_begin(ctx, "k_bin_corr");
        k_bin_corr<<<grid_for(ctx, (uint64_t)nb * 32, 128), 128, 0, s>>>(d_abd, nabd, d_off, d_mem, nb, d_bc);
        ctx_timer_end(ctx, "k_bin_corr");
        MDET_LAUNCHED(ctx, "k_bin_corr");
        ctx_timer_begin(ctx, "k_recruit");
        k_recruit<<<grid_for(ctx, (nl + n_small) * (uint64_t)nb, 256), 256, 0, s>>>(
            d_abd, d_sabd, nabd, d_left, nl, n_small, d_off, d_mem, nb, d_bc, d_qc, d_qb);
        ctx_timer_end(ctx, "k_recruit");
        MDET_LAUNCHED(ctx, "k_recruit");
    }
    std::vector<uint32_t> qc(nl + n_small), qb(nl + n_small);
    if (nl + n_small) {
        MDET_CUDA(ctx, cudaMemcpyAsync(qc.data(), d_qc, (nl + n_small) * 4, cudaMemcpyDeviceToHost, s));
        MDET_CUDA(ctx, cudaMemcpyAsync(qb.data(), d_qb, (nl + n_small) * 4, cudaMemcpyDeviceToHost, s));
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
