// labelprop.cu -- binning by label propagation over the scored edge graph:
// the traversal of main (cuda/Cuda2.cu:1980-2061) and label_propagation
// (cuda/Cuda2.cu:569-656), on the device.
//
// The traversal takes the edges in decreasing score.  An edge whose two
// contigs are in different bins connects them (first-seen order) and, above
// min_s, joins the traversal graph; the first such edge at or below min_s
// ends the traversal.  Propagation runs when the connected share of the
// contigs reaches max_p/10 * (1..10), and at the last edge.  Between two
// runs the bins do not change, so each stretch of edges up to the next run
// is one data-parallel step: the differing-bin test, the early stop, the
// first appearance of each contig (an atomic minimum of the edge position)
// and the run position follow from one pass and a sort.
//
// Label propagation is Gauss-Seidel: each contig, in first-seen order, takes
// the neighbour label with the largest Fisher-combined chi-squared CDF,
// reading the labels its predecessors in that order have just written.
// Contigs that share no edge do not read each other, so the sweep runs level
// by level over the order's dependency graph (level = 1 + the deepest level
// among the contig's neighbours earlier in the order, found by Kahn peeling):
// one block per contig of a level, the levels in turn -- the same result as
// the sequential sweep.  A block sorts its contig's (neighbour label, edge
// position) keys (bitonic sort in shared memory, or in a global slice for
// contigs with more than 2,048 edges), folds each label's log(1 - score) in
// edge order (the reference's summation order), evaluates the CDF
// (lp_math.h, bit-identical to the host checker) and breaks exact ties by the
// reference map's iteration order (lp_umap.h); contigs with at most 32 edges
// take a warp each, the keys sorted across its lanes.  A contig none of whose
// neighbours changed label since its last evaluation is skipped: the same
// label would win and its update would change nothing -- across runs too:
// a run's first sweep evaluates the contigs with new edges, those frozen in
// the previous run, and those whose neighbours changed since.  The visited (contig, label)
// pairs of a call live in an open-addressing table; a call that overfills it
// is re-run from its starting labels with a larger table.
#include <cub/cub.cuh>
#include <thrust/iterator/counting_iterator.h>

#include <algorithm>
#include <climits>
#include <cmath>
#include <vector>

#include "common.cuh"
#include "lp_math.h"
#include "lp_umap.h"

int check_flag(mdet_ctx* ctx);

namespace {

constexpr uint32_t kSmallCap = 2048;  // incident edges a block sorts in shared memory
constexpr uint32_t kWarpCap = 32;     // incident edges a warp sorts in registers
constexpr int kThreads = 256;
constexpr uint32_t kProbeLimit = 1u << 16;

// flags
constexpr unsigned long long kErrTable = 1;     // visited table too full
constexpr unsigned long long kErrSlots = 2;     // global sort slice missing
constexpr unsigned long long kErrScore = 4;     // a score outside [0, 1]

__host__ __device__ inline uint32_t pow2_at_least(uint32_t d) {
    uint32_t n = 2;
    while (n < d) n <<= 1;
    return n;
}

// bytes of one contig's work area for a sort of n keys (n a power of two)
__host__ __device__ inline size_t ws_bytes(uint32_t n) {
    return (size_t)n * (8 + 8 + 8 + 4 + 4 + 4) + (size_t)lpu::buckets_for(n) * 4;
}

__device__ __forceinline__ uint64_t mix64(uint64_t z) {
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

struct LpArgs {
    const uint32_t* inc_off;  // [n + 1]
    const uint32_t* oth;      // per incidence (a contig's traversal edges, increasing): the other contig
    const double* ilw;        // per incidence: the edge's log(1 - score)
    uint32_t* mem;
    uint8_t* stuck;
    uint8_t* dirty;           // a neighbour's label changed since the contig was last evaluated
    unsigned long long* vt;   // visited (contig, label) table, 0 = empty
    unsigned long long vt_mask;
    const lpf::F2* logfact;
    const lpf::F2* recip;     // 1/j for j < nrecip (the CDF's series steps)
    uint32_t nrecip;
    unsigned long long* counters;  // [0] moved, [1] table entries, [2] error flags, [3] tied picks
    unsigned char* big_ws;
    size_t big_stride;
    uint32_t big_slots;
    const uint32_t* slot_of;
};

// true when (v, lab) was not in the table
__device__ bool visit(const LpArgs& P, uint32_t v, uint32_t lab) {
    const unsigned long long key = (((unsigned long long)v << 32) | lab) + 1ull;
    unsigned long long h = mix64(key) & P.vt_mask;
    for (uint32_t it = 0; it < kProbeLimit; ++it) {
        const unsigned long long old = atomicCAS(P.vt + h, 0ull, key);
        if (old == 0ull) {
            const unsigned long long cnt = atomicAdd(P.counters + 1, 1ull) + 1;
            if (cnt * 4 > (P.vt_mask + 1) * 3) atomicOr(P.counters + 2, kErrTable);
            return true;
        }
        if (old == key) return false;
        h = (h + 1) & P.vt_mask;
    }
    atomicOr(P.counters + 2, kErrTable);
    return false;
}

// One sweep step for the contigs of one level: block per contig.
__global__ void __launch_bounds__(kThreads) k_lp_level(LpArgs P, const uint32_t* __restrict__ nodes) {
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ double red_v[kThreads / 32];
    __shared__ uint32_t red_c[kThreads / 32];
    __shared__ double s_vmax;
    __shared__ uint32_t s_ties, s_best, s_changed;
    const uint32_t v = nodes[blockIdx.x];
    const uint32_t s = P.inc_off[v];
    const uint32_t d = P.inc_off[v + 1] - s;
    // no neighbour changed since the last evaluation: the same label wins
    // and the update is a no-op
    if (d == 0 || !P.dirty[v]) return;
    const uint32_t N = pow2_at_least(d);
    unsigned char* base = smem;
    if (N > kSmallCap) {
        const uint32_t slot = P.slot_of[v];
        if (slot >= P.big_slots) {
            if (threadIdx.x == 0) atomicOr(P.counters + 2, kErrSlots);
            return;
        }
        base = P.big_ws + (size_t)slot * P.big_stride;
    }
    unsigned long long* sk = reinterpret_cast<unsigned long long*>(base);
    double* w = reinterpret_cast<double*>(base + (size_t)N * 8);
    double* val = reinterpret_cast<double*>(base + (size_t)N * 16);
    int32_t* fidx = reinterpret_cast<int32_t*>(base + (size_t)N * 24);
    uint32_t* ins = reinterpret_cast<uint32_t*>(base + (size_t)N * 28);
    int32_t* nxt = reinterpret_cast<int32_t*>(base + (size_t)N * 32);
    int32_t* bb = reinterpret_cast<int32_t*>(base + (size_t)N * 36);
    const uint32_t t = threadIdx.x;

    // (neighbour label, edge position) keys and the edges' log(1 - score)
    for (uint32_t j = t; j < N; j += kThreads) {
        if (j < d) {
            const uint32_t o = P.oth[s + j];
            sk[j] = ((unsigned long long)P.mem[o] << 32) | j;
            w[j] = P.ilw[s + j];
        } else {
            sk[j] = ~0ull;
        }
        fidx[j] = -1;
    }
    __syncthreads();
    // bitonic sort, ascending
    for (uint32_t k = 2; k <= N; k <<= 1) {
        for (uint32_t jj = k >> 1; jj > 0; jj >>= 1) {
            for (uint32_t i = t; i < N; i += kThreads) {
                const uint32_t l = i ^ jj;
                if (l > i) {
                    const unsigned long long a = sk[i], b = sk[l];
                    const bool up = (i & k) == 0;
                    if ((a > b) == up) {
                        sk[i] = b;
                        sk[l] = a;
                    }
                }
            }
            __syncthreads();
        }
    }
    // each label's run: the Fisher-combined CDF of its edges, folded in edge
    // order (positions are sorted within a label)
    double vmax = -1.0;
    for (uint32_t p = t; p < d; p += kThreads) {
        const uint32_t lab = (uint32_t)(sk[p] >> 32);
        double vp = -1.0;
        if (p == 0 || (uint32_t)(sk[p - 1] >> 32) != lab) {
            double sum = 0.0;
            uint32_t q = p;
            do {
                sum = sum + w[(uint32_t)sk[q]];
                ++q;
            } while (q < d && (uint32_t)(sk[q] >> 32) == lab);
            vp = lpf::chi2_cdf(2.0 * (double)(q - p), -2.0 * sum, P.logfact, P.recip, P.nrecip);
            fidx[(uint32_t)sk[p]] = (int32_t)p;
        }
        val[p] = vp;
        vmax = fmax(vmax, vp);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) vmax = fmax(vmax, __shfl_xor_sync(0xffffffffu, vmax, o));
    if ((t & 31) == 0) red_v[t >> 5] = vmax;
    __syncthreads();
    if (t == 0) {
        double m = red_v[0];
        for (int i = 1; i < kThreads / 32; ++i) m = fmax(m, red_v[i]);
        s_vmax = m;
    }
    __syncthreads();
    const double top = s_vmax;
    uint32_t ties = 0;
    for (uint32_t p = t; p < d; p += kThreads) ties += val[p] == top;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) ties += __shfl_xor_sync(0xffffffffu, ties, o);
    if ((t & 31) == 0) red_c[t >> 5] = ties;
    __syncthreads();
    if (t == 0) {
        uint32_t nt = 0;
        for (int i = 0; i < kThreads / 32; ++i) nt += red_c[i];
        s_ties = nt;
    }
    __syncthreads();
    if (s_ties == 1) {
        for (uint32_t p = t; p < d; p += kThreads)
            if (val[p] == top) s_best = (uint32_t)(sk[p] >> 32);
    }
    __syncthreads();
    if (t == 0) {
        P.dirty[v] = 0;
        if (s_ties > 1) {
            atomicAdd(P.counters + 3, 1ull);
        // the first tied label in the map's iteration order: labels in
        // first-seen order (edge position of their first edge), then the map
        uint32_t K = 0;
        for (uint32_t j = 0; j < d; ++j) {
            const int32_t p = fidx[j];
            if (p >= 0) {
                fidx[K] = p;  // K <= j: fidx[j] is read before any later write reaches it
                ins[K] = (uint32_t)(sk[p] >> 32);
                ++K;
            }
        }
        int32_t q = lpu::order(ins, K, nxt, bb);
        while (q >= 0 && val[fidx[q]] != top) q = nxt[q];
        s_best = ins[q >= 0 ? q : 0];
        }
        const uint32_t b = s_best;
        s_changed = 0;
        if (P.mem[v] != b && !P.stuck[v]) {
            P.mem[v] = b;
            s_changed = 1;
            if (visit(P, v, b))
                atomicAdd(P.counters, 1ull);
            else
                P.stuck[v] = 1;
        }
    }
    __syncthreads();
    if (s_changed)
        for (uint32_t j = t; j < d; j += kThreads) {
            P.dirty[P.oth[s + j]] = 1;
        }
}

// The same step for contigs with at most 32 edges: a warp per contig, the
// keys sorted in registers (bitonic over lanes), a lane per edge.
constexpr int kWarpsPerBlock = kThreads / 32;
struct WarpWs {
    unsigned long long sk[32];
    double w[32];
    double val[32];
    int32_t fidx[32];
    uint32_t ins[32];
    int32_t nxt[32];
    int32_t bb[64];  // lpu::buckets_for(32) = 59
};

__global__ void __launch_bounds__(kThreads) k_lp_level_warp(LpArgs P, const uint32_t* __restrict__ nodes,
                                                            uint32_t count) {
    __shared__ WarpWs ws_all[kWarpsPerBlock];
    const uint32_t wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t idx = blockIdx.x * kWarpsPerBlock + wid;
    if (idx >= count) return;
    WarpWs& W = ws_all[wid];
    const uint32_t v = nodes[idx];
    const uint32_t s = P.inc_off[v];
    const uint32_t d = P.inc_off[v + 1] - s;
    if (d == 0 || !P.dirty[v]) return;  // as in the block form
    unsigned long long key = ~0ull;
    uint32_t o = 0;
    if (lane < d) {
        o = P.oth[s + lane];
        key = ((unsigned long long)P.mem[o] << 32) | lane;
        W.w[lane] = P.ilw[s + lane];
    }
    W.fidx[lane] = -1;
    // bitonic sort over the lanes, ascending
#pragma unroll
    for (uint32_t k = 2; k <= 32; k <<= 1) {
#pragma unroll
        for (uint32_t j = k >> 1; j > 0; j >>= 1) {
            const unsigned long long o = __shfl_xor_sync(0xffffffffu, key, j);
            const bool lower = (lane & j) == 0, up = (lane & k) == 0;
            key = (lower == up) ? (o < key ? o : key) : (o > key ? o : key);
        }
    }
    W.sk[lane] = key;
    __syncwarp();
    const uint32_t lab = (uint32_t)(key >> 32);
    const uint32_t prev = __shfl_up_sync(0xffffffffu, lab, 1);
    double val = -1.0;
    if (lane < d && (lane == 0 || prev != lab)) {
        double sum = 0.0;
        uint32_t q = lane;
        do {
            sum = sum + W.w[(uint32_t)W.sk[q]];
            ++q;
        } while (q < d && (uint32_t)(W.sk[q] >> 32) == lab);
        val = lpf::chi2_cdf(2.0 * (double)(q - lane), -2.0 * sum, P.logfact, P.recip, P.nrecip);
        W.fidx[(uint32_t)key] = (int32_t)lane;
    }
    W.val[lane] = val;
    double top = val;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) top = fmax(top, __shfl_xor_sync(0xffffffffu, top, o));
    const unsigned tied = __ballot_sync(0xffffffffu, lane < d && val == top);
    __syncwarp();
    uint32_t best = __shfl_sync(0xffffffffu, lab, __ffs(tied) - 1);
    uint32_t changed = 0;
    if (lane == 0) {
        P.dirty[v] = 0;
        if (__popc(tied) > 1) {
            atomicAdd(P.counters + 3, 1ull);
            uint32_t K = 0;
            for (uint32_t j = 0; j < d; ++j) {
                const int32_t p = W.fidx[j];
                if (p >= 0) {
                    W.fidx[K] = p;  // K <= j: fidx[j] is read before any later write reaches it
                    W.ins[K] = (uint32_t)(W.sk[p] >> 32);
                    ++K;
                }
            }
            int32_t q = lpu::order(W.ins, K, W.nxt, W.bb);
            while (q >= 0 && W.val[W.fidx[q]] != top) q = W.nxt[q];
            best = W.ins[q >= 0 ? q : 0];
        }
        if (P.mem[v] != best && !P.stuck[v]) {
            P.mem[v] = best;
            changed = 1;
            if (visit(P, v, best))
                atomicAdd(P.counters, 1ull);
            else
                P.stuck[v] = 1;
        }
    }
    if (__shfl_sync(0xffffffffu, changed, 0) && lane < d) P.dirty[o] = 1;
}

// ---- dependency levels of the order --------------------------------------

__global__ void k_lp_pos(const uint32_t* __restrict__ order, uint32_t norder, uint32_t* __restrict__ pos_of) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < norder) pos_of[order[i]] = i;
}

// a level's contigs: those with at most kWarpCap edges (a warp each) and the
// others (a block each; maxdeg and the global slices are theirs); off and
// soff: where the level starts in the block and warp lists
struct LevelInfo {
    unsigned int count, maxdeg, nbig, nsmall, maxall, off, soff, pad;
};

__device__ __forceinline__ void lp_enqueue(uint32_t w, uint32_t deg, uint32_t* next, uint32_t* next_small,
                                           LevelInfo* info, uint32_t* slot_of) {
    atomicMax(&info->maxall, deg);
    if (deg <= kWarpCap) {
        next_small[atomicAdd(&info->nsmall, 1u)] = w;
        return;
    }
    next[atomicAdd(&info->count, 1u)] = w;
    atomicMax(&info->maxdeg, deg);
    if (pow2_at_least(deg) > kSmallCap) slot_of[w] = atomicAdd(&info->nbig, 1u);
}

// earlier neighbours of each contig of the order (warp per contig); those
// with none form level 0
__global__ void __launch_bounds__(256) k_lp_pred(const uint32_t* __restrict__ order, uint32_t norder,
                                                 const uint32_t* __restrict__ pos_of,
                                                 const uint32_t* __restrict__ inc_off,
                                                 const uint32_t* __restrict__ oth, uint32_t* __restrict__ pred,
                                                 uint32_t* __restrict__ level0, uint32_t* __restrict__ level0_small,
                                                 LevelInfo* info, uint32_t* __restrict__ slot_of) {
    const uint32_t wid = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (wid >= norder) return;
    const uint32_t u = order[wid], pu = wid;
    const uint32_t s = inc_off[u], d = inc_off[u + 1] - s;
    uint32_t c = 0;
    for (uint32_t j = lane; j < d; j += 32) c += pos_of[oth[s + j]] < pu;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
    if (lane == 0) {
        pred[u] = c;
        if (c == 0) lp_enqueue(u, d, level0, level0_small, info, slot_of);
    }
}

// One Kahn step for level L (its size and place read from info[L], so steps
// can be queued without the host): contigs whose last earlier neighbour is
// in this level join level L + 1.  A warp per contig, grid-stride.
__global__ void __launch_bounds__(256) k_lp_kahn(uint32_t L, const uint32_t* __restrict__ pos_of,
                                                 const uint32_t* __restrict__ inc_off,
                                                 const uint32_t* __restrict__ oth, uint32_t* __restrict__ pred,
                                                 uint32_t* __restrict__ lvl, uint32_t* __restrict__ lvls,
                                                 LevelInfo* info, uint32_t* __restrict__ slot_of) {
    const LevelInfo cur = info[L];
    const uint32_t total = cur.count + cur.nsmall;
    const uint32_t noff = cur.off + cur.count, nsoff = cur.soff + cur.nsmall;
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        info[L + 1].off = noff;
        info[L + 1].soff = nsoff;
    }
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t nw = gridDim.x * (blockDim.x >> 5);
    for (uint32_t wid = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; wid < total; wid += nw) {
        const uint32_t u = wid < cur.count ? lvl[cur.off + wid] : lvls[cur.soff + wid - cur.count];
        const uint32_t pu = pos_of[u];
        const uint32_t s = inc_off[u], d = inc_off[u + 1] - s;
        for (uint32_t j = lane; j < d; j += 32) {
            const uint32_t o = oth[s + j];
            if (pos_of[o] > pu && atomicSub(pred + o, 1u) == 1u)
                lp_enqueue(o, inc_off[o + 1] - inc_off[o], lvl + noff, lvls + nsoff, info + L + 1, slot_of);
        }
    }
}

// ---- the traversal ----------------------------------------------------------

__global__ void k_lp_gather(const uint64_t* __restrict__ from, const uint64_t* __restrict__ to,
                            const double* __restrict__ sscr, const uint32_t* __restrict__ ord, uint64_t ne, uint64_t n,
                            uint32_t* __restrict__ sa, uint32_t* __restrict__ sb, double* __restrict__ ss,
                            unsigned long long* __restrict__ flags) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < ne; i += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t e = ord[i];
        const double s = sscr[e];
        const uint64_t a = to[e], b = from[e];
        if (!(s >= 0.0 && s <= 1.0) || a >= n || b >= n) atomicOr(flags, kErrScore);
        sa[i] = (uint32_t)min(a, n - 1);
        sb[i] = (uint32_t)min(b, n - 1);
        ss[i] = s;
    }
}

__device__ __forceinline__ unsigned long long block_min(unsigned long long v, unsigned long long* red) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long u = __shfl_xor_sync(0xffffffffu, v, o);
        v = u < v ? u : v;
    }
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x == 0)
        for (unsigned w = 1; w < blockDim.x / 32; ++w) v = red[w] < v ? red[w] : v;
    return v;  // valid in thread 0
}

// over [p0, p1): the first differing-bin edge at or below min_s (the early
// stop, out[0]) and the first one above it (out[1]); one atomic per block
__global__ void __launch_bounds__(256) k_lp_seg(const uint32_t* __restrict__ sa, const uint32_t* __restrict__ sb,
                                                const double* __restrict__ ss, uint64_t p0, uint64_t p1,
                                                const uint32_t* __restrict__ mem, double min_s,
                                                unsigned long long* __restrict__ out) {
    __shared__ unsigned long long red[8];
    unsigned long long lo = ~0ull, hi = ~0ull;
    for (uint64_t i = p0 + blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < p1;
         i += (uint64_t)gridDim.x * blockDim.x) {
        if (mem[sa[i]] == mem[sb[i]]) continue;
        if (ss[i] > min_s) {
            if (hi == ~0ull) hi = i;
        } else if (lo == ~0ull) {
            lo = i;
        }
    }
    lo = block_min(lo, red);
    if (threadIdx.x == 0 && lo != ~0ull) atomicMin(out, lo);
    __syncthreads();
    hi = block_min(hi, red);
    if (threadIdx.x == 0 && hi != ~0ull) atomicMin(out + 1, hi);
}

// first appearance (2 * position, + 1 for the second contig) of the contigs
// not yet connected, over the differing-bin edges of [p0, p1)
__global__ void k_lp_first(const uint32_t* __restrict__ sa, const uint32_t* __restrict__ sb, uint64_t p0,
                           uint64_t p1, const uint32_t* __restrict__ mem, const uint8_t* __restrict__ seen,
                           unsigned long long* __restrict__ first) {
    for (uint64_t i = p0 + blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < p1;
         i += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t a = sa[i], b = sb[i];
        if (mem[a] == mem[b]) continue;
        if (!seen[a]) atomicMin(first + a, 2ull * i);
        if (!seen[b]) atomicMin(first + b, 2ull * i + 1);
    }
}

// slot 2k (+1) of [p0, p1) is set when the edge at p0 + k is where its first
// (second) contig is seen first: the first-seen order of the new contigs is
// the order of the set slots
__global__ void k_lp_slots(const uint32_t* __restrict__ sa, const uint32_t* __restrict__ sb, uint64_t p0,
                           uint64_t cnt, const uint32_t* __restrict__ mem, const uint8_t* __restrict__ seen,
                           const unsigned long long* __restrict__ first, uint8_t* __restrict__ slot) {
    const uint64_t k = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (k >= cnt) return;
    const uint64_t i = p0 + k;
    const uint32_t a = sa[i], b = sb[i];
    const bool d = mem[a] != mem[b];
    slot[2 * k] = d && !seen[a] && first[a] == 2ull * i;
    slot[2 * k + 1] = d && !seen[b] && first[b] == 2ull * i + 1;
}

// the contigs of the selected slots, appended to the order and marked
__global__ void k_lp_take(const uint32_t* __restrict__ sel, uint64_t k, uint64_t p0, const uint32_t* __restrict__ sa,
                          const uint32_t* __restrict__ sb, uint32_t* __restrict__ order, uint8_t* __restrict__ seen) {
    const uint64_t j = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (j >= k) return;
    const uint32_t sl = sel[j];
    const uint64_t i = p0 + (sl >> 1);
    const uint32_t v = (sl & 1) ? sb[i] : sa[i];
    order[j] = v;
    seen[v] = 1;
}

__global__ void k_lp_iota(uint32_t* __restrict__ v, uint64_t n) {
    const uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (i < n) v[i] = (uint32_t)i;
}

// the edges of [pos, end] that join the traversal graph, appended in order
__global__ void k_lp_edge_flags(const uint32_t* __restrict__ sa, const uint32_t* __restrict__ sb,
                                const double* __restrict__ ss, uint64_t pos, uint64_t cnt,
                                const uint32_t* __restrict__ mem, double min_s, uint8_t* __restrict__ flag) {
    const uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (i >= cnt) return;
    const uint64_t p = pos + i;
    flag[i] = mem[sa[p]] != mem[sb[p]] && ss[p] > min_s;
}

__global__ void k_lp_append(const uint32_t* __restrict__ sel, uint64_t k, uint64_t pos,
                            const uint32_t* __restrict__ sa, const uint32_t* __restrict__ sb,
                            const double* __restrict__ ss, uint32_t* __restrict__ ea, uint32_t* __restrict__ eb,
                            double* __restrict__ lw) {
    const uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (i >= k) return;
    const uint64_t p = pos + sel[i];
    ea[i] = sa[p];
    eb[i] = sb[p];
    lw[i] = lpm::log(1. - ss[p]);
}

// incidence entries: (contig, edge) for both ends, edges in order
__global__ void k_lp_inc_keys(const uint32_t* __restrict__ ea, const uint32_t* __restrict__ eb, uint64_t m,
                              uint32_t* __restrict__ key, uint32_t* __restrict__ val,
                              unsigned int* __restrict__ deg) {
    const uint64_t e = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (e >= m) return;
    key[2 * e] = ea[e];
    val[2 * e] = (uint32_t)e;
    key[2 * e + 1] = eb[e];
    val[2 * e + 1] = (uint32_t)e;
    atomicAdd(deg + ea[e], 1u);
    atomicAdd(deg + eb[e], 1u);
}

// per incidence (sorted by contig, then edge): the other contig and the
// edge's log(1 - score), so that the sweeps read them in order
__global__ void k_lp_inc_fill(const uint32_t* __restrict__ inc, const uint32_t* __restrict__ node, uint64_t cnt,
                              const uint32_t* __restrict__ ea, const uint32_t* __restrict__ eb,
                              const double* __restrict__ lw, uint32_t* __restrict__ oth, double* __restrict__ ilw) {
    const uint64_t j = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (j >= cnt) return;
    const uint32_t e = inc[j], v = node[j];
    oth[j] = ea[e] == v ? eb[e] : ea[e];
    ilw[j] = lw[e];
}

__global__ void k_lp_logfact(lpf::F2* out, uint32_t count) { lpf::log_factorials(out, count); }

__global__ void k_lp_recip(lpf::F2* out, uint32_t count) {
    const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;  // lpf::reciprocals, one entry per thread
    if (j < count) out[j] = j ? lpf::from_double(1.0 / (double)j) : lpf::make(0.0f, 0.0f);
}

// before a run: contigs with an edge added since the last run, and contigs
// frozen in the last run (free again now), are evaluated in its first sweep;
// the others keep their flag
__global__ void k_lp_dirty_edges(const uint32_t* __restrict__ ea, const uint32_t* __restrict__ eb, uint64_t m0,
                                 uint64_t m1, uint8_t* __restrict__ dirty) {
    const uint64_t e = m0 + blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (e >= m1) return;
    dirty[ea[e]] = 1;
    dirty[eb[e]] = 1;
}

__global__ void k_lp_dirty_stuck(const uint8_t* __restrict__ stuck, uint64_t n, uint8_t* __restrict__ dirty) {
    const uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (i < n && stuck[i]) dirty[i] = 1;
}

__global__ void k_lp_count_stuck(const uint8_t* __restrict__ stuck, uint64_t n, unsigned long long* __restrict__ out) {
    unsigned long long c = 0;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
        c += stuck[i];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
    if ((threadIdx.x & 31) == 0 && c) atomicAdd(out, c);
}

__global__ void k_lp_widen(const uint32_t* __restrict__ mem, uint64_t n, uint64_t* __restrict__ out) {
    const uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (i < n) out[i] = mem[i];
}

inline unsigned grid_for(uint64_t n, unsigned b = 256) { return (unsigned)std::max<uint64_t>(1, (n + b - 1) / b); }

struct LpState {
    uint64_t n = 0, ne = 0;
    uint32_t *sa = nullptr, *sb = nullptr, *mem = nullptr, *mem0 = nullptr, *order = nullptr;
    double* ss = nullptr;
    uint8_t *seen = nullptr, *stuck = nullptr, *dirty = nullptr, *dirty0 = nullptr, *eflag = nullptr;
    unsigned long long *first = nullptr, *cnt = nullptr;
    uint32_t *ea = nullptr, *eb = nullptr;
    double* lw = nullptr;
    uint64_t m2 = 0, norder = 0;
    uint64_t m_run = 0;  // traversal-graph edges at the last propagation run
    lpf::F2* logfact = nullptr;  // log(j!) for j < logfact_n
    uint64_t logfact_n = 0;
    lpf::F2* recip = nullptr;    // 1/j for j < recip_n
    uint64_t recip_n = 0;
};

// A CUDA graph recorded from a body of stream work (owned; freed on scope exit).
struct SweepGraph {
    cudaGraphExec_t exec = nullptr;
    uint64_t launches = 0;  // kernels in the graph
    SweepGraph() = default;
    SweepGraph(const SweepGraph&) = delete;
    SweepGraph& operator=(const SweepGraph&) = delete;
    ~SweepGraph() {
        if (exec) cudaGraphExecDestroy(exec);
    }
    template <class Body>
    int record(mdet_ctx* ctx, Body body) {
        if (!ctx->cap_stream)
            MDET_CUDA(ctx, cudaStreamCreateWithFlags(&ctx->cap_stream, cudaStreamNonBlocking));
        if (!ctx->cap_stream2)
            MDET_CUDA(ctx, cudaStreamCreateWithFlags(&ctx->cap_stream2, cudaStreamNonBlocking));
        if (!ctx->cap_fork) MDET_CUDA(ctx, cudaEventCreateWithFlags(&ctx->cap_fork, cudaEventDisableTiming));
        if (!ctx->cap_join) MDET_CUDA(ctx, cudaEventCreateWithFlags(&ctx->cap_join, cudaEventDisableTiming));
        const cudaStream_t cs = ctx->cap_stream;
        MDET_CUDA(ctx, cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal));
        const uint64_t l0 = ctx->launches;
        body(cs);
        launches = ctx->launches - l0;
        ctx->launches = l0;  // counted per replay
        const cudaError_t le = cudaGetLastError();  // a launch that failed to enqueue
        cudaGraph_t graph = nullptr;
        const cudaError_t ce = cudaStreamEndCapture(cs, &graph);
        int rc = ctx_cuda(ctx, le != cudaSuccess ? le : ce, "sweep capture");
        if (rc == MDET_OK) rc = ctx_cuda(ctx, cudaGraphInstantiate(&exec, graph, 0), "sweep graph instantiate");
        if (graph) cudaGraphDestroy(graph);
        return rc;
    }
};

// One propagation call over the traversal graph (m2 edges) and order.
int lp_call(mdet_ctx* ctx, LpState& S, mdet_lp_stats* st) {
    cudaStream_t s = ctx->stream;
    const uint64_t n = S.n, m = S.m2, no = S.norder;
    // incidence lists
    uint32_t* ikey = (uint32_t*)ctx_scratch(ctx, "lp.ikey", 2 * m * 4 + 8);
    uint32_t* ival = (uint32_t*)ctx_scratch(ctx, "lp.ival", 2 * m * 4 + 8);
    uint32_t* ikey2 = (uint32_t*)ctx_scratch(ctx, "lp.ikey2", 2 * m * 4 + 8);
    uint32_t* inc = (uint32_t*)ctx_scratch(ctx, "lp.inc", 2 * m * 4 + 8);
    uint32_t* oth = (uint32_t*)ctx_scratch(ctx, "lp.oth", 2 * m * 4 + 8);
    double* ilw = (double*)ctx_scratch(ctx, "lp.ilw", 2 * m * 8 + 8);
    unsigned int* deg = (unsigned int*)ctx_scratch(ctx, "lp.deg", (n + 1) * 4);
    uint32_t* inc_off = (uint32_t*)ctx_scratch(ctx, "lp.incoff", (n + 1) * 4);
    uint32_t* pos_of = (uint32_t*)ctx_scratch(ctx, "lp.pos", n * 4);
    uint32_t* pred = (uint32_t*)ctx_scratch(ctx, "lp.pred", n * 4);
    uint32_t* lvl = (uint32_t*)ctx_scratch(ctx, "lp.lvl", (no + 1) * 4);
    uint32_t* lvls = (uint32_t*)ctx_scratch(ctx, "lp.lvls", (no + 1) * 4);
    uint32_t* slot_of = (uint32_t*)ctx_scratch(ctx, "lp.slotof", n * 4);
    if (!ikey || !ival || !ikey2 || !inc || !oth || !ilw || !deg || !inc_off || !pos_of || !pred || !lvl || !lvls ||
        !slot_of)
        return MDET_ERR_NOMEM;
    ctx_timer_begin(ctx, "lp_levels");
    MDET_CUDA(ctx, cudaMemsetAsync(deg, 0, (n + 1) * 4, s));
    k_lp_inc_keys<<<grid_for(m), 256, 0, s>>>(S.ea, S.eb, m, ikey, ival, deg);
    MDET_LAUNCHED(ctx, "k_lp_inc_keys");
    {
        size_t tb = 0;
        cub::DeviceRadixSort::SortPairs(nullptr, tb, ikey, ikey2, ival, inc, (int)(2 * m), 0, 32, s);
        void* tmp = ctx_scratch(ctx, "lp.sorttmp", tb);
        if (!tmp) return MDET_ERR_NOMEM;
        MDET_CUDA(ctx, cub::DeviceRadixSort::SortPairs(tmp, tb, ikey, ikey2, ival, inc, (int)(2 * m), 0, 32, s));
        tb = 0;
        cub::DeviceScan::ExclusiveSum(nullptr, tb, deg, inc_off, (int)(n + 1), s);
        tmp = ctx_scratch(ctx, "lp.scantmp", tb);
        if (!tmp) return MDET_ERR_NOMEM;
        MDET_CUDA(ctx, cub::DeviceScan::ExclusiveSum(tmp, tb, deg, inc_off, (int)(n + 1), s));
    }
    k_lp_inc_fill<<<grid_for(2 * m), 256, 0, s>>>(inc, ikey2, 2 * m, S.ea, S.eb, S.lw, oth, ilw);
    MDET_LAUNCHED(ctx, "k_lp_inc_fill");
    // dependency levels: per level, the warp contigs (lvls) and the block
    // contigs (lvl), each list's levels stored one after another
    MDET_CUDA(ctx, cudaMemsetAsync(pos_of, 0xFF, n * 4, s));
    k_lp_pos<<<grid_for(no), 256, 0, s>>>(S.order, (uint32_t)no, pos_of);
    MDET_LAUNCHED(ctx, "k_lp_pos");
    // levels: Kahn steps queued sixteen at a time, their table read back once
    // per batch
    const uint64_t lcap = no + 18;
    LevelInfo* info = (LevelInfo*)ctx_scratch(ctx, "lp.info", lcap * sizeof(LevelInfo));
    if (!info) return MDET_ERR_NOMEM;
    MDET_CUDA(ctx, cudaMemsetAsync(info, 0, lcap * sizeof(LevelInfo), s));
    k_lp_pred<<<grid_for(no * 32), 256, 0, s>>>(S.order, (uint32_t)no, pos_of, inc_off, oth, pred, lvl, lvls, info,
                                                 slot_of);
    MDET_LAUNCHED(ctx, "k_lp_pred");
    std::vector<uint64_t> loff{0}, soff{0};
    std::vector<LevelInfo> linfo;
    uint64_t done = 0;
    uint32_t maxdeg = 0, maxall = 0, maxbig = 0;
    const unsigned kgrid = (unsigned)ctx->num_sms * 8;
    std::vector<LevelInfo> batch(17);
    for (uint32_t L0 = 0; done < no && L0 + 17 <= lcap;) {
        for (uint32_t L = L0; L < L0 + 16; ++L) {
            k_lp_kahn<<<kgrid, 256, 0, s>>>(L, pos_of, inc_off, oth, pred, lvl, lvls, info, slot_of);
            MDET_LAUNCHED(ctx, "k_lp_kahn");
        }
        MDET_CUDA(ctx, cudaMemcpyAsync(batch.data(), info + L0, 17 * sizeof(LevelInfo), cudaMemcpyDeviceToHost, s));
        MDET_CUDA(ctx, cudaStreamSynchronize(s));
        bool ended = false;
        for (int k = 0; k < 16; ++k) {
            const LevelInfo& h = batch[k];
            if (h.count + h.nsmall == 0) {
                ended = true;
                break;
            }
            linfo.push_back(h);
            maxdeg = std::max(maxdeg, h.maxdeg);
            maxall = std::max(maxall, h.maxall);
            maxbig = std::max(maxbig, h.nbig);
            loff.push_back(h.off + h.count);
            soff.push_back(h.soff + h.nsmall);
            done += h.count + h.nsmall;
        }
        if (ended || done >= no) break;
        L0 += 16;
    }
    ctx_timer_end(ctx, "lp_levels");
    if (done != no) return ctx_fail(ctx, MDET_ERR_INTERNAL, "label propagation: %llu of %llu contigs levelled",
                                    (unsigned long long)done, (unsigned long long)no);
    st->levels_max = std::max<uint64_t>(st->levels_max, linfo.size());
    st->degree_max = std::max<uint64_t>(st->degree_max, maxall);
    maxdeg = std::max(maxdeg, kWarpCap);
    // the CDF's log-factorials up to the largest label count
    // (one thread sums the table in order; it is rebuilt only when a run
    // needs a longer one)
    if ((uint64_t)maxdeg + 2 > S.logfact_n) {
        const uint64_t len = std::max<uint64_t>((uint64_t)maxdeg + 2, 2 * S.logfact_n);
        S.logfact = (lpf::F2*)ctx_scratch(ctx, "lp.logfact", len * sizeof(lpf::F2));
        if (!S.logfact) return MDET_ERR_NOMEM;
        k_lp_logfact<<<1, 1, 0, s>>>(S.logfact, (uint32_t)len);
        MDET_LAUNCHED(ctx, "k_lp_logfact");
        S.logfact_n = len;
        // the series runs past c by up to a few thousand steps; beyond the
        // table the CDF divides, with the same result
        S.recip_n = len + 8192;
        S.recip = (lpf::F2*)ctx_scratch(ctx, "lp.recip", S.recip_n * sizeof(lpf::F2));
        if (!S.recip) return MDET_ERR_NOMEM;
        k_lp_recip<<<grid_for(S.recip_n), 256, 0, s>>>(S.recip, (uint32_t)S.recip_n);
        MDET_LAUNCHED(ctx, "k_lp_recip");
    }
    const lpf::F2* logfact = S.logfact;
    // global sort slices for the contigs with more than kSmallCap edges
    const size_t big_stride = maxdeg > kSmallCap ? (ws_bytes(pow2_at_least(maxdeg)) + 255) / 256 * 256 : 0;
    unsigned char* big_ws = nullptr;
    if (maxbig) {
        big_ws = (unsigned char*)ctx_scratch(ctx, "lp.bigws", big_stride * maxbig);
        if (!big_ws) return MDET_ERR_NOMEM;
    }
    const size_t small_max = ws_bytes(kSmallCap);
    MDET_CUDA(ctx, cudaFuncSetAttribute(k_lp_level, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)small_max));
    // visited table: sized for the order, doubled (and the call re-run from
    // its starting labels) when a call overfills it
    uint64_t vt_cap = 1u << 20;
    while (vt_cap < 8 * no) vt_cap <<= 1;
    // which contigs the first sweep evaluates; kept with the labels for a re-run
    k_lp_dirty_stuck<<<grid_for(n), 256, 0, s>>>(S.stuck, n, S.dirty);
    MDET_LAUNCHED(ctx, "k_lp_dirty_stuck");
    if (m > S.m_run) {
        k_lp_dirty_edges<<<grid_for(m - S.m_run), 256, 0, s>>>(S.ea, S.eb, S.m_run, m, S.dirty);
        MDET_LAUNCHED(ctx, "k_lp_dirty_edges");
    }
    S.m_run = m;
    MDET_CUDA(ctx, cudaMemcpyAsync(S.mem0, S.mem, n * 4, cudaMemcpyDeviceToDevice, s));
    MDET_CUDA(ctx, cudaMemcpyAsync(S.dirty0, S.dirty, n, cudaMemcpyDeviceToDevice, s));
    for (int attempt_table = 0;; ++attempt_table) {
        unsigned long long* vt = (unsigned long long*)ctx_scratch(ctx, "lp.vt", vt_cap * 8);
        if (!vt) return MDET_ERR_NOMEM;
        MDET_CUDA(ctx, cudaMemsetAsync(vt, 0, vt_cap * 8, s));
        MDET_CUDA(ctx, cudaMemsetAsync(S.stuck, 0, n, s));
        MDET_CUDA(ctx, cudaMemsetAsync(S.cnt, 0, 4 * 8, s));
        LpArgs P{inc_off,  oth,   ilw,       S.mem,   S.stuck,    S.dirty,          vt,
                 vt_cap - 1, logfact, S.recip, (uint32_t)S.recip_n, S.cnt, big_ws, big_stride, maxbig, slot_of};
        uint64_t low = INT_MAX, attempt = 0, sweeps = 0;
        unsigned long long* hc = (unsigned long long*)ctx_pinned(ctx, 32);
        if (!hc) return MDET_ERR_NOMEM;
        bool overfull = false;
        // one sweep -- the moved counter cleared, a launch or two per level,
        // the counters copied back -- recorded once as a CUDA graph on the
        // context's capture stream and replayed on its stream for every sweep.
        // A level's contigs are never neighbours of one another (a contig's
        // level exceeds its earlier neighbours'), so its warp-per-contig and
        // block-per-contig launches are independent branches of the graph,
        // joined before the next level.
        SweepGraph sg;
        MDET_TRY(sg.record(ctx, [&](cudaStream_t cs) {
            const cudaStream_t cs2 = ctx->cap_stream2;
            cudaMemsetAsync(S.cnt, 0, 8, cs);
            for (size_t L = 0; L < linfo.size(); ++L) {
                const bool both = linfo[L].nsmall && linfo[L].count;
                if (both) {
                    cudaEventRecord(ctx->cap_fork, cs);
                    cudaStreamWaitEvent(cs2, ctx->cap_fork, 0);
                }
                if (linfo[L].nsmall) {
                    k_lp_level_warp<<<(linfo[L].nsmall + kWarpsPerBlock - 1) / kWarpsPerBlock, kThreads, 0, cs>>>(
                        P, lvls + soff[L], linfo[L].nsmall);
                    ctx->launches++;
                }
                if (linfo[L].count) {
                    const uint32_t cap = std::min<uint32_t>(pow2_at_least(linfo[L].maxdeg), kSmallCap);
                    k_lp_level<<<linfo[L].count, kThreads, ws_bytes(cap), both ? cs2 : cs>>>(P, lvl + loff[L]);
                    ctx->launches++;
                }
                if (both) {
                    cudaEventRecord(ctx->cap_join, cs2);
                    cudaStreamWaitEvent(cs, ctx->cap_join, 0);
                }
            }
            cudaMemcpyAsync(hc, S.cnt, 32, cudaMemcpyDeviceToHost, cs);
        }));
        while (true) {
            ctx_timer_begin(ctx, "lp_sweep");
            MDET_CUDA(ctx, cudaGraphLaunch(sg.exec, s));
            ctx->launches += sg.launches;
            ctx->total_launches += sg.launches;
            ctx_timer_end(ctx, "lp_sweep");
            MDET_CUDA(ctx, cudaStreamSynchronize(s));
            ++sweeps;
            if (hc[2] & (kErrSlots | kErrScore))
                return ctx_fail(ctx, MDET_ERR_INTERNAL, "label propagation: flags %llu", hc[2]);
            if (hc[2] & kErrTable) {
                overfull = true;
                break;
            }
            const uint64_t moved = hc[0];
            if (moved < low) {
                low = moved;
                attempt = 0;
            } else if (++attempt >= 10) {
                break;
            }
            if (moved == 0) break;
        }
        if (!overfull) {
            st->sweeps += sweeps;
            st->ties += hc[3];
            break;
        }
        if (attempt_table >= 6) return ctx_fail(ctx, MDET_ERR_CAPACITY, "label propagation: visited table");
        vt_cap <<= 1;
        MDET_CUDA(ctx, cudaMemcpyAsync(S.mem, S.mem0, n * 4, cudaMemcpyDeviceToDevice, s));
        MDET_CUDA(ctx, cudaMemcpyAsync(S.dirty, S.dirty0, n, cudaMemcpyDeviceToDevice, s));
    }
    MDET_CUDA(ctx, cudaMemsetAsync(S.cnt + 2, 0, 8, s));
    k_lp_count_stuck<<<std::min<unsigned>(grid_for(n), 1024), 256, 0, s>>>(S.stuck, n, S.cnt + 2);
    MDET_LAUNCHED(ctx, "k_lp_count_stuck");
    unsigned long long fz = 0;
    MDET_CUDA(ctx, cudaMemcpyAsync(&fz, S.cnt + 2, 8, cudaMemcpyDeviceToHost, s));
    MDET_CUDA(ctx, cudaStreamSynchronize(s));
    st->frozen += fz;
    return MDET_OK;
}

int lp_impl(mdet_ctx* ctx, const uint64_t* d_from, const uint64_t* d_to, const double* d_sscr, uint64_t ne,
            uint64_t n, double max_p, double min_s, uint64_t* d_out, mdet_lp_stats* st) {
    cudaStream_t s = ctx->stream;
    LpState S;
    S.n = n;
    S.ne = ne;
    const uint64_t ne1 = std::max<uint64_t>(ne, 1);
    uint32_t* ord0 = (uint32_t*)ctx_scratch(ctx, "lp.ord0", ne1 * 4);
    uint32_t* ord = (uint32_t*)ctx_scratch(ctx, "lp.ord", ne1 * 4);
    double* key2 = (double*)ctx_scratch(ctx, "lp.skey", ne1 * 8);
    S.sa = (uint32_t*)ctx_scratch(ctx, "lp.sa", ne1 * 4);
    S.sb = (uint32_t*)ctx_scratch(ctx, "lp.sb", ne1 * 4);
    S.ss = (double*)ctx_scratch(ctx, "lp.ss", ne1 * 8);
    S.mem = (uint32_t*)ctx_scratch(ctx, "lp.mem", n * 4);
    S.mem0 = (uint32_t*)ctx_scratch(ctx, "lp.mem0", n * 4);
    S.order = (uint32_t*)ctx_scratch(ctx, "lp.order", n * 4);
    S.seen = (uint8_t*)ctx_scratch(ctx, "lp.seen", n);
    S.stuck = (uint8_t*)ctx_scratch(ctx, "lp.stuck", n);
    S.dirty = (uint8_t*)ctx_scratch(ctx, "lp.dirty", n);
    S.dirty0 = (uint8_t*)ctx_scratch(ctx, "lp.dirty0", n);
    S.eflag = (uint8_t*)ctx_scratch(ctx, "lp.eflag", std::min<uint64_t>(ne1, 1ull << 22));
    S.first = (unsigned long long*)ctx_scratch(ctx, "lp.first", n * 8);
    S.cnt = (unsigned long long*)ctx_scratch(ctx, "lp.cnt", 64);
    S.ea = (uint32_t*)ctx_scratch(ctx, "lp.ea", ne1 * 4);
    S.eb = (uint32_t*)ctx_scratch(ctx, "lp.eb", ne1 * 4);
    S.lw = (double*)ctx_scratch(ctx, "lp.lw", ne1 * 8);
    const uint64_t kChunk = std::min<uint64_t>(ne1, 1ull << 22);  // edges traversed per pass
    uint8_t* slot = (uint8_t*)ctx_scratch(ctx, "lp.slot", 2 * kChunk);
    uint32_t* ssel = (uint32_t*)ctx_scratch(ctx, "lp.ssel", 2 * kChunk * 4);
    uint32_t* sel = (uint32_t*)ctx_scratch(ctx, "lp.sel", kChunk * 4);
    if (!ord0 || !ord || !key2 || !S.sa || !S.sb || !S.ss || !S.mem || !S.mem0 || !S.order || !S.seen || !S.stuck || !S.dirty || !S.dirty0 ||
        !S.eflag || !S.first || !S.cnt || !S.ea || !S.eb || !S.lw || !slot || !ssel || !sel)
        return MDET_ERR_NOMEM;
    k_lp_iota<<<grid_for(n), 256, 0, s>>>(S.mem, n);
    MDET_LAUNCHED(ctx, "k_lp_iota");
    MDET_CUDA(ctx, cudaMemsetAsync(S.seen, 0, n, s));
    MDET_CUDA(ctx, cudaMemsetAsync(S.stuck, 0, n, s));
    MDET_CUDA(ctx, cudaMemsetAsync(S.dirty, 0, n, s));
    if (ne) {
        // edges by decreasing score; equal scores keep edge order (stable)
        k_lp_iota<<<grid_for(ne), 256, 0, s>>>(ord0, ne);
        MDET_LAUNCHED(ctx, "k_lp_iota");
        size_t tb = 0;
        cub::DeviceRadixSort::SortPairsDescending(nullptr, tb, d_sscr, key2, ord0, ord, (int)ne, 0, 64, s);
        void* tmp = ctx_scratch(ctx, "lp.esort", tb);
        if (!tmp) return MDET_ERR_NOMEM;
        MDET_CUDA(ctx, cub::DeviceRadixSort::SortPairsDescending(tmp, tb, d_sscr, key2, ord0, ord, (int)ne, 0, 64, s));
        MDET_CUDA(ctx, cudaMemsetAsync(S.cnt, 0, 64, s));
        k_lp_gather<<<std::min<unsigned>(grid_for(ne), 8 * ctx->num_sms), 256, 0, s>>>(d_from, d_to, d_sscr, ord, ne,
                                                                                       n, S.sa, S.sb, S.ss, S.cnt);
        MDET_LAUNCHED(ctx, "k_lp_gather");
        unsigned long long bad = 0;
        MDET_CUDA(ctx, cudaMemcpyAsync(&bad, S.cnt, 8, cudaMemcpyDeviceToHost, s));
        MDET_CUDA(ctx, cudaStreamSynchronize(s));
        if (bad) return ctx_fail(ctx, MDET_ERR_INVALID, "label propagation: a score outside [0, 1] or a contig >= n");
    }
    std::vector<double> sched;
    for (int i = 1; i <= 10; ++i) sched.push_back(max_p / 10 * i);
    size_t which = 0;
    uint64_t pos = 0;
    constexpr uint64_t kNone = ~0ull;
    // select the set flags of [0, cnt) into out; returns how many
    auto select = [&](const uint8_t* flags, uint64_t cnt, uint32_t* out, const char* tag) -> long long {
        thrust::counting_iterator<uint32_t> it(0);
        size_t tb = 0;
        cub::DeviceSelect::Flagged(nullptr, tb, it, flags, out, S.cnt + 3, (int)cnt, s);
        void* tmp = ctx_scratch(ctx, tag, tb);
        if (!tmp) return -MDET_ERR_NOMEM;
        if (ctx_cuda(ctx, cub::DeviceSelect::Flagged(tmp, tb, it, flags, out, S.cnt + 3, (int)cnt, s), "select"))
            return -MDET_ERR_CUDA;
        unsigned long long k = 0;
        if (ctx_cuda(ctx, cudaMemcpyAsync(&k, S.cnt + 3, 8, cudaMemcpyDeviceToHost, s), "select count") ||
            ctx_cuda(ctx, cudaStreamSynchronize(s), "select count"))
            return -MDET_ERR_CUDA;
        return (long long)k;
    };
    while (ne && pos < ne) {
        ctx_timer_begin(ctx, "lp_traverse");
        MDET_CUDA(ctx, cudaMemsetAsync(S.first, 0xFF, n * 8, s));
        // connected contigs the schedule asks for
        const double thr = sched[which];
        uint64_t c_need = (uint64_t)std::ceil(thr * (double)n);
        while (c_need > 0 && (double)(c_need - 1) / (double)n >= thr) --c_need;
        while ((double)c_need / (double)n < thr) ++c_need;
        uint64_t first_add = S.m2 > 0 ? pos : kNone;   // the graph has an edge from here on
        uint64_t i_c = c_need <= S.norder ? pos : kNone;  // the connected count is reached here
        uint64_t i_run = kNone;
        bool at_last = false, ended = false;
        // the stretch from pos, a chunk at a time, until the run position
        for (uint64_t p0 = pos;;) {
            const uint64_t p1 = std::min(ne, p0 + kChunk);
            unsigned long long h2[2] = {kNone, kNone};
            MDET_CUDA(ctx, cudaMemcpyAsync(S.cnt, h2, 16, cudaMemcpyHostToDevice, s));
            k_lp_seg<<<std::min<unsigned>(grid_for(p1 - p0), 8 * ctx->num_sms), 256, 0, s>>>(S.sa, S.sb, S.ss, p0,
                                                                                             p1, S.mem, min_s, S.cnt);
            MDET_LAUNCHED(ctx, "k_lp_seg");
            MDET_CUDA(ctx, cudaMemcpyAsync(h2, S.cnt, 16, cudaMemcpyDeviceToHost, s));
            MDET_CUDA(ctx, cudaStreamSynchronize(s));
            const bool stop_here = h2[0] != kNone;
            const uint64_t end = stop_here ? h2[0] + 1 : p1;   // [p0, end) is traversed
            const uint64_t last_here = end - 1;
            const bool is_last = stop_here || p1 == ne;
            if (first_add == kNone && h2[1] != kNone && h2[1] < end) first_add = h2[1];
            // the contigs first seen in [p0, end), in first-seen order
            k_lp_first<<<std::min<unsigned>(grid_for(end - p0), 8 * ctx->num_sms), 256, 0, s>>>(
                S.sa, S.sb, p0, end, S.mem, S.seen, S.first);
            MDET_LAUNCHED(ctx, "k_lp_first");
            k_lp_slots<<<grid_for(end - p0), 256, 0, s>>>(S.sa, S.sb, p0, end - p0, S.mem, S.seen, S.first, slot);
            MDET_LAUNCHED(ctx, "k_lp_slots");
            const long long kn = select(slot, 2 * (end - p0), ssel, "lp.seltmp");
            if (kn < 0) return (int)-kn;
            if (i_c == kNone && S.norder + (uint64_t)kn >= c_need) {
                uint32_t sl = 0;
                MDET_CUDA(ctx, cudaMemcpyAsync(&sl, ssel + (c_need - S.norder - 1), 4, cudaMemcpyDeviceToHost, s));
                MDET_CUDA(ctx, cudaStreamSynchronize(s));
                i_c = p0 + (sl >> 1);
            }
            if (first_add != kNone && i_c != kNone && std::max(i_c, first_add) <= last_here) {
                i_run = std::max(i_c, first_add);
            } else if (is_last) {
                if (first_add != kNone)
                    i_run = last_here;
                else
                    ended = true;  // no edge joins: the traversal ends without a run
            }
            at_last = is_last && i_run == last_here;
            // commit [p0, cend): the new contigs and the joining edges
            const uint64_t cend = i_run != kNone ? i_run + 1 : end;
            uint64_t kc = (uint64_t)kn;
            if (cend < end && kn > 0) {  // the selected slots below 2 * (cend - p0), by bisection
                std::vector<uint32_t> hs((size_t)kn);
                MDET_CUDA(ctx, cudaMemcpyAsync(hs.data(), ssel, (size_t)kn * 4, cudaMemcpyDeviceToHost, s));
                MDET_CUDA(ctx, cudaStreamSynchronize(s));
                kc = (uint64_t)(std::lower_bound(hs.begin(), hs.end(), (uint32_t)(2 * (cend - p0))) - hs.begin());
            }
            if (kc) {
                k_lp_take<<<grid_for(kc), 256, 0, s>>>(ssel, kc, p0, S.sa, S.sb, S.order + S.norder, S.seen);
                MDET_LAUNCHED(ctx, "k_lp_take");
                S.norder += kc;
            }
            k_lp_edge_flags<<<grid_for(cend - p0), 256, 0, s>>>(S.sa, S.sb, S.ss, p0, cend - p0, S.mem, min_s,
                                                                 S.eflag);
            MDET_LAUNCHED(ctx, "k_lp_edge_flags");
            const long long ka = select(S.eflag, cend - p0, sel, "lp.seltmp2");
            if (ka < 0) return (int)-ka;
            if (ka) {
                k_lp_append<<<grid_for((uint64_t)ka), 256, 0, s>>>(sel, (uint64_t)ka, p0, S.sa, S.sb, S.ss,
                                                                  S.ea + S.m2, S.eb + S.m2, S.lw + S.m2);
                MDET_LAUNCHED(ctx, "k_lp_append");
                S.m2 += (uint64_t)ka;
            }
            if (i_run != kNone || ended) break;
            p0 = end;
        }
        ctx_timer_end(ctx, "lp_traverse");
        if (ended) break;
        ++st->calls;
        MDET_TRY(lp_call(ctx, S, st));
        if (++which == sched.size() || at_last) break;
        pos = i_run + 1;
    }
    st->graph_edges = S.m2;
    st->connected = S.norder;
    k_lp_widen<<<grid_for(n), 256, 0, s>>>(S.mem, n, d_out);
    MDET_LAUNCHED(ctx, "k_lp_widen");
    return MDET_OK;
}

}  // namespace

extern "C" {

int mdet_label_propagation_dev(mdet_ctx* ctx, const uint64_t* d_from, const uint64_t* d_to, const double* d_sscr,
                               uint64_t n_edges, uint64_t n, double max_p, double min_s, uint64_t* d_mem,
                               mdet_lp_stats* stats) {
    if (!ctx) return MDET_ERR_INVALID;
    MDET_CUDA(ctx, cudaSetDevice(ctx->device));
    mdet_lp_stats st{};
    if (stats) *stats = st;
    if (n == 0) return MDET_OK;
    if (!d_mem || (n_edges && (!d_from || !d_to || !d_sscr))) return ctx_fail(ctx, MDET_ERR_INVALID, "null pointer");
    if (n >= 0x7FFFFFFFull || n_edges >= 0x3FFFFFFFull)
        return ctx_fail(ctx, MDET_ERR_INVALID, "label propagation: 2^31 contigs or 2^30 edges or more");
    if (!(max_p > 0 && max_p <= 1) || !(min_s >= 0 && min_s < 1))
        return ctx_fail(ctx, MDET_ERR_INVALID, "label propagation: max_p in (0, 1], min_s in [0, 1)");
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventRecord(e0, ctx->stream);
    int rc = lp_impl(ctx, d_from, d_to, d_sscr, n_edges, n, max_p, min_s, d_mem, &st);
    cudaEventRecord(e1, ctx->stream);
    if (rc == MDET_OK) {
        cudaEventSynchronize(e1);
        float ms = 0;
        cudaEventElapsedTime(&ms, e0, e1);
        st.ms_total = ms;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc == MDET_OK) rc = check_flag(ctx);
    if (stats) *stats = st;
    return rc;
}

int mdet_label_propagation(mdet_ctx* ctx, const uint64_t* from, const uint64_t* to, const double* sscr,
                           uint64_t n_edges, uint64_t n, double max_p, double min_s, uint64_t* mem,
                           mdet_lp_stats* stats) {
    if (!ctx) return MDET_ERR_INVALID;
    MDET_CUDA(ctx, cudaSetDevice(ctx->device));
    if (n == 0) {
        if (stats) *stats = mdet_lp_stats{};
        return MDET_OK;
    }
    if (!mem || (n_edges && (!from || !to || !sscr))) return ctx_fail(ctx, MDET_ERR_INVALID, "null pointer");
    cudaStream_t s = ctx->stream;
    const uint64_t ne1 = std::max<uint64_t>(n_edges, 1);
    uint64_t* d_from = (uint64_t*)ctx_scratch(ctx, "lpio.from", ne1 * 8);
    uint64_t* d_to = (uint64_t*)ctx_scratch(ctx, "lpio.to", ne1 * 8);
    double* d_s = (double*)ctx_scratch(ctx, "lpio.sscr", ne1 * 8);
    uint64_t* d_mem = (uint64_t*)ctx_scratch(ctx, "lpio.mem", n * 8);
    if (!d_from || !d_to || !d_s || !d_mem) return MDET_ERR_NOMEM;
    if (n_edges) {
        MDET_CUDA(ctx, cudaMemcpyAsync(d_from, from, n_edges * 8, cudaMemcpyHostToDevice, s));
        MDET_CUDA(ctx, cudaMemcpyAsync(d_to, to, n_edges * 8, cudaMemcpyHostToDevice, s));
        MDET_CUDA(ctx, cudaMemcpyAsync(d_s, sscr, n_edges * 8, cudaMemcpyHostToDevice, s));
    }
    MDET_TRY(mdet_label_propagation_dev(ctx, d_from, d_to, d_s, n_edges, n, max_p, min_s, d_mem, stats));
    MDET_CUDA(ctx, cudaMemcpyAsync(mem, d_mem, n * 8, cudaMemcpyDeviceToHost, s));
    MDET_CUDA(ctx, cudaStreamSynchronize(s));
    return MDET_OK;
}

}  // extern "C"
