// graph_exact.cu -- exact scoring of filtered pairs and per-contig top-k.
//
// Every pair that passed a distance filter is scored again from the FP32
// TNF rows: the reference's terms float((a_k - b_k)^2) (cuda/Cuda2.cu:194-196)
// summed with compensated FP32 arithmetic, the square root and the MetaBAT2
// logistic model (cuda/Cuda2.cu:199-240) in float-float arithmetic (ff.cuh,
// about 48 significant bits) from per-contig parts F(x), G(y) and the pair
// term H(x*y).  A pair is an edge when its
// pre-probability beats logit(cutoff) (cuda/Cuda2.cu:257-260); its score is
// sigmoid(pre).  Edges are then grouped per contig (both directions), each
// contig keeps its best max_edges by (score desc, original column asc), and
// (i, j) is emitted for i < j in original indices (cuda/Cuda2.cu:921-946).
#include <cub/cub.cuh>

#include "exact.cuh"

using namespace mdet_exact;

namespace {

struct ExactArgs {
    const uint2* cand;
    unsigned long long ncand;
    const uint32_t* row_map;  // maxprob: sample slot -> sorted position; graph: null
    bool swapped;             // maxprob: pairs are (sorted position, sample slot)
    const float* x32;
    const PartsFF* parts;
    ModelHFF H;
    double L;
    ff Lff;
    const BlkCut* blk_L;  // optional per-256-row-block cutoff
    const unsigned long long* ncand_dev;  // optional device candidate count (ncand is then its cap)
    const uint8_t* low;   // optional abundance gate per sorted position (graph only)
    // graph outputs
    Edge* edges;
    unsigned long long* nedges;
    uint32_t* deg;
    // maxprob output
    unsigned long long* maxkey;
};

// Squared distances of 32 candidates per warp: candidate base + L belongs to
// lane L.  Eight lanes share one candidate at a time, so each row is read in
// coalesced 128-byte runs (lane k of the group takes float4 columns k, k+8,
// ...); partial sums keep their rounding errors (TwoSum) through the group
// reduction.  Returns the owner lane's (sum, error) pair and its rows.
__device__ __forceinline__ ff warp_dist2(const uint2* __restrict__ cand, unsigned long long ncand,
                                         unsigned long long base, const uint32_t* __restrict__ row_map,
                                         const float* __restrict__ x32, uint32_t lane, uint32_t& si, uint32_t& sj,
                                         bool swapped = false) {
    const uint32_t grp = lane >> 3, sub = lane & 7;
    // every lane loads its own candidate once (one coalesced read for the
    // warp); the rounds below take the row indices by shuffle, so the row
    // reads of a round depend on no further load
    const bool own = base + lane < ncand;
    si = sj = 0;
    if (own) {
        uint2 cd = cand[base + lane];
        if (swapped) cd = make_uint2(cd.y, cd.x);
        si = row_map ? row_map[cd.x] : cd.x;
        sj = cd.y;
    }
    float ms = 0.f, mc = 0.f;
#pragma unroll 1
    for (uint32_t it = 0; it < 8; ++it) {
        const uint32_t from = it * 4 + grp;  // lane owning the candidate of this group and round
        const unsigned long long k = base + from;
        const uint32_t a = __shfl_sync(0xffffffffu, si, from);
        const uint32_t b = __shfl_sync(0xffffffffu, sj, from);
        float s = 0.f, c = 0.f;
        if (k < ncand) {
            const float4* ra = reinterpret_cast<const float4*>(x32 + (uint64_t)a * MDET_NTNF);
            const float4* rb = reinterpret_cast<const float4*>(x32 + (uint64_t)b * MDET_NTNF);
#pragma unroll
            for (uint32_t q = 0; q < 5; ++q) {
                const uint32_t col = sub + 8 * q;
                if (col < MDET_NTNF / 4) {
                    const float4 x = __ldg(ra + col), y = __ldg(rb + col);
                    const float d0 = __fsub_rn(x.x, y.x), d1 = __fsub_rn(x.y, y.y);
                    const float d2 = __fsub_rn(x.z, y.z), d3 = __fsub_rn(x.w, y.w);
                    two_sum_acc(s, c, __fmul_rn(d0, d0));
                    two_sum_acc(s, c, __fmul_rn(d1, d1));
                    two_sum_acc(s, c, __fmul_rn(d2, d2));
                    two_sum_acc(s, c, __fmul_rn(d3, d3));
                }
            }
        }
#pragma unroll
        for (int o = 1; o < 8; o <<= 1) {
            const float s2 = __shfl_xor_sync(0xffffffffu, s, o);
            const float c2 = __shfl_xor_sync(0xffffffffu, c, o);
            const ff t = two_sum(s, s2);
            s = t.hi;
            c = __fadd_rn(__fadd_rn(c, c2), t.lo);
        }
        // candidate base + L was handled in round L / 4 by group L % 4
        const uint32_t src = 8 * (lane & 3);
        const float vs = __shfl_sync(0xffffffffu, s, src);
        const float vc = __shfl_sync(0xffffffffu, c, src);
        if ((lane >> 2) == it) {
            ms = vs;
            mc = vc;
        }
    }
    return quick_two_sum(ms, mc);
}

__global__ void __launch_bounds__(256) k_exact_graph(ExactArgs p) {
    __shared__ uint32_t wcount[8];
    __shared__ unsigned long long bbase;
    if (p.ncand_dev) p.ncand = min(*p.ncand_dev, p.ncand);
    const bool model2 = p.L < kLn9;
    const uint32_t lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    // the block takes 256 candidates per round (32 per warp), so every warp
    // runs the same number of rounds and the block reserves its edge slots
    // with one global atomic per round
    for (unsigned long long bb = (unsigned long long)blockIdx.x * 256; bb < p.ncand;
         bb += (unsigned long long)gridDim.x * 256) {
        const unsigned long long base = bb + 32ull * w;
        uint32_t si, sj;
        const ff d2 = warp_dist2(p.cand, p.ncand, base, nullptr, p.x32, lane, si, sj);
        bool edge = false;
        double sim = 0;
        // a pair of two contigs without a depth above 1 is never an edge (is_nz)
        if (base + lane < p.ncand && !(p.low && p.low[si] && p.low[sj])) {
            ff Lc = p.Lff;
            bool m2 = model2;
            if (p.blk_L) {
                const BlkCut bc = p.blk_L[si >> 8];
                Lc = bc.L;
                m2 = bc.model2 != 0;
            }
            const ff pre = pre_prob(p.parts[si], p.parts[sj], ff_sqrt(d2), p.H, m2);
            if (ff_gt(pre, Lc)) {
                edge = true;
                sim = sim_of(pre);
            }
        }
        const uint32_t bal = __ballot_sync(0xffffffffu, edge);
        if (lane == 0) wcount[w] = __popc(bal);
        __syncthreads();
        if (threadIdx.x == 0) {
            uint32_t t = 0;
            for (int k = 0; k < 8; ++k) t += wcount[k];
            bbase = t ? atomicAdd(p.nedges, (unsigned long long)t) : 0ull;
        }
        __syncthreads();
        uint32_t before = 0;
        for (uint32_t k = 0; k < w; ++k) before += wcount[k];
        if (edge) {
            Edge e;
            e.i = si;
            e.j = sj;
            e.sim = sim;
            p.edges[bbase + before + __popc(bal & ((1u << lane) - 1u))] = e;
            atomicAdd(&p.deg[si], 1u);
            atomicAdd(&p.deg[sj], 1u);
        }
        __syncthreads();  // wcount and bbase are rewritten next round
    }
}

__global__ void __launch_bounds__(256) k_exact_maxprob(ExactArgs p) {
    const uint32_t lane = threadIdx.x & 31;
    const unsigned long long warps = (unsigned long long)gridDim.x * (blockDim.x / 32);
    for (unsigned long long base = ((unsigned long long)blockIdx.x * (blockDim.x / 32) + (threadIdx.x >> 5)) * 32;
         base < p.ncand; base += warps * 32) {
        uint32_t si, sj;
        const ff d2 = warp_dist2(p.cand, p.ncand, base, p.row_map, p.x32, lane, si, sj, p.swapped);
        const unsigned long long idx = base + lane;
        if (idx < p.ncand && si != sj) {  // skip the sampled contig itself
            const ff pre = pre_prob(p.parts[si], p.parts[sj], ff_sqrt(d2), p.H, true);
            const uint2 cd = p.cand[idx];
            atomicMax(&p.maxkey[p.swapped ? cd.y : cd.x], dkey(ff_to_double(pre)));
        }
    }
}

// Distance and probability of given pairs (original indices, mapped through inv).
__global__ void k_pair_scores(const uint64_t* __restrict__ pairs, uint64_t m, const uint32_t* __restrict__ inv,
                              const float* __restrict__ x32, const PartsFF* __restrict__ parts, ModelHFF H,
                              double* __restrict__ dist, double* __restrict__ prob) {
    for (uint64_t q = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; q < m; q += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t i = inv[pairs[2 * q]], j = inv[pairs[2 * q + 1]];
        const ff d = exact_dist(x32 + (uint64_t)i * MDET_NTNF, x32 + (uint64_t)j * MDET_NTNF);
        const ff pre = pre_prob(parts[i], parts[j], d, H, true);
        if (dist) dist[q] = ff_to_double(d);
        if (prob) prob[q] = sim_of(pre);
    }
}

__global__ void k_scatter(const Edge* __restrict__ edges, unsigned long long ne_cap,
                          const unsigned long long* __restrict__ ne_dev, const uint32_t* __restrict__ perm,
                          const unsigned long long* __restrict__ rowptr, uint32_t* __restrict__ cursor,
                          Ent* __restrict__ list) {
    const unsigned long long ne = ne_dev ? min(*ne_dev, ne_cap) : ne_cap;
    for (unsigned long long e = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x; e < ne;
         e += (unsigned long long)gridDim.x * blockDim.x) {
        Edge ed = edges[e];
        uint32_t a = atomicAdd(&cursor[ed.i], 1u);
        uint32_t b = atomicAdd(&cursor[ed.j], 1u);
        Ent x;
        x.sim = ed.sim;
        x.pad = 0;
        x.ocol = perm[ed.j];
        list[rowptr[ed.i] + a] = x;
        x.ocol = perm[ed.i];
        list[rowptr[ed.j] + b] = x;
    }
}

__device__ __forceinline__ bool before(const Ent& a, const Ent& b) {
    return a.sim > b.sim || (a.sim == b.sim && a.ocol < b.ocol);
}

constexpr int kWarpCap = 1024;
constexpr int kTopkWarps = 4;

// Warp per contig (sorted position s) with at most 1024 edges: bitonic sort
// in shared memory, keep the best max_edges in place.
__global__ void __launch_bounds__(kTopkWarps * 32) k_topk_warp(
    const unsigned long long* __restrict__ rowptr, const uint32_t* __restrict__ deg, const uint32_t* __restrict__ perm,
    uint32_t n, uint32_t max_edges, Ent* __restrict__ list, uint32_t* __restrict__ out_cnt,
    uint32_t* __restrict__ big, unsigned int* __restrict__ nbig) {
    extern __shared__ __align__(16) unsigned char sm[];
    const uint32_t w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    Ent* e = reinterpret_cast<Ent*>(sm) + (size_t)w * kWarpCap;
    for (uint32_t s = blockIdx.x * kTopkWarps + w; s < n; s += gridDim.x * kTopkWarps) {
        const uint32_t cnt = deg[s];
        const uint32_t orow = perm[s];
        if (cnt > kWarpCap) {
            if (lane == 0) big[atomicAdd(nbig, 1u)] = s;
            continue;
        }
        Ent* row = list + rowptr[s];
        uint32_t P = 1;
        while (P < cnt) P <<= 1;
        if (cnt > max_edges || cnt > 1) {
            for (uint32_t i = lane; i < P; i += 32) {
                if (i < cnt)
                    e[i] = row[i];
                else {
                    e[i].sim = -1.0;
                    e[i].ocol = 0xFFFFFFFFu;
                }
            }
            __syncwarp();
            for (uint32_t k = 2; k <= P; k <<= 1)
                for (uint32_t j = k >> 1; j > 0; j >>= 1) {
                    for (uint32_t i = lane; i < P; i += 32) {
                        uint32_t ixj = i ^ j;
                        if (ixj > i) {
                            Ent a = e[i], b = e[ixj];
                            bool up = (i & k) == 0;
                            if (up ? before(b, a) : before(a, b)) {
                                e[i] = b;
                                e[ixj] = a;
                            }
                        }
                    }
                    __syncwarp();
                }
        } else {
            for (uint32_t i = lane; i < cnt; i += 32) e[i] = row[i];
            __syncwarp();
        }
        const uint32_t keep = cnt < max_edges ? cnt : max_edges;
        uint32_t c = 0;
        for (uint32_t i = lane; i < keep; i += 32) {
            row[i] = e[i];
            c += e[i].ocol > orow;
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
        if (lane == 0) out_cnt[orow] = c;
        __syncwarp();
    }
}

constexpr int kBigCap = 8192;

// Block per contig with more than 1024 edges: repeated sort of the running
// best plus the next chunk in a 8192-entry shared buffer.
__global__ void __launch_bounds__(1024) k_topk_big(const uint32_t* __restrict__ big, const unsigned int* __restrict__ nbig,
                                                   const unsigned long long* __restrict__ rowptr,
                                                   const uint32_t* __restrict__ deg, const uint32_t* __restrict__ perm,
                                                   uint32_t max_edges, Ent* __restrict__ list,
                                                   uint32_t* __restrict__ out_cnt) {
    extern __shared__ __align__(16) unsigned char sm[];
    Ent* e = reinterpret_cast<Ent*>(sm);
    __shared__ uint32_t red;
    const uint32_t nb = *nbig;
    for (uint32_t bi = blockIdx.x; bi < nb; bi += gridDim.x) {
        const uint32_t s = big[bi];
        const uint32_t cnt = deg[s], orow = perm[s];
        Ent* row = list + rowptr[s];
        uint32_t kept = 0, base = 0;
        while (base < cnt) {
            uint32_t take = min((uint32_t)kBigCap - kept, cnt - base);
            for (uint32_t i = threadIdx.x; i < (uint32_t)kBigCap - kept; i += blockDim.x) {
                if (i < take)
                    e[kept + i] = row[base + i];
                else {
                    e[kept + i].sim = -1.0;
                    e[kept + i].ocol = 0xFFFFFFFFu;
                }
            }
            __syncthreads();
            for (uint32_t k = 2; k <= (uint32_t)kBigCap; k <<= 1)
                for (uint32_t j = k >> 1; j > 0; j >>= 1) {
                    for (uint32_t i = threadIdx.x; i < (uint32_t)kBigCap; i += blockDim.x) {
                        uint32_t ixj = i ^ j;
                        if (ixj > i) {
                            Ent a = e[i], b = e[ixj];
                            bool up = (i & k) == 0;
                            if (up ? before(b, a) : before(a, b)) {
                                e[i] = b;
                                e[ixj] = a;
                            }
                        }
                    }
                    __syncthreads();
                }
            base += take;
            kept = min(max_edges, kept + take);
            __syncthreads();
        }
        if (threadIdx.x == 0) red = 0;
        __syncthreads();
        uint32_t c = 0;
        for (uint32_t i = threadIdx.x; i < kept; i += blockDim.x) {
            row[i] = e[i];
            c += e[i].ocol > orow;
        }
        atomicAdd(&red, c);
        __syncthreads();
        if (threadIdx.x == 0) out_cnt[orow] = red;
        __syncthreads();
    }
}

// ---- selection top-k: warp per contig --------------------------------------
// A row's kept set is its max_edges best entries under (sim descending, ocol
// ascending).  Ordered as the 96-bit key (bits of sim, ~ocol) -- sim is a
// positive double, so its bits order like its value -- the kept set is every
// entry whose key is >= the max_edges-th largest key, found by a radix
// select (8-bit digits, most significant first, stopping as soon as the
// digit's bin holds exactly the entries still needed).  Only kept entries
// with ocol above the row's own index are emitted, so only those are sorted
// (bitonic network in registers: entry i of a chunk of 32*E in lane i % 32,
// slot i / 32) and written to the front of the row.

// Keys are the bit patterns of positive doubles, which order like the
// values, so every comparison is an integer one (FP64 is slow on this part).
__device__ __forceinline__ bool kv_less(unsigned long long s1, uint32_t c1, unsigned long long s2, uint32_t c2) {
    return s1 > s2 || (s1 == s2 && c1 < c2);
}

// In-lane compare-exchange of slots e and e | JE (stride >= 32 entries).
template <int E, int JE>
__device__ __forceinline__ void stage_in_lane(unsigned long long (&s)[E], uint32_t (&c)[E], uint32_t lane,
                                              uint32_t k) {
#pragma unroll
    for (int e = 0; e < E; ++e) {
        if ((e & JE) == 0) {
            const int e2 = e | JE;
            const bool up = ((((uint32_t)e * 32u + lane) & k) == 0);
            const bool sw = up ? kv_less(s[e2], c[e2], s[e], c[e]) : kv_less(s[e], c[e], s[e2], c[e2]);
            const unsigned long long s1 = sw ? s[e2] : s[e], s2 = sw ? s[e] : s[e2];
            const uint32_t c1 = sw ? c[e2] : c[e], c2 = sw ? c[e] : c[e2];
            s[e] = s1;
            s[e2] = s2;
            c[e] = c1;
            c[e2] = c2;
        }
    }
}

template <int E>
__device__ __forceinline__ void bitonic_stage(unsigned long long (&s)[E], uint32_t (&c)[E], uint32_t lane, uint32_t k,
                                              uint32_t j) {
    if (j >= 32) {
        const uint32_t je = j >> 5;
        if (E >= 2 && je == 1) stage_in_lane<E, 1>(s, c, lane, k);
        if (E >= 4 && je == 2) stage_in_lane<E, (E >= 4 ? 2 : 1)>(s, c, lane, k);
        if (E >= 8 && je == 4) stage_in_lane<E, (E >= 8 ? 4 : 1)>(s, c, lane, k);
        if (E >= 16 && je == 8) stage_in_lane<E, (E >= 16 ? 8 : 1)>(s, c, lane, k);
    } else {
        const bool lower = (lane & j) == 0;
#pragma unroll
        for (int e = 0; e < E; ++e) {
            const bool up = ((((uint32_t)e * 32u + lane) & k) == 0);
            const unsigned long long os = __shfl_xor_sync(0xffffffffu, s[e], (int)j);
            const uint32_t oc = __shfl_xor_sync(0xffffffffu, c[e], (int)j);
            const bool take = (lower == up) ? kv_less(os, oc, s[e], c[e]) : kv_less(s[e], c[e], os, oc);
            s[e] = take ? os : s[e];
            c[e] = take ? oc : c[e];
        }
    }
}

// Sorts entries [0, m) of the warp's staging buffer best-first into row[0, m).
template <int E>
__device__ __forceinline__ void sort_out(const unsigned long long* __restrict__ key, const uint32_t* __restrict__ col,
                                         uint32_t m, uint32_t lane, Ent* __restrict__ row) {
    unsigned long long s[E];
    uint32_t c[E];
#pragma unroll
    for (int e = 0; e < E; ++e) {
        const uint32_t i = (uint32_t)e * 32u + lane;
        s[e] = i < m ? key[i] : 0ull;  // padding sorts last (every real key is a positive double)
        c[e] = i < m ? col[i] : 0xFFFFFFFFu;
    }
    uint32_t P = 32u * E;
    while (P / 2 >= m && P > 64) P >>= 1;  // the network only needs the next power of two
#pragma unroll 1
    for (uint32_t k = 2; k <= P; k <<= 1)
#pragma unroll 1
        for (uint32_t j = k >> 1; j > 0; j >>= 1) bitonic_stage<E>(s, c, lane, k, j);
#pragma unroll
    for (int e = 0; e < E; ++e) {
        const uint32_t i = (uint32_t)e * 32u + lane;
        if (i < m) {
            Ent x;
            x.sim = __longlong_as_double((long long)s[e]);
            x.ocol = c[e];
            x.pad = 0;
            row[i] = x;
        }
    }
}

constexpr int kSelWarps = 4;
constexpr uint32_t kSelCap = 896;  // entries staged in shared memory per warp (46 KB per block)

__device__ __forceinline__ uint32_t sel_digit(unsigned long long hi, uint32_t lo, int p) {
    return p < 8 ? (uint32_t)(hi >> (56 - 8 * p)) & 255u : (lo >> (24 - 8 * (p - 8))) & 255u;
}

// key (hi, lo) agrees with the prefix (P_hi, P_lo) on its first p digits
__device__ __forceinline__ bool sel_match(unsigned long long hi, uint32_t lo, unsigned long long P_hi, uint32_t P_lo,
                                          int p) {
    if (p == 0) return true;
    if (p < 8) return (hi >> (64 - 8 * p)) == (P_hi >> (64 - 8 * p));
    if (hi != P_hi) return false;
    return p == 8 || (lo >> (32 - 8 * (p - 8))) == (P_lo >> (32 - 8 * (p - 8)));
}

template <int EMAX>
__global__ void __launch_bounds__(kSelWarps * 32) k_topk_sel(const unsigned long long* __restrict__ rowptr,
                                                             const uint32_t* __restrict__ deg,
                                                             const uint32_t* __restrict__ perm, uint32_t n,
                                                             uint32_t max_edges_all, const uint32_t* __restrict__ blk_K,
                                                             Ent* __restrict__ list, uint32_t* __restrict__ out_cnt) {
    __shared__ unsigned long long s_key[kSelWarps][kSelCap];
    __shared__ uint32_t s_col[kSelWarps][kSelCap];
    __shared__ uint32_t s_hist[kSelWarps][256];
    const uint32_t w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    unsigned long long* key = s_key[w];
    uint32_t* col = s_col[w];
    uint32_t* hist = s_hist[w];
    for (uint32_t sp = blockIdx.x * kSelWarps + w; sp < n; sp += gridDim.x * kSelWarps) {
        const uint32_t cnt = deg[sp], orow = perm[sp];
        const uint32_t max_edges = blk_K ? blk_K[sp >> 8] : max_edges_all;
        Ent* row = list + rowptr[sp];
        const bool staged = cnt <= kSelCap;
        if (staged)
            for (uint32_t i = lane; i < cnt; i += 32) {
                const Ent x = row[i];
                key[i] = (unsigned long long)__double_as_longlong(x.sim);
                col[i] = x.ocol;
            }
        __syncwarp();
        // threshold key (P_hi, P_lo): kept iff key >= it
        unsigned long long P_hi = 0;
        uint32_t P_lo = 0;
        if (cnt > max_edges) {
            uint32_t need = max_edges;
            for (int p = 0; p < 12; ++p) {
#pragma unroll
                for (int t = 0; t < 8; ++t) hist[lane * 8 + t] = 0;
                __syncwarp();
                for (uint32_t i = lane; i < cnt; i += 32) {
                    unsigned long long hi;
                    uint32_t c;
                    if (staged) {
                        hi = key[i];
                        c = col[i];
                    } else {
                        const Ent x = row[i];
                        hi = (unsigned long long)__double_as_longlong(x.sim);
                        c = x.ocol;
                    }
                    const uint32_t lo = ~c;
                    if (sel_match(hi, lo, P_hi, P_lo, p)) atomicAdd(&hist[sel_digit(hi, lo, p)], 1u);
                }
                __syncwarp();
                // lane L owns bins [8L, 8L + 8); count the bins above each lane's
                uint32_t b[8], own = 0;
#pragma unroll
                for (int t = 0; t < 8; ++t) {
                    b[t] = hist[lane * 8 + t];
                    own += b[t];
                }
                uint32_t suf = own;  // inclusive sum over lanes >= lane
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    const uint32_t v = __shfl_down_sync(0xffffffffu, suf, o);
                    if (lane + o < 32) suf += v;
                }
                uint32_t above = suf - own;
                int bin = -1;
                uint32_t bin_above = 0, bin_cnt = 0;
                if (above < need && need <= suf) {
#pragma unroll
                    for (int t = 7; t >= 0; --t) {
                        if (bin < 0 && above + b[t] >= need) {
                            bin = (int)(lane * 8 + t);
                            bin_above = above;
                            bin_cnt = b[t];
                        }
                        if (bin < 0) above += b[t];
                    }
                }
                const uint32_t who = __ffs(__ballot_sync(0xffffffffu, bin >= 0)) - 1;
                bin = __shfl_sync(0xffffffffu, bin, who);
                bin_above = __shfl_sync(0xffffffffu, bin_above, who);
                bin_cnt = __shfl_sync(0xffffffffu, bin_cnt, who);
                need -= bin_above;
                if (p < 8)
                    P_hi |= (unsigned long long)bin << (56 - 8 * p);
                else
                    P_lo |= (uint32_t)bin << (24 - 8 * (p - 8));
                if (bin_cnt == need) break;
            }
        }
        // compact the kept entries with ocol > orow to the front of the buffer
        uint32_t m = 0;
        const uint32_t cap = max_edges;
        for (uint32_t base = 0; base < cnt; base += 32) {
            const uint32_t i = base + lane;
            unsigned long long hi = 0;
            uint32_t c = 0;
            bool take = false;
            if (i < cnt) {
                if (staged) {
                    hi = key[i];
                    c = col[i];
                } else {
                    const Ent x = row[i];
                    hi = (unsigned long long)__double_as_longlong(x.sim);
                    c = x.ocol;
                }
                const uint32_t lo = ~c;
                take = c > orow && (hi > P_hi || (hi == P_hi && lo >= P_lo));
            }
            const uint32_t bal = __ballot_sync(0xffffffffu, take);
            __syncwarp();  // every lane has read its entry before any slot is rewritten
            const uint32_t q = m + __popc(bal & ((1u << lane) - 1u));
            if (take && q < cap) {
                key[q] = hi;
                col[q] = c;
            }
            m += __popc(bal);
            __syncwarp();
        }
        m = min(m, cap);
        if (m <= 64)
            sort_out<2>(key, col, m, lane, row);
        else if (m <= 128)
            sort_out<4>(key, col, m, lane, row);
        else
            sort_out<EMAX>(key, col, m, lane, row);
        if (lane == 0) out_cnt[orow] = m;
        __syncwarp();
    }
}

// Warp per original row: write its kept edges with ocol > row, in order.
// compacted: the row starts with exactly those edges (selection top-k).
// Rows (original index o) outside the sorted-position range [k0, k1) emit nothing.
__global__ void k_keep_rows(const uint32_t* __restrict__ inv, uint32_t n, uint32_t k0, uint32_t k1,
                            uint32_t* __restrict__ out_cnt) {
    const uint32_t o = blockIdx.x * blockDim.x + threadIdx.x;
    if (o >= n) return;
    const uint32_t s = inv[o];
    if (s < k0 || s >= k1) out_cnt[o] = 0;
}

__global__ void k_emit(const uint32_t* __restrict__ inv, const unsigned long long* __restrict__ rowptr,
                       const uint32_t* __restrict__ deg, const Ent* __restrict__ list,
                       const unsigned long long* __restrict__ outptr, uint32_t n, uint32_t max_edges, int compacted,
                       uint64_t* __restrict__ from, uint64_t* __restrict__ to, double* __restrict__ stnf) {
    const uint32_t lane = threadIdx.x & 31;
    for (uint32_t o = blockIdx.x * (blockDim.x / 32) + (threadIdx.x >> 5); o < n; o += gridDim.x * (blockDim.x / 32)) {
        const uint32_t s = inv[o];
        const uint32_t keep = compacted ? (uint32_t)(outptr[o + 1] - outptr[o]) : min(deg[s], max_edges);
        const Ent* row = list + rowptr[s];
        unsigned long long pos = outptr[o];
        for (uint32_t b = 0; b < keep; b += 32) {
            uint32_t i = b + lane;
            Ent x;
            bool ok = false;
            if (i < keep) {
                x = row[i];
                ok = x.ocol > o;
            }
            uint32_t bal = __ballot_sync(0xffffffffu, ok);
            if (ok) {
                unsigned long long q = pos + __popc(bal & ((1u << lane) - 1u));
                from[q] = o;
                to[q] = x.ocol;
                stnf[q] = x.sim;
            }
            pos += __popc(bal);
        }
    }
}

__global__ void k_maxprob_finish(const unsigned long long* __restrict__ maxkey, const uint32_t* __restrict__ slot_of,
                                 uint64_t m, double* __restrict__ out) {
    uint64_t b = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (b >= m) return;
    double pre = dkey_inv(maxkey[slot_of[b]]);
    // the reference seeds its running max with DBL_MIN (cuda/Cuda2.cu:287)
    const double dbl_min = 2.2250738585072014e-308;
    if (!(pre > dbl_min)) pre = dbl_min;
    out[b] = 1. - (1. / (1. + exp(pre)));
}

__global__ void k_widen(const uint32_t* __restrict__ src, uint64_t n, unsigned long long* __restrict__ dst) {
    uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (i < n) dst[i] = src[i];
    if (i == n) dst[i] = 0;
}

__global__ void k_fill_u64(unsigned long long* p, uint64_t n, unsigned long long v) {
    uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (i < n) p[i] = v;
}

}  // namespace

// ------------------------------------------------------------ host side --

int exact_graph(mdet_ctx* ctx, const GraphPrep& g, const uint2* cand, unsigned long long ncand, double L,
                Edge** edges_out, unsigned long long* nedges_out, uint32_t** deg_out, const BlkCut* blk_L,
                const unsigned long long* ncand_dev, unsigned long long** nedges_dev) {
    cudaStream_t s = ctx->stream;
    Edge* edges = (Edge*)ctx_scratch(ctx, "ex.edges", (ncand ? ncand : 1) * sizeof(Edge));
    unsigned long long* cnt = (unsigned long long*)ctx_scratch(ctx, "ex.cnt", 8);
    uint32_t* deg = (uint32_t*)ctx_scratch(ctx, "ex.deg", (uint64_t)g.n * 4);
    if (!edges || !cnt || !deg) return MDET_ERR_NOMEM;
    MDET_CUDA(ctx, cudaMemsetAsync(cnt, 0, 8, s));
    MDET_CUDA(ctx, cudaMemsetAsync(deg, 0, (uint64_t)g.n * 4, s));
    if (ncand) {
        ExactArgs p;
        memset(&p, 0, sizeof(p));
        p.cand = cand;
        p.ncand = ncand;
        p.x32 = g.x32;
        p.parts = g.parts;
        p.H = model_h_ff();
        p.L = L;
        p.Lff.hi = (float)L;
        p.Lff.lo = (float)(L - (double)p.Lff.hi);
        p.blk_L = blk_L;
        p.ncand_dev = ncand_dev;
        p.low = g.low;
        p.edges = edges;
        p.nedges = cnt;
        p.deg = deg;
        // a block takes 256 candidates per round; blocks per SM (how many
        // candidates are in flight, hence how far apart in the list the rows
        // read at one time lie) is tuned once per shape class
        const unsigned long long blocks = (ncand + 255) / 256;
        auto run = [&](int per_sm) -> int {
            MDET_CUDA(ctx, cudaMemsetAsync(cnt, 0, 8, s));
            MDET_CUDA(ctx, cudaMemsetAsync(deg, 0, (uint64_t)g.n * 4, s));
            const unsigned long long cap = (unsigned long long)ctx->num_sms * per_sm;
            ctx_timer_begin(ctx, "k_exact_graph");
            k_exact_graph<<<(unsigned)(blocks < cap ? blocks : cap), 256, 0, s>>>(p);
            ctx_timer_end(ctx, "k_exact_graph");
            MDET_LAUNCHED(ctx, "k_exact_graph");
            return MDET_OK;
        };
        if (ctx->forced_exact) {
            MDET_TRY(run(ctx->forced_exact));
        } else {
            // candidates: as many blocks per SM as fit, half that, and 2
            int fit = 0;
            MDET_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&fit, k_exact_graph, 256, 0));
            fit = fit < 2 ? 2 : fit;
            std::vector<int> cands = {fit};
            if (fit / 2 > 2) cands.push_back(fit / 2);
            if (fit > 2) cands.push_back(2);
            MDET_TRY(launch_autotune(ctx, ctx->exact_shape, tc_shape_key(false, false, ncand, g.n), cands, run));
        }
    }
    *edges_out = edges;
    *deg_out = deg;
    if (nedges_dev) {  // counts stay on the device (capturable); ncand bounds the edges
        *nedges_dev = cnt;
        *nedges_out = ncand;
        return MDET_OK;
    }
    MDET_CUDA(ctx, cudaMemcpyAsync(nedges_out, cnt, 8, cudaMemcpyDeviceToHost, s));
    MDET_CUDA(ctx, cudaStreamSynchronize(s));
    return MDET_OK;
}

int exact_maxprob(mdet_ctx* ctx, const GraphPrep& g, const uint2* cand, unsigned long long ncand,
                  const uint32_t* row_map, uint64_t m, const uint32_t* slot_of, double* d_out, bool swapped) {
    cudaStream_t s = ctx->stream;
    unsigned long long* maxkey = (unsigned long long*)ctx_scratch(ctx, "mp.maxkey", (m ? m : 1) * 8);
    if (!maxkey) return MDET_ERR_NOMEM;
    k_fill_u64<<<(unsigned)((m + 255) / 256), 256, 0, s>>>(maxkey, m, 0ull);
    MDET_LAUNCHED(ctx, "k_fill_u64");
    if (ncand) {
        ExactArgs p;
        memset(&p, 0, sizeof(p));
        p.cand = cand;
        p.ncand = ncand;
        p.row_map = row_map;
        p.swapped = swapped;
        p.x32 = g.x32;
        p.parts = g.parts;
        p.H = model_h_ff();
        p.maxkey = maxkey;
        unsigned long long blocks = (ncand + 255) / 256;
        int fit = 0;
        MDET_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&fit, k_exact_maxprob, 256, 0));
        unsigned long long cap = (unsigned long long)ctx->num_sms * (fit < 1 ? 1 : fit);
        ctx_timer_begin(ctx, "k_exact_maxprob");
    k_exact_maxprob<<<(unsigned)(blocks < cap ? blocks : cap), 256, 0, s>>>(p);
        ctx_timer_end(ctx, "k_exact_maxprob");
    MDET_LAUNCHED(ctx, "k_exact_maxprob");
    }
    k_maxprob_finish<<<(unsigned)((m + 255) / 256), 256, 0, s>>>(maxkey, slot_of, m, d_out);
    MDET_LAUNCHED(ctx, "k_maxprob_finish");
    return MDET_OK;
}

int pair_scores(mdet_ctx* ctx, const GraphPrep& g, const uint64_t* pairs, uint64_t m, double* dist, double* prob) {
    if (m == 0) return MDET_OK;
    const uint64_t blocks = std::min<uint64_t>((m + 255) / 256, (uint64_t)ctx->num_sms * 16);
    k_pair_scores<<<(unsigned)blocks, 256, 0, ctx->stream>>>(pairs, m, g.inv, g.x32, g.parts, model_h_ff(), dist, prob);
    MDET_LAUNCHED(ctx, "k_pair_scores");
    return MDET_OK;
}

int select_topk(mdet_ctx* ctx, const GraphPrep& g, const Edge* edges, unsigned long long ne, uint32_t* deg,
                uint32_t max_edges, uint64_t* n_out, const uint32_t* blk_K, const unsigned long long* ne_dev,
                uint32_t keep0, uint32_t keep1) {
    cudaStream_t s = ctx->stream;
    const uint32_t n = g.n;
    unsigned long long* rowptr = (unsigned long long*)ctx_scratch(ctx, "tk.rowptr", ((uint64_t)n + 1) * 8);
    uint32_t* cursor = (uint32_t*)ctx_scratch(ctx, "tk.cursor", (uint64_t)n * 4);
    Ent* list = (Ent*)ctx_scratch(ctx, "tk.list", (ne ? 2 * ne : 1) * sizeof(Ent));
    uint32_t* out_cnt = (uint32_t*)ctx_scratch(ctx, "tk.outcnt", (uint64_t)n * 4);
    unsigned long long* outptr = (unsigned long long*)ctx_scratch(ctx, "tk.outptr", ((uint64_t)n + 1) * 8);
    uint32_t* big = (uint32_t*)ctx_scratch(ctx, "tk.big", (uint64_t)n * 4);
    unsigned int* nbig = (unsigned int*)ctx_scratch(ctx, "tk.nbig", 8);
    if (!rowptr || !cursor || !list || !out_cnt || !outptr || !big || !nbig) return MDET_ERR_NOMEM;
    // 64-bit scans: widen the per-row counts (plus a trailing zero) first
    unsigned long long* w64 = (unsigned long long*)ctx_scratch(ctx, "tk.w64", ((uint64_t)n + 1) * 8);
    if (!w64) return MDET_ERR_NOMEM;
    size_t tb = 0;
    cub::DeviceScan::ExclusiveSum(nullptr, tb, w64, rowptr, (int)n + 1, s);
    void* tmp = ctx_scratch(ctx, "tk.cubtmp", tb);
    if (!tmp) return MDET_ERR_NOMEM;
    const unsigned wblocks = (unsigned)(((uint64_t)n + 1 + 255) / 256);
    k_widen<<<wblocks, 256, 0, s>>>(deg, n, w64);
    MDET_LAUNCHED(ctx, "k_widen");
    MDET_CUDA(ctx, cub::DeviceScan::ExclusiveSum(tmp, tb, w64, rowptr, (int)n + 1, s));
    MDET_CUDA(ctx, cudaMemsetAsync(cursor, 0, (uint64_t)n * 4, s));
    if (ne) {
        unsigned long long blocks = (ne + 255) / 256, cap = (unsigned long long)ctx->num_sms * 16;
        ctx_timer_begin(ctx, "k_scatter");
        k_scatter<<<(unsigned)(blocks < cap ? blocks : cap), 256, 0, s>>>(edges, ne, ne_dev, g.perm, rowptr, cursor,
                                                                           list);
        ctx_timer_end(ctx, "k_scatter");
        MDET_LAUNCHED(ctx, "k_scatter");
    }
    MDET_CUDA(ctx, cudaMemsetAsync(nbig, 0, 4, s));
    MDET_CUDA(ctx, cudaMemsetAsync(out_cnt, 0, (uint64_t)n * 4, s));
    if (max_edges <= 512) {
        // selection top-k, warp per row
        const unsigned blocks =
            (unsigned)std::min<uint64_t>(((uint64_t)n + kSelWarps - 1) / kSelWarps, (uint64_t)ctx->num_sms * 32);
        ctx_timer_begin(ctx, "k_topk_sel");
        if (max_edges <= 256)
            k_topk_sel<8><<<blocks, kSelWarps * 32, 0, s>>>(rowptr, deg, g.perm, n, max_edges, blk_K, list, out_cnt);
        else
            k_topk_sel<16><<<blocks, kSelWarps * 32, 0, s>>>(rowptr, deg, g.perm, n, max_edges, blk_K, list, out_cnt);
        ctx_timer_end(ctx, "k_topk_sel");
        MDET_LAUNCHED(ctx, "k_topk_sel");
    } else {
        if (blk_K) return ctx_fail(ctx, MDET_ERR_INVALID, "per-row max_edges needs max_edges <= 512");
        size_t dyn = (size_t)kTopkWarps * kWarpCap * sizeof(Ent);
        static bool set[64] = {false};
        if (!set[ctx->device & 63]) {
            MDET_CUDA(ctx, cudaFuncSetAttribute(k_topk_warp, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dyn));
            MDET_CUDA(ctx, cudaFuncSetAttribute(k_topk_big, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                (int)(kBigCap * sizeof(Ent))));
            set[ctx->device & 63] = true;
        }
        unsigned blocks = (unsigned)std::min<uint64_t>(((uint64_t)n + kTopkWarps - 1) / kTopkWarps,
                                                       (uint64_t)ctx->num_sms * 32);
        k_topk_warp<<<blocks, kTopkWarps * 32, dyn, s>>>(rowptr, deg, g.perm, n, max_edges, list, out_cnt, big, nbig);
        MDET_LAUNCHED(ctx, "k_topk_warp");
        k_topk_big<<<ctx->num_sms, 1024, kBigCap * sizeof(Ent), s>>>(big, nbig, rowptr, deg, g.perm, max_edges, list,
                                                                    out_cnt);
        MDET_LAUNCHED(ctx, "k_topk_big");
    }
    if (keep0 > 0 || keep1 < n) {
        if (max_edges > 512) return ctx_fail(ctx, MDET_ERR_INVALID, "row shards need max_edges <= 512");
        k_keep_rows<<<wblocks, 256, 0, s>>>(g.inv, n, keep0, keep1, out_cnt);
        MDET_LAUNCHED(ctx, "k_keep_rows");
    }
    k_widen<<<wblocks, 256, 0, s>>>(out_cnt, n, w64);
    MDET_LAUNCHED(ctx, "k_widen");
    MDET_CUDA(ctx, cub::DeviceScan::ExclusiveSum(tmp, tb, w64, outptr, (int)n + 1, s));
    if (ne_dev) {  // capturable: the total stays on the device (outptr[n])
        *n_out = 0;
        return MDET_OK;
    }
    unsigned long long total = 0;
    MDET_CUDA(ctx, cudaMemcpyAsync(&total, outptr + n, 8, cudaMemcpyDeviceToHost, s));
    MDET_CUDA(ctx, cudaStreamSynchronize(s));
    *n_out = total;
    return MDET_OK;
}

int emit_topk(mdet_ctx* ctx, const GraphPrep& g, uint32_t max_edges, uint64_t* d_from, uint64_t* d_to,
              double* d_stnf, uint64_t total) {
    cudaStream_t s = ctx->stream;
    const uint32_t n = g.n;
    const unsigned long long* rowptr = (const unsigned long long*)ctx->bufs["tk.rowptr"].p;
    const unsigned long long* outptr = (const unsigned long long*)ctx->bufs["tk.outptr"].p;
    const Ent* list = (const Ent*)ctx->bufs["tk.list"].p;
    const uint32_t* deg = (const uint32_t*)ctx->bufs["ex.deg"].p;
    if (total) {
        unsigned blocks = (unsigned)std::min<uint64_t>(((uint64_t)n + 7) / 8, (uint64_t)ctx->num_sms * 32);
        k_emit<<<blocks, 256, 0, s>>>(g.inv, rowptr, deg, list, outptr, n, max_edges, max_edges <= 512 ? 1 : 0,
                                      d_from, d_to, d_stnf);
        MDET_LAUNCHED(ctx, "k_emit");
    }
    return MDET_OK;
}
