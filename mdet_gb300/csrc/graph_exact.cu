// graph_exact.cu -- exact scoring of filtered pairs and per-contig top-k.
//
// Every pair that passed a distance filter is scored again from the FP32
// TNF rows: the reference's terms float((a_k - b_k)^2) (cuda/Cuda2.cu:194-196)
// summed with compensated FP32 arithmetic, sqrt in FP64, then the
// MetaBAT2 logistic model in FP64 (cuda/Cuda2.cu:199-240) from per-contig
// parts F(x), G(y) and the pair term H(x*y).  A pair is an edge when its
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
    const float* x32;
    const double* ls;
    const ModelParts* parts;
    ModelH H;
    double L;
    // graph outputs
    Edge* edges;
    unsigned long long* nedges;
    uint32_t* deg;
    // maxprob output
    unsigned long long* maxkey;
};

__global__ void __launch_bounds__(256) k_exact_graph(ExactArgs p) {
    const bool model2 = p.L < kLn9;
    const uint32_t lane = threadIdx.x & 31;
    for (unsigned long long base = (unsigned long long)blockIdx.x * blockDim.x; base < p.ncand;
         base += (unsigned long long)gridDim.x * blockDim.x) {
        unsigned long long idx = base + threadIdx.x;
        bool edge = false;
        uint32_t si = 0, sj = 0;
        double sim = 0;
        if (idx < p.ncand) {
            uint2 c = p.cand[idx];
            si = c.x;
            sj = c.y;
            double d = exact_dist(p.x32 + (uint64_t)si * MDET_NTNF, p.x32 + (uint64_t)sj * MDET_NTNF);
            ModelParts pi = p.parts[si], pj = p.parts[sj];
            double pre = pre_prob(pi, pj, p.ls[si], p.ls[sj], d, p.H, model2);
            if (pre > p.L) {
                edge = true;
                sim = 1. - 1. / (1. + exp(pre));
            }
        }
        uint32_t bal = __ballot_sync(0xffffffffu, edge);
        if (bal) {
            unsigned long long wb = 0;
            int leader = __ffs(bal) - 1;
            if (lane == (uint32_t)leader) wb = atomicAdd(p.nedges, (unsigned long long)__popc(bal));
            wb = __shfl_sync(0xffffffffu, wb, leader);
            if (edge) {
                Edge e;
                e.i = si;
                e.j = sj;
                e.sim = sim;
                p.edges[wb + __popc(bal & ((1u << lane) - 1u))] = e;
                atomicAdd(&p.deg[si], 1u);
                atomicAdd(&p.deg[sj], 1u);
            }
        }
    }
}

__global__ void __launch_bounds__(256) k_exact_maxprob(ExactArgs p) {
    for (unsigned long long idx = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x; idx < p.ncand;
         idx += (unsigned long long)gridDim.x * blockDim.x) {
        uint2 c = p.cand[idx];
        uint32_t si = p.row_map[c.x], sj = c.y;
        if (si == sj) continue;  // the sampled contig itself
        double d = exact_dist(p.x32 + (uint64_t)si * MDET_NTNF, p.x32 + (uint64_t)sj * MDET_NTNF);
        ModelParts pi = p.parts[si], pj = p.parts[sj];
        double pre = pre_prob(pi, pj, p.ls[si], p.ls[sj], d, p.H, true);
        atomicMax(&p.maxkey[c.x], dkey(pre));
    }
}

__global__ void k_scatter(const Edge* __restrict__ edges, unsigned long long ne, const uint32_t* __restrict__ perm,
                          const unsigned long long* __restrict__ rowptr, uint32_t* __restrict__ cursor,
                          Ent* __restrict__ list) {
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

// ---- register top-k: warp per contig, entries held in registers ----------
// Entry i of a chunk of C = 32*E lives in lane i % 32, slot i / 32.  A
// bitonic network sorts a chunk best-first (exchanges across lanes by
// shuffles, within a lane by register swaps); a longer row is consumed chunk
// by chunk, each sorted chunk merged into the running best C (elementwise
// better of best[i] and chunk[C-1-i] is bitonic, then a bitonic merge), so a
// row of any length needs C >= max_edges registers' worth of entries only.

__device__ __forceinline__ bool kv_less(double s1, uint32_t c1, double s2, uint32_t c2) {
    return s1 > s2 || (s1 == s2 && c1 < c2);
}

// In-lane compare-exchange of slots e and e | JE (stride >= 32 entries).
template <int E, int JE>
__device__ __forceinline__ void stage_in_lane(double (&s)[E], uint32_t (&c)[E], uint32_t lane, uint32_t k,
                                              bool all_up) {
#pragma unroll
    for (int e = 0; e < E; ++e) {
        if ((e & JE) == 0) {
            const int e2 = e | JE;
            const bool up = all_up || ((((uint32_t)e * 32u + lane) & k) == 0);
            const bool sw = up ? kv_less(s[e2], c[e2], s[e], c[e]) : kv_less(s[e], c[e], s[e2], c[e2]);
            const double s1 = sw ? s[e2] : s[e], s2 = sw ? s[e] : s[e2];
            const uint32_t c1 = sw ? c[e2] : c[e], c2 = sw ? c[e] : c[e2];
            s[e] = s1;
            s[e2] = s2;
            c[e] = c1;
            c[e2] = c2;
        }
    }
}

template <int E>
__device__ __forceinline__ void bitonic_stage(double (&s)[E], uint32_t (&c)[E], uint32_t lane, uint32_t k, uint32_t j,
                                           bool all_up) {
    if (j >= 32) {
        const uint32_t je = j >> 5;
        if (je == 1) stage_in_lane<E, 1>(s, c, lane, k, all_up);
        if (E >= 4 && je == 2) stage_in_lane<E, (E >= 4 ? 2 : 1)>(s, c, lane, k, all_up);
        if (E >= 8 && je == 4) stage_in_lane<E, (E >= 8 ? 4 : 1)>(s, c, lane, k, all_up);
        if (E >= 16 && je == 8) stage_in_lane<E, (E >= 16 ? 8 : 1)>(s, c, lane, k, all_up);
    } else {
        const bool lower = (lane & j) == 0;
#pragma unroll
        for (int e = 0; e < E; ++e) {
            const bool up = all_up || ((((uint32_t)e * 32u + lane) & k) == 0);
            const double os = __shfl_xor_sync(0xffffffffu, s[e], (int)j);
            const uint32_t oc = __shfl_xor_sync(0xffffffffu, c[e], (int)j);
            const bool take = (lower == up) ? kv_less(os, oc, s[e], c[e]) : kv_less(s[e], c[e], os, oc);
            s[e] = take ? os : s[e];
            c[e] = take ? oc : c[e];
        }
    }
}

template <int E>
__device__ __forceinline__ void bitonic_sort(double (&s)[E], uint32_t (&c)[E], uint32_t lane) {
#pragma unroll 1
    for (uint32_t k = 2; k <= 32u * E; k <<= 1)
#pragma unroll 1
        for (uint32_t j = k >> 1; j > 0; j >>= 1) bitonic_stage<E>(s, c, lane, k, j, false);
}

template <int E>
__device__ __forceinline__ void load_chunk(const Ent* __restrict__ row, uint32_t base, uint32_t cnt, uint32_t lane,
                                           double (&s)[E], uint32_t (&c)[E]) {
#pragma unroll
    for (int e = 0; e < E; ++e) {
        const uint32_t i = base + (uint32_t)e * 32u + lane;
        if (i < cnt) {
            const Ent x = row[i];
            s[e] = x.sim;
            c[e] = x.ocol;
        } else {
            s[e] = -1.0;
            c[e] = 0xFFFFFFFFu;
        }
    }
}

// Sorts the row's best min(cnt, keep) entries into row[0..) and returns how
// many of them have a column above orow (lane 0 holds the total).
template <int E>
__device__ __forceinline__ uint32_t topk_row(Ent* __restrict__ row, uint32_t cnt, uint32_t keep, uint32_t orow,
                                             uint32_t lane) {
    double bs[E], cs[E];
    uint32_t bc[E], cc[E];
    load_chunk<E>(row, 0, cnt, lane, bs, bc);
    bitonic_sort<E>(bs, bc, lane);
    for (uint32_t base = 32u * E; base < cnt; base += 32u * E) {
        load_chunk<E>(row, base, cnt, lane, cs, cc);
        bitonic_sort<E>(cs, cc, lane);
#pragma unroll
        for (int e = 0; e < E; ++e) {
            const double os = __shfl_sync(0xffffffffu, cs[E - 1 - e], 31 - lane);
            const uint32_t oc = __shfl_sync(0xffffffffu, cc[E - 1 - e], 31 - lane);
            if (kv_less(os, oc, bs[e], bc[e])) {
                bs[e] = os;
                bc[e] = oc;
            }
        }
#pragma unroll 1
        for (uint32_t j = 16u * E; j > 0; j >>= 1) bitonic_stage<E>(bs, bc, lane, 0, j, true);
    }
    __syncwarp();
    uint32_t n_up = 0;
#pragma unroll
    for (int e = 0; e < E; ++e) {
        const uint32_t i = (uint32_t)e * 32u + lane;
        if (i < keep) {
            Ent x;
            x.sim = bs[e];
            x.ocol = bc[e];
            x.pad = 0;
            row[i] = x;
            n_up += bc[e] > orow;
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) n_up += __shfl_xor_sync(0xffffffffu, n_up, o);
    return n_up;
}

template <int EMAX>
__global__ void __launch_bounds__(256) k_topk_reg(const unsigned long long* __restrict__ rowptr,
                                                  const uint32_t* __restrict__ deg, const uint32_t* __restrict__ perm,
                                                  uint32_t n, uint32_t max_edges, Ent* __restrict__ list,
                                                  uint32_t* __restrict__ out_cnt) {
    const uint32_t lane = threadIdx.x & 31;
    for (uint32_t s = blockIdx.x * (blockDim.x / 32) + (threadIdx.x >> 5); s < n; s += gridDim.x * (blockDim.x / 32)) {
        const uint32_t cnt = deg[s], orow = perm[s];
        const uint32_t keep = cnt < max_edges ? cnt : max_edges;
        Ent* row = list + rowptr[s];
        uint32_t c;
        if (cnt <= 128)
            c = topk_row<4>(row, cnt, keep, orow, lane);
        else
            c = topk_row<EMAX>(row, cnt, keep, orow, lane);
        if (lane == 0) out_cnt[orow] = c;
    }
}

// Warp per original row: write its kept edges with ocol > row, in order.
__global__ void k_emit(const uint32_t* __restrict__ inv, const unsigned long long* __restrict__ rowptr,
                       const uint32_t* __restrict__ deg, const Ent* __restrict__ list,
                       const unsigned long long* __restrict__ outptr, uint32_t n, uint32_t max_edges,
                       uint64_t* __restrict__ from, uint64_t* __restrict__ to, double* __restrict__ stnf) {
    const uint32_t lane = threadIdx.x & 31;
    for (uint32_t o = blockIdx.x * (blockDim.x / 32) + (threadIdx.x >> 5); o < n; o += gridDim.x * (blockDim.x / 32)) {
        const uint32_t s = inv[o];
        const uint32_t keep = min(deg[s], max_edges);
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
                Edge** edges_out, unsigned long long* nedges_out, uint32_t** deg_out) {
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
        p.ls = g.ls;
        p.parts = g.parts;
        p.H = model_h();
        p.L = L;
        p.edges = edges;
        p.nedges = cnt;
        p.deg = deg;
        unsigned long long blocks = (ncand + 255) / 256;
        unsigned long long cap = (unsigned long long)ctx->num_sms * 16;
        ctx_timer_begin(ctx, "k_exact_graph");
    k_exact_graph<<<(unsigned)(blocks < cap ? blocks : cap), 256, 0, s>>>(p);
        ctx_timer_end(ctx, "k_exact_graph");
    MDET_LAUNCHED(ctx, "k_exact_graph");
    }
    MDET_CUDA(ctx, cudaMemcpyAsync(nedges_out, cnt, 8, cudaMemcpyDeviceToHost, s));
    MDET_CUDA(ctx, cudaStreamSynchronize(s));
    *edges_out = edges;
    *deg_out = deg;
    return MDET_OK;
}

int exact_maxprob(mdet_ctx* ctx, const GraphPrep& g, const uint2* cand, unsigned long long ncand,
                  const uint32_t* row_map, uint64_t m, const uint32_t* slot_of, double* d_out) {
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
        p.x32 = g.x32;
        p.ls = g.ls;
        p.parts = g.parts;
        p.H = model_h();
        p.maxkey = maxkey;
        unsigned long long blocks = (ncand + 255) / 256;
        unsigned long long cap = (unsigned long long)ctx->num_sms * 16;
        ctx_timer_begin(ctx, "k_exact_maxprob");
    k_exact_maxprob<<<(unsigned)(blocks < cap ? blocks : cap), 256, 0, s>>>(p);
        ctx_timer_end(ctx, "k_exact_maxprob");
    MDET_LAUNCHED(ctx, "k_exact_maxprob");
    }
    k_maxprob_finish<<<(unsigned)((m + 255) / 256), 256, 0, s>>>(maxkey, slot_of, m, d_out);
    MDET_LAUNCHED(ctx, "k_maxprob_finish");
    return MDET_OK;
}

int select_topk(mdet_ctx* ctx, const GraphPrep& g, const Edge* edges, unsigned long long ne, uint32_t* deg,
                uint32_t max_edges, uint64_t* n_out) {
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
        k_scatter<<<(unsigned)(blocks < cap ? blocks : cap), 256, 0, s>>>(edges, ne, g.perm, rowptr, cursor, list);
        ctx_timer_end(ctx, "k_scatter");
        MDET_LAUNCHED(ctx, "k_scatter");
    }
    MDET_CUDA(ctx, cudaMemsetAsync(nbig, 0, 4, s));
    MDET_CUDA(ctx, cudaMemsetAsync(out_cnt, 0, (uint64_t)n * 4, s));
    if (max_edges <= 512) {
        // register top-k (chunk of 256 or 512 entries per warp)
        const unsigned blocks = (unsigned)std::min<uint64_t>(((uint64_t)n + 7) / 8, (uint64_t)ctx->num_sms * 16);
        ctx_timer_begin(ctx, "k_topk_reg");
        if (max_edges <= 256)
            k_topk_reg<8><<<blocks, 256, 0, s>>>(rowptr, deg, g.perm, n, max_edges, list, out_cnt);
        else
            k_topk_reg<16><<<blocks, 256, 0, s>>>(rowptr, deg, g.perm, n, max_edges, list, out_cnt);
        ctx_timer_end(ctx, "k_topk_reg");
        MDET_LAUNCHED(ctx, "k_topk_reg");
    } else {
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
    k_widen<<<wblocks, 256, 0, s>>>(out_cnt, n, w64);
    MDET_LAUNCHED(ctx, "k_widen");
    MDET_CUDA(ctx, cub::DeviceScan::ExclusiveSum(tmp, tb, w64, outptr, (int)n + 1, s));
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
        k_emit<<<blocks, 256, 0, s>>>(g.inv, rowptr, deg, list, outptr, n, max_edges, d_from, d_to, d_stnf);
        MDET_LAUNCHED(ctx, "k_emit");
    }
    return MDET_OK;
}
