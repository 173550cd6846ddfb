// graph.cu -- C ABI of the pairwise stage: TNF graph, max-probability
// sample and the pTNF search, orchestrating prep -> filter -> exact ->
// per-contig top-k on the context's stream.
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <numeric>
#include <vector>

#include <cub/cub.cuh>

#include "graph.cuh"

namespace {

struct PhaseTimer {
    cudaEvent_t ev[6];
    int n = 0;
    cudaStream_t s;
    explicit PhaseTimer(cudaStream_t st) : s(st) {
        for (auto& e : ev) cudaEventCreate(&e);
    }
    ~PhaseTimer() {
        for (auto& e : ev) cudaEventDestroy(e);
    }
    void mark() {
        if (n < 6) cudaEventRecord(ev[n++], s);
    }
    double ms(int a, int b) {
        if (b >= n) return 0;
        float t = 0;
        cudaEventSynchronize(ev[b]);
        cudaEventElapsedTime(&t, ev[a], ev[b]);
        return t;
    }
};

__global__ void k_sample_sort_keys(const uint64_t* __restrict__ contigs, const uint32_t* __restrict__ inv, uint64_t m,
                                   uint32_t* __restrict__ keys, uint32_t* __restrict__ vals) {
    uint64_t b = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (b >= m) return;
    keys[b] = inv[contigs[b]];
    vals[b] = (uint32_t)b;
}

__global__ void k_sample_gather(const uint32_t* __restrict__ row_map, const uint32_t* __restrict__ order, uint64_t m,
                                const float* __restrict__ x32, const double* __restrict__ ls,
                                float* __restrict__ a32, double* __restrict__ als, uint32_t* __restrict__ slot_of) {
    uint64_t r = blockIdx.x;
    if (r >= m) return;
    uint32_t sp = row_map[r];
    for (int k = threadIdx.x; k < MDET_NTNF; k += blockDim.x) a32[r * MDET_NTNF + k] = x32[(uint64_t)sp * MDET_NTNF + k];
    if (threadIdx.x == 0) {
        als[r] = ls[sp];
        slot_of[order[r]] = (uint32_t)r;
    }
}

__global__ void k_sample_gather_bf16(const uint32_t* __restrict__ row_map, uint64_t m, uint64_t mpad,
                                     const uint16_t* __restrict__ xb, const float* __restrict__ nsq,
                                     uint16_t* __restrict__ ab, float* __restrict__ ansq) {
    uint64_t r = blockIdx.x;
    if (r >= mpad) return;
    if (r < m) {
        uint32_t sp = row_map[r];
        for (int k = threadIdx.x; k < MDET_KPAD; k += blockDim.x) ab[r * MDET_KPAD + k] = xb[(uint64_t)sp * MDET_KPAD + k];
        if (threadIdx.x == 0) ansq[r] = nsq[sp];
    } else {
        // padding row of the A role: zeros with the two unit columns
        for (int k = threadIdx.x; k < MDET_KPAD; k += blockDim.x)
            ab[r * MDET_KPAD + k] = (k == MDET_NTNF || k == MDET_NTNF + 1) ? 0x3F80 : 0;
        if (threadIdx.x == 0) ansq[r] = __int_as_float(0x7f800000);
    }
}

// The sample's rows in the B role: row r = xb row row_map[r]; padding rows
// carry -inf in the column-term slot so that no pair with them passes.
__global__ void k_sample_gather_b(const uint32_t* __restrict__ row_map, uint64_t m, uint64_t mpad,
                                  const uint16_t* __restrict__ xb, uint16_t* __restrict__ sb) {
    const uint64_t r = blockIdx.x * (uint64_t)(blockDim.x / 32) + (threadIdx.x >> 5);
    const uint32_t lane = threadIdx.x & 31;
    if (r >= mpad) return;
    if (r < m) {
        const uint32_t* src = reinterpret_cast<const uint32_t*>(xb + (uint64_t)row_map[r] * MDET_KPAD);
        uint32_t* dst = reinterpret_cast<uint32_t*>(sb + r * MDET_KPAD);
        for (int k = lane; k < MDET_KPAD / 2; k += 32) dst[k] = src[k];
    } else {
        for (int k = lane; k < MDET_KPAD; k += 32) sb[r * MDET_KPAD + k] = k == MDET_NTNF ? 0xFF80 : 0;
    }
}

// per-128 block metadata of the gathered sample (log-size range, and for
// BF16 rows the max rounding error / norm of the gathered rows)
// Metadata of the sample's blocks of MDET_BLK rows, one warp per block: lane
// l takes rows l, l + 32, ... of the block (the gathers overlap instead of
// running one after another).  NaN is the identity of fmin/fmax here, so the
// result is the same as a walk over the rows in order.
__global__ void k_sample_meta(const uint32_t* __restrict__ row_map, uint64_t m, const double* __restrict__ ls,
                              const BlockMeta* __restrict__ src_meta, uint64_t nblk, BlockMeta* __restrict__ out) {
    const uint64_t b = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
    const uint32_t lane = threadIdx.x & 31;
    if (b >= nblk) return;  // warp-uniform
    const uint64_t r0 = b * MDET_BLK, r1 = min(m, r0 + MDET_BLK);
    BlockMeta o;
    o.emax = o.nmax = 0.f;
    if (r0 < m) {
        double lo = __longlong_as_double(0x7ff8000000000000ll), hi = lo;
        float e = 0.f, nm = 0.f;
        for (uint64_t r = r0 + lane; r < r1; r += 32) {
            const uint32_t row = row_map[r];
            const double v = ls[row];
            lo = fmin(lo, v);
            hi = fmax(hi, v);
            const BlockMeta& sm = src_meta[row / MDET_BLK];
            e = fmaxf(e, sm.emax);
            nm = fmaxf(nm, sm.nmax);
        }
#pragma unroll
        for (int d = 16; d; d >>= 1) {
            lo = fmin(lo, __shfl_xor_sync(0xffffffffu, lo, d));
            hi = fmax(hi, __shfl_xor_sync(0xffffffffu, hi, d));
            e = fmaxf(e, __shfl_xor_sync(0xffffffffu, e, d));
            nm = fmaxf(nm, __shfl_xor_sync(0xffffffffu, nm, d));
        }
        o.lo = __double2float_rd(lo);
        o.hi = __double2float_ru(hi);
        o.emax = e;
        o.nmax = nm;
    } else {
        o.lo = o.hi = __double2float_rd(ls[row_map[m - 1]]);
    }
    if (lane == 0) out[b] = o;
}

}  // namespace

double logit(double cutoff) { return log((1.0 / (1. - cutoff)) - 1.0); }

uint64_t tc_shape_key(bool rect, bool list, uint64_t na, uint64_t nb) {
    auto lg = [](uint64_t v) {
        uint64_t b = 0;
        while (v > 1) {
            v >>= 1;
            ++b;
        }
        return b;
    };
    return (rect ? 1ull : 0ull) | (list ? 2ull : 0ull) | (lg(na) << 2) | (lg(nb) << 10);
}

int launch_autotune(mdet_ctx* ctx, std::map<uint64_t, int>& table, uint64_t key, const std::vector<int>& values,
                    const std::function<int(int)>& run) {
    auto it = table.find(key);
    if (it != table.end()) return run(it->second);
    if (!ctx->autotune || values.size() < 2) return run(values[0]);
    std::vector<cudaEvent_t> ev(values.size() + 1);
    for (auto& e : ev) cudaEventCreate(&e);
    int rc = MDET_OK;
    cudaEventRecord(ev[0], ctx->stream);
    for (size_t k = 0; k < values.size() && rc == MDET_OK; ++k) {
        rc = run(values[k]);
        cudaEventRecord(ev[k + 1], ctx->stream);
    }
    if (rc == MDET_OK) {
        cudaEventSynchronize(ev.back());
        float best = 0;
        int pick = values[0];
        for (size_t k = 0; k < values.size(); ++k) {
            float t = 0;
            cudaEventElapsedTime(&t, ev[k], ev[k + 1]);
            if (k == 0 || t < best) {
                best = t;
                pick = values[k];
            }
        }
        table[key] = pick;
    }
    for (auto& e : ev) cudaEventDestroy(e);
    return rc;
}

int tc_autotune(mdet_ctx* ctx, uint64_t key, const std::function<int(int)>& run, bool list) {
    if (ctx->forced_shape) {
        const int f = ctx->forced_shape;
        const int w = f == 128128 ? 128 : (f == 256128 && !list ? kShapeTall : 256);
        return run(w);
    }
    if (list) return launch_autotune(ctx, ctx->tc_shape, key, {256, 128}, run);
    return launch_autotune(ctx, ctx->tc_shape, key, {256, 128, kShapeTall}, run);
}

int run_filter(mdet_ctx* ctx, int mode, const GraphPrep& g, bool rect, const float* a32, const uint16_t* ab,
               const float* ansq, uint32_t na, const BlockMeta* ameta, const BlockMeta* ameta32,
               const DstarTable& tbl, const char* tag, uint2** cand_out, unsigned long long* ncand_out,
               const uint32_t* tiles, uint64_t nlist, const uint8_t* row_tbl, uint64_t tbl_stride, int bn,
               unsigned long long fixed_cap, unsigned long long** cnt_dev, const unsigned long long* rowoff,
               const BSide* bside) {
    cudaStream_t s = ctx->stream;
    if (bside && (mode == MDET_MODE_PLAIN || fixed_cap || tiles))
        return ctx_fail(ctx, MDET_ERR_INVALID, "a B-role subset needs a tensor-core form without a tile list");
    const bool tf32 = mode == MDET_MODE_TF32;
    if (tf32 && (rect || bside || g.tck != kTcTf32))
        return ctx_fail(ctx, MDET_ERR_INVALID, "the TF32 filter runs over a TF32 preparation, all pairs");
    unsigned long long* cnt = (unsigned long long*)ctx_scratch(ctx, "flt.cnt", 8);
    if (!cnt) return MDET_ERR_NOMEM;
    if (fixed_cap) {
        // one pass into a buffer of fixed_cap pairs; the count stays on the
        // device (pairs beyond the capacity are dropped and only counted)
        uint2* cand = (uint2*)ctx_scratch(ctx, (std::string(tag) + ".cand").c_str(), fixed_cap * sizeof(uint2));
        if (!cand) return MDET_ERR_NOMEM;
        MDET_CUDA(ctx, cudaMemsetAsync(cnt, 0, 8, s));
        CandBuf out{cand, cnt, fixed_cap};
        if (mode == MDET_MODE_PLAIN) {
            MDET_TRY(filter_simt(ctx, rect ? a32 : g.x32, rect ? na : g.n, rect ? ameta32 : g.meta32, g.x32, g.n,
                                 g.meta32, !rect, tbl, out, tiles, nlist, row_tbl, tbl_stride));
        } else if (tf32) {
            MDET_TRY(filter_tc(ctx, g.ta, g.nsq, g.n, g.meta, g.tb, g.n, g.meta, true, tbl, out, tiles, nlist, row_tbl,
                               tbl_stride, kShapeTf32, rowoff));
        } else {
            MDET_TRY(filter_tc(ctx, rect ? ab : g.xa, rect ? ansq : g.nsq, rect ? na : g.n, rect ? ameta : g.meta, g.xb,
                               g.n, g.meta, !rect, tbl, out, tiles, nlist, row_tbl, tbl_stride, bn ? bn : 256, rowoff));
        }
        *cand_out = cand;
        *ncand_out = fixed_cap;
        if (cnt_dev) *cnt_dev = cnt;
        return MDET_OK;
    }
    // remembered capacity (bytes of the candidate buffer) from earlier calls
    size_t guess = ((size_t)256 * (bside ? bside->nb : (rect ? na : g.n)) + (1u << 20)) * sizeof(uint2);
    DevBuf& cb = ctx->bufs[std::string(tag) + ".cand"];
    if (cb.cap > guess) guess = cb.cap;
    for (int attempt = 0; attempt < 3; ++attempt) {
        uint2* cand = (uint2*)ctx_scratch(ctx, (std::string(tag) + ".cand").c_str(), guess);
        if (!cand) return MDET_ERR_NOMEM;
        unsigned long long cap = ctx->bufs[std::string(tag) + ".cand"].cap / sizeof(uint2);
        CandBuf out{cand, cnt, cap};
        auto run = [&](int w) -> int {
            MDET_CUDA(ctx, cudaMemsetAsync(cnt, 0, 8, s));
            if (mode == MDET_MODE_PLAIN) {
                const float* A = rect ? a32 : g.x32;
                MDET_TRY(filter_simt(ctx, A, rect ? na : g.n, rect ? ameta32 : g.meta32, g.x32, g.n, g.meta32, !rect,
                                     tbl, out, tiles, nlist, row_tbl, tbl_stride));
                ctx->last_tile_n = 128128;
            } else if (tf32) {
                MDET_TRY(filter_tc(ctx, g.ta, g.nsq, g.n, g.meta, g.tb, g.n, g.meta, true, tbl, out, tiles, nlist,
                                   row_tbl, tbl_stride, kShapeTf32, rowoff));
                ctx->last_tile_n = 128128;
            } else if (bside) {  // all rows (A role) against a B-role subset
                MDET_TRY(filter_tc(ctx, g.xa, g.nsq, g.n, g.meta, bside->xb, bside->nb, bside->meta, false, tbl, out,
                                   nullptr, 0, nullptr, 0, w, nullptr));
            } else {
                const uint16_t* A = rect ? ab : g.xa;
                const float* An = rect ? ansq : g.nsq;
                MDET_TRY(filter_tc(ctx, A, An, rect ? na : g.n, rect ? ameta : g.meta, g.xb, g.n, g.meta, !rect, tbl,
                                   out, tiles, nlist, row_tbl, tbl_stride, w, rowoff));
                ctx->last_tile_n = w == kShapeTall ? 256128 : 128 * 1000 + w;
            }
            return MDET_OK;
        };
        if (mode == MDET_MODE_PLAIN || tf32 || bn != 0 || tiles)
            MDET_TRY(run(bn ? bn : 256));
        else
            MDET_TRY(tc_autotune(ctx, bside ? tc_shape_key(true, false, g.n, bside->nb)
                                            : tc_shape_key(rect, false, rect ? na : g.n, g.n),
                                 run));
        unsigned long long found = 0;
        MDET_CUDA(ctx, cudaMemcpyAsync(&found, cnt, 8, cudaMemcpyDeviceToHost, s));
        MDET_CUDA(ctx, cudaStreamSynchronize(s));
        if (found <= cap) {
            *cand_out = cand;
            *ncand_out = found;
            return MDET_OK;
        }
        guess = (size_t)(found + found / 8 + 1024) * sizeof(uint2);
    }
    return ctx_fail(ctx, MDET_ERR_NOMEM, "candidate buffer kept overflowing");
}

int check_mode(mdet_ctx* ctx, int mode) {
    if (mode == MDET_MODE_PLAIN) return MDET_OK;
    if (mode == MDET_MODE_BF16 || mode == MDET_MODE_TF32) {
        if (ctx->cc_major != 10 || ctx->cc_minor != 3)
            return ctx_fail(ctx, MDET_ERR_UNSUPPORTED, "tensor-core forms need an sm_103 device (have sm_%d%d)",
                            ctx->cc_major, ctx->cc_minor);
        return MDET_OK;
    }
    if (mode == MDET_MODE_LEARNED) {
        if (ctx->cc_major != 10 || ctx->cc_minor != 3)
            return ctx_fail(ctx, MDET_ERR_UNSUPPORTED, "the learned form needs an sm_103 device");
        if (!ctx->mlp) return ctx_fail(ctx, MDET_ERR_INVALID, "no network set (mdet_ctx_set_learned)");
        return MDET_OK;
    }
    return ctx_fail(ctx, MDET_ERR_UNSUPPORTED, "mode %d not available", mode);
}

int check_flag(mdet_ctx* ctx) {
    int h = 0;
    MDET_CUDA(ctx, cudaMemcpyAsync(&h, ctx->d_flag, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    MDET_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    if (h) {
        cudaMemsetAsync(ctx->d_flag, 0, sizeof(int), ctx->stream);
        return ctx_fail(ctx, MDET_ERR_TIMEOUT, "a bounded device wait ran out (flag %d)", h);
    }
    return MDET_OK;
}

int gather_rows_bf16(mdet_ctx* ctx, const GraphPrep& g, const uint32_t* row_map, uint64_t m, const char* tag,
                     RowSet* out) {
    cudaStream_t s = ctx->stream;
    const std::string t(tag);
    const uint64_t mpad = (m + 255) / 256 * 256, nblk = mpad / MDET_BLK;
    out->ab = (uint16_t*)ctx_scratch(ctx, (t + ".ab").c_str(), mpad * MDET_KPAD * 2);
    out->ansq = (float*)ctx_scratch(ctx, (t + ".ansq").c_str(), mpad * 4);
    out->meta = (BlockMeta*)ctx_scratch(ctx, (t + ".meta").c_str(), nblk * sizeof(BlockMeta));
    if (!out->ab || !out->ansq || !out->meta) return MDET_ERR_NOMEM;
    if (m == 0) return MDET_OK;
    k_sample_gather_bf16<<<(unsigned)mpad, 64, 0, s>>>(row_map, m, mpad, g.xa, g.nsq, out->ab, out->ansq);
    MDET_LAUNCHED(ctx, "k_sample_gather_bf16");
    k_sample_meta<<<(unsigned)((nblk * 32 + 127) / 128), 128, 0, s>>>(row_map, m, g.ls, g.meta, nblk, out->meta);
    MDET_LAUNCHED(ctx, "k_sample_meta");
    return MDET_OK;
}

int graph_candidates(mdet_ctx* ctx, const GraphPrep& g, double cutoff, int mode, uint2** cand, uint64_t* ncand) {
    DstarTable tbl;
    MDET_TRY(build_dstar_table(ctx, g.ls, g.n, logit(cutoff), &tbl));
    unsigned long long nc = 0;
    MDET_TRY(run_filter(ctx, mode, g, false, nullptr, nullptr, nullptr, 0, nullptr, nullptr, tbl, "g", cand, &nc));
    *ncand = nc;
    return MDET_OK;
}

int graph_core(mdet_ctx* ctx, const float* d_tnf, const double* d_ls, uint64_t n, double cutoff, uint32_t max_edges,
               int mode, mdet_graph_stats* st, GraphPrep& g, uint64_t* total) {
    if (mode == MDET_MODE_LEARNED) return graph_learned(ctx, d_tnf, d_ls, n, cutoff, max_edges, st, g, total);
    PhaseTimer tm(ctx->stream);
    tm.mark();
    MDET_TRY(prep_sorted(ctx, d_tnf, d_ls, n, tc_kind(mode), &g));
    MDET_TRY(abd_gate(ctx, g));
    const double L = logit(cutoff);
    DstarTable tbl;
    MDET_TRY(build_dstar_table(ctx, g.ls, n, L, &tbl));
    tm.mark();
    uint2* cand = nullptr;
    unsigned long long ncand = 0;
    MDET_TRY(run_filter(ctx, mode, g, false, nullptr, nullptr, nullptr, 0, nullptr, nullptr, tbl, "g", &cand, &ncand));
    tm.mark();
    Edge* edges = nullptr;
    unsigned long long ne = 0;
    uint32_t* deg = nullptr;
    MDET_TRY(exact_graph(ctx, g, cand, ncand, L, &edges, &ne, &deg));
    tm.mark();
    MDET_TRY(select_topk(ctx, g, edges, ne, deg, max_edges, total));
    tm.mark();
    if (st) {
        st->n_candidates = ncand;
        st->n_above_cutoff = ne;
        // 128 x 256 tiles of the triangular schedule
        const uint64_t ta = (n + 127) / 128, tb = (n + 255) / 256, h = ta >> 1;
        st->tiles_total = ta * tb - ((ta & 1) ? h * h : (h ? h * (h - 1) : 0));
        st->tiles_computed = st->tiles_total;
        st->ms_prep = tm.ms(0, 1);
        st->ms_filter = tm.ms(1, 2);
        st->ms_exact = tm.ms(2, 3);
        st->ms_select = tm.ms(3, 4);
        st->tile_m_n = (uint32_t)ctx->last_tile_n;
    }
    return MDET_OK;
}

// Candidates of a rectangular pass (A row a = sorted position s0 + a, B
// column c) compacted into pairs of sorted positions: the pair with itself
// goes, and a pair of two rows of the shard is kept once (r < c); so every
// unordered pair that touches the shard is scored exactly once.
__global__ void k_shard_pairs(const uint2* __restrict__ in, unsigned long long nin, uint32_t s0, uint32_t s1,
                              uint2* __restrict__ out, unsigned long long* __restrict__ nout) {
    for (unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; i < nin;
         i += (unsigned long long)gridDim.x * blockDim.x) {
        const uint2 p = in[i];
        const uint32_t r = s0 + p.x, c = p.y;
        if (c == r || (c >= s0 && c < s1 && c < r)) continue;
        out[atomicAdd(nout, 1ull)] = make_uint2(r, c);
    }
}

// Row shard `shard` of `nshards` (PLAIN or BF16): the contiguous block
// [s0, s1) of the size-sorted rows (256-row boundaries) against all rows;
// the edges emitted are those of the block's rows, so the shards' outputs
// together are the whole graph (cuda/Cuda2.cu:888-891 splits row tiles over
// devices the same way).
int graph_shard_core(mdet_ctx* ctx, const float* d_tnf, const double* d_ls, uint64_t n, double cutoff,
                     uint32_t max_edges, int mode, uint32_t shard, uint32_t nshards, mdet_graph_stats* st,
                     GraphPrep& g, uint64_t* total) {
    if (mode != MDET_MODE_PLAIN && mode != MDET_MODE_BF16)
        return ctx_fail(ctx, MDET_ERR_UNSUPPORTED, "row shards run the plain or BF16 form");
    if (nshards == 0 || shard >= nshards) return ctx_fail(ctx, MDET_ERR_INVALID, "shard %u of %u", shard, nshards);
    if (max_edges > 512) return ctx_fail(ctx, MDET_ERR_INVALID, "row shards need max_edges <= 512");
    PhaseTimer tm(ctx->stream);
    tm.mark();
    MDET_TRY(prep_sorted(ctx, d_tnf, d_ls, n, tc_kind(mode), &g));
    MDET_TRY(abd_gate(ctx, g));
    const uint64_t blocks = (n + 255) / 256;
    const uint32_t s0 = (uint32_t)std::min<uint64_t>(n, blocks * shard / nshards * 256);
    const uint32_t s1 = (uint32_t)std::min<uint64_t>(n, blocks * (shard + 1) / nshards * 256);
    const double L = logit(cutoff);
    DstarTable tbl;
    MDET_TRY(build_dstar_table(ctx, g.ls, n, L, &tbl));
    tm.mark();
    uint2* cand = nullptr;
    unsigned long long ncand = 0;
    const uint32_t na = s1 - s0;
    if (na) {
        uint2* raw = nullptr;
        unsigned long long nraw = 0;
        MDET_TRY(run_filter(ctx, mode, g, true, g.x32 + (uint64_t)s0 * MDET_NTNF,
                            mode == MDET_MODE_BF16 ? g.xa + (uint64_t)s0 * MDET_KPAD : nullptr,
                            mode == MDET_MODE_BF16 ? g.nsq + s0 : nullptr, na,
                            mode == MDET_MODE_BF16 ? g.meta + s0 / MDET_BLK : nullptr, g.meta32 + s0 / MDET_BLK, tbl,
                            "sh", &raw, &nraw));
        cand = (uint2*)ctx_scratch(ctx, "sh.pairs", (nraw ? nraw : 1) * sizeof(uint2));
        unsigned long long* dn = (unsigned long long*)ctx_scratch(ctx, "sh.np", 8);
        if (!cand || !dn) return MDET_ERR_NOMEM;
        MDET_CUDA(ctx, cudaMemsetAsync(dn, 0, 8, ctx->stream));
        if (nraw) {
            const unsigned gb = (unsigned)std::min<unsigned long long>((nraw + 255) / 256, ctx->num_sms * 16ull);
            k_shard_pairs<<<gb, 256, 0, ctx->stream>>>(raw, nraw, s0, s1, cand, dn);
            MDET_LAUNCHED(ctx, "k_shard_pairs");
        }
        MDET_CUDA(ctx, cudaMemcpyAsync(&ncand, dn, 8, cudaMemcpyDeviceToHost, ctx->stream));
        MDET_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    }
    tm.mark();
    Edge* edges = nullptr;
    unsigned long long ne = 0;
    uint32_t* deg = nullptr;
    MDET_TRY(exact_graph(ctx, g, cand, ncand, L, &edges, &ne, &deg));
    tm.mark();
    MDET_TRY(select_topk(ctx, g, edges, ne, deg, max_edges, total, nullptr, nullptr, s0, s1));
    tm.mark();
    if (st) {
        st->n_candidates = ncand;
        st->n_above_cutoff = ne;
        st->tiles_total = st->tiles_computed = ((uint64_t)na + 127) / 128 * ((n + 255) / 256);
        st->ms_prep = tm.ms(0, 1);
        st->ms_filter = tm.ms(1, 2);
        st->ms_exact = tm.ms(2, 3);
        st->ms_select = tm.ms(3, 4);
        st->tile_m_n = (uint32_t)ctx->last_tile_n;
    }
    return MDET_OK;
}

int validate_graph_args(mdet_ctx* ctx, uint64_t n, double cutoff, uint32_t max_edges, int mode) {
    if (!(cutoff > 0.0 && cutoff < 1.0)) return ctx_fail(ctx, MDET_ERR_INVALID, "cutoff must lie in (0, 1)");
    if (max_edges == 0 || max_edges > 4096) return ctx_fail(ctx, MDET_ERR_INVALID, "max_edges must be in [1, 4096]");
    if (n >= (1ull << 31)) return ctx_fail(ctx, MDET_ERR_INVALID, "too many contigs");
    return check_mode(ctx, mode);
}

// --- max-probability sample on a prepared contig set ---
int maxprob_core(mdet_ctx* ctx, const GraphPrep& g, const uint64_t* d_contigs, uint64_t m, int mode,
                 double floor_prob, double* d_out, double* lrange = nullptr) {
    cudaStream_t s = ctx->stream;
    if (m == 0) return MDET_OK;
    uint32_t* keys = (uint32_t*)ctx_scratch(ctx, "mp.keys", m * 4);
    uint32_t* keys2 = (uint32_t*)ctx_scratch(ctx, "mp.keys2", m * 4);
    uint32_t* vals = (uint32_t*)ctx_scratch(ctx, "mp.vals", m * 4);
    uint32_t* order = (uint32_t*)ctx_scratch(ctx, "mp.order", m * 4);
    uint32_t* slot_of = (uint32_t*)ctx_scratch(ctx, "mp.slot", m * 4);
    uint64_t mpad = (m + 255) / 256 * 256;
    float* a32 = (float*)ctx_scratch(ctx, "mp.a32", m * MDET_NTNF * 4);
    double* als = (double*)ctx_scratch(ctx, "mp.als", m * 8);
    uint64_t nblk = mpad / MDET_BLK;
    BlockMeta* ameta32 = (BlockMeta*)ctx_scratch(ctx, "mp.meta32", nblk * sizeof(BlockMeta));
    BlockMeta* ameta = (BlockMeta*)ctx_scratch(ctx, "mp.meta", nblk * sizeof(BlockMeta));
    if (!keys || !keys2 || !vals || !order || !slot_of || !a32 || !als || !ameta32 || !ameta) return MDET_ERR_NOMEM;
    k_sample_sort_keys<<<(unsigned)((m + 255) / 256), 256, 0, s>>>(d_contigs, g.inv, m, keys, vals);
    MDET_LAUNCHED(ctx, "k_sample_sort_keys");
    size_t tb = 0;
    cub::DeviceRadixSort::SortPairs(nullptr, tb, keys, keys2, vals, order, (int)m, 0, 32, s);
    void* tmp = ctx_scratch(ctx, "mp.cubtmp", tb);
    if (!tmp) return MDET_ERR_NOMEM;
    MDET_CUDA(ctx, cub::DeviceRadixSort::SortPairs(tmp, tb, keys, keys2, vals, order, (int)m, 0, 32, s));
    const uint32_t* row_map = keys2;  // sorted positions of the sample, ascending
    k_sample_gather<<<(unsigned)m, 64, 0, s>>>(row_map, order, m, g.x32, g.ls, a32, als, slot_of);
    MDET_LAUNCHED(ctx, "k_sample_gather");
    const double L = floor_prob > 0 ? logit(floor_prob) : -INFINITY;
    DstarTable tbl;
    MDET_TRY(build_dstar_table(ctx, g.ls, g.n, L, &tbl, true, lrange));
    uint2* cand = nullptr;
    unsigned long long ncand = 0;
    if (mode != MDET_MODE_PLAIN) {
        // tensor-core forms: all rows in the A role (each A tile read once)
        // against the sample in the B role (small enough to stay in L2), so
        // the pairs come out as (row, sample slot)
        uint16_t* sb = (uint16_t*)ctx_scratch(ctx, "mp.sb", mpad * MDET_KPAD * 2);
        if (!sb) return MDET_ERR_NOMEM;
        k_sample_gather_b<<<(unsigned)((mpad + 7) / 8), 256, 0, s>>>(row_map, m, mpad, g.xb, sb);
        MDET_LAUNCHED(ctx, "k_sample_gather_b");
        k_sample_meta<<<(unsigned)((nblk * 32 + 127) / 128), 128, 0, s>>>(row_map, m, g.ls, g.meta, nblk, ameta);
        MDET_LAUNCHED(ctx, "k_sample_meta");
        const BSide bs{sb, (uint32_t)m, ameta};
        MDET_TRY(run_filter(ctx, mode, g, true, nullptr, nullptr, nullptr, 0, nullptr, nullptr, tbl, "mp", &cand,
                            &ncand, nullptr, 0, nullptr, 0, 0, 0, nullptr, nullptr, &bs));
        MDET_TRY(exact_maxprob(ctx, g, cand, ncand, row_map, m, slot_of, d_out, true));
        return MDET_OK;
    }
    k_sample_meta<<<(unsigned)((nblk * 32 + 127) / 128), 128, 0, s>>>(row_map, m, g.ls, g.meta32, nblk, ameta32);
    MDET_LAUNCHED(ctx, "k_sample_meta");
    MDET_TRY(run_filter(ctx, mode, g, true, a32, nullptr, nullptr, (uint32_t)m, ameta, ameta32, tbl, "mp", &cand,
                        &ncand));
    MDET_TRY(exact_maxprob(ctx, g, cand, ncand, row_map, m, slot_of, d_out));
    return MDET_OK;
}

extern "C" {

// The graph, or with nshards > 0 row shard `shard` of it (graph_shard_core).
static int graph_select(mdet_ctx* ctx, const float* d_tnf, const double* d_ls, uint64_t n, double cutoff,
                        uint32_t max_edges, int mode, uint32_t shard, uint32_t nshards, mdet_graph_stats* st,
                        GraphPrep& g, uint64_t* total) {
    if (nshards) return graph_shard_core(ctx, d_tnf, d_ls, n, cutoff, max_edges, mode, shard, nshards, st, g, total);
    return graph_core(ctx, d_tnf, d_ls, n, cutoff, max_edges, mode, st, g, total);
}

static int graph_dev_impl(mdet_ctx* ctx, const float* d_tnf, const double* d_log_size, uint64_t n, double cutoff,
                          uint32_t max_edges, int mode, uint32_t shard, uint32_t nshards, uint64_t* d_from,
                          uint64_t* d_to, double* d_stnf, uint64_t capacity, uint64_t* n_edges,
                          mdet_graph_stats* stats) {
    if (!ctx || !n_edges) return MDET_ERR_INVALID;
    MDET_CUDA(ctx, cudaSetDevice(ctx->device));
    ctx->launches = 0;
    if (stats) memset(stats, 0, sizeof(*stats));
    *n_edges = 0;
    MDET_TRY(validate_graph_args(ctx, n, cutoff, max_edges, mode));
    if (n < 2) return MDET_OK;
    if (!d_tnf || !d_log_size) return ctx_fail(ctx, MDET_ERR_INVALID, "null pointer");
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventRecord(e0, ctx->stream);
    GraphPrep g;
    uint64_t total = 0;
    int rc = graph_select(ctx, d_tnf, d_log_size, n, cutoff, max_edges, mode, shard, nshards, stats, g, &total);
    if (rc == MDET_OK) {
        *n_edges = total;
        if (total > capacity)
            rc = ctx_fail(ctx, MDET_ERR_CAPACITY, "edge output needs %llu entries, capacity %llu",
                          (unsigned long long)total, (unsigned long long)capacity);
        else if (total && (!d_from || !d_to || !d_stnf))
            rc = ctx_fail(ctx, MDET_ERR_INVALID, "null output pointer");
        else
            rc = emit_topk(ctx, g, max_edges, d_from, d_to, d_stnf, total);
    }
    cudaEventRecord(e1, ctx->stream);
    if (rc == MDET_OK) rc = check_flag(ctx);
    if (stats) {
        float ms = 0;
        cudaEventSynchronize(e1);
        cudaEventElapsedTime(&ms, e0, e1);
        stats->ms_total = ms;
        stats->n_edges = total;
        stats->gpu_launches = ctx->launches;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return rc;
}

int mdet_tnf_graph_dev(mdet_ctx* ctx, const float* d_tnf, const double* d_log_size, uint64_t n, double cutoff,
                       uint32_t max_edges, int mode, uint64_t* d_from, uint64_t* d_to, double* d_stnf,
                       uint64_t capacity, uint64_t* n_edges, mdet_graph_stats* stats) {
    return graph_dev_impl(ctx, d_tnf, d_log_size, n, cutoff, max_edges, mode, 0, 0, d_from, d_to, d_stnf, capacity,
                          n_edges, stats);
}

int mdet_tnf_graph_shard_dev(mdet_ctx* ctx, const float* d_tnf, const double* d_log_size, uint64_t n, double cutoff,
                             uint32_t max_edges, int mode, uint32_t shard, uint32_t nshards, uint64_t* d_from,
                             uint64_t* d_to, double* d_stnf, uint64_t capacity, uint64_t* n_edges,
                             mdet_graph_stats* stats) {
    if (!ctx) return MDET_ERR_INVALID;
    if (nshards == 0) return ctx_fail(ctx, MDET_ERR_INVALID, "nshards must be at least 1");
    return graph_dev_impl(ctx, d_tnf, d_log_size, n, cutoff, max_edges, mode, shard, nshards, d_from, d_to, d_stnf,
                          capacity, n_edges, stats);
}

static int graph_host_impl(mdet_ctx* ctx, const float* tnf, const double* log_size, uint64_t n, double cutoff,
                           uint32_t max_edges, int mode, uint32_t shard, uint32_t nshards, uint64_t* from,
                           uint64_t* to, double* stnf, uint64_t capacity, uint64_t* n_edges,
                           mdet_graph_stats* stats) {
    if (!ctx || !n_edges) return MDET_ERR_INVALID;
    MDET_CUDA(ctx, cudaSetDevice(ctx->device));
    ctx->launches = 0;
    if (stats) memset(stats, 0, sizeof(*stats));
    *n_edges = 0;
    MDET_TRY(validate_graph_args(ctx, n, cutoff, max_edges, mode));
    if (n < 2) return MDET_OK;
    if (!tnf || !log_size) return ctx_fail(ctx, MDET_ERR_INVALID, "null pointer");
    cudaStream_t s = ctx->stream;
    float* d_tnf = (float*)ctx_scratch(ctx, "io.gtnf", n * MDET_NTNF * 4);
    double* d_ls = (double*)ctx_scratch(ctx, "io.gls", n * 8);
    if (!d_tnf || !d_ls) return MDET_ERR_NOMEM;
    MDET_CUDA(ctx, cudaMemcpyAsync(d_tnf, tnf, n * MDET_NTNF * 4, cudaMemcpyHostToDevice, s));
    MDET_CUDA(ctx, cudaMemcpyAsync(d_ls, log_size, n * 8, cudaMemcpyHostToDevice, s));
    GraphPrep g;
    uint64_t total = 0;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventRecord(e0, s);
    int rc = graph_select(ctx, d_tnf, d_ls, n, cutoff, max_edges, mode, shard, nshards, stats, g, &total);
    if (rc == MDET_OK) {
        *n_edges = total;
        if (total > capacity) {
            rc = ctx_fail(ctx, MDET_ERR_CAPACITY, "edge output needs %llu entries, capacity %llu",
                          (unsigned long long)total, (unsigned long long)capacity);
        } else if (total) {
            uint64_t* df = (uint64_t*)ctx_scratch(ctx, "io.from", total * 8);
            uint64_t* dt = (uint64_t*)ctx_scratch(ctx, "io.to", total * 8);
            double* ds = (double*)ctx_scratch(ctx, "io.stnf", total * 8);
            if (!df || !dt || !ds) {
                rc = MDET_ERR_NOMEM;
            } else if (!from || !to || !stnf) {
                rc = ctx_fail(ctx, MDET_ERR_INVALID, "null output pointer");
            } else {
                rc = emit_topk(ctx, g, max_edges, df, dt, ds, total);
                if (rc == MDET_OK) {
                    cudaMemcpyAsync(from, df, total * 8, cudaMemcpyDeviceToHost, s);
                    cudaMemcpyAsync(to, dt, total * 8, cudaMemcpyDeviceToHost, s);
                    rc = ctx_cuda(ctx, cudaMemcpyAsync(stnf, ds, total * 8, cudaMemcpyDeviceToHost, s), "copy out");
                }
            }
        }
    }
    cudaEventRecord(e1, s);
    if (rc == MDET_OK) rc = check_flag(ctx);
    if (stats) {
        float ms = 0;
        cudaEventSynchronize(e1);
        cudaEventElapsedTime(&ms, e0, e1);
        stats->ms_total = ms;
        stats->n_edges = total;
        stats->gpu_launches = ctx->launches;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return rc;
}

int mdet_tnf_graph(mdet_ctx* ctx, const float* tnf, const double* log_size, uint64_t n, double cutoff,
                   uint32_t max_edges, int mode, uint64_t* from, uint64_t* to, double* stnf, uint64_t capacity,
                   uint64_t* n_edges, mdet_graph_stats* stats) {
    return graph_host_impl(ctx, tnf, log_size, n, cutoff, max_edges, mode, 0, 0, from, to, stnf, capacity, n_edges,
                           stats);
}

int mdet_tnf_graph_shard(mdet_ctx* ctx, const float* tnf, const double* log_size, uint64_t n, double cutoff,
                         uint32_t max_edges, int mode, uint32_t shard, uint32_t nshards, uint64_t* from,
                         uint64_t* to, double* stnf, uint64_t capacity, uint64_t* n_edges, mdet_graph_stats* stats) {
    if (!ctx) return MDET_ERR_INVALID;
    if (nshards == 0) return ctx_fail(ctx, MDET_ERR_INVALID, "nshards must be at least 1");
    return graph_host_impl(ctx, tnf, log_size, n, cutoff, max_edges, mode, shard, nshards, from, to, stnf, capacity,
                           n_edges, stats);
}

int mdet_tnf_pair_scores_dev(mdet_ctx* ctx, const float* d_tnf, const double* d_log_size, uint64_t n,
                             const uint64_t* d_pairs, uint64_t m, double* d_dist, double* d_prob) {
    if (!ctx) return MDET_ERR_INVALID;
    MDET_CUDA(ctx, cudaSetDevice(ctx->device));
    ctx->launches = 0;
    if (m == 0) return MDET_OK;
    if (!d_tnf || !d_log_size || !d_pairs || (!d_dist && !d_prob)) return ctx_fail(ctx, MDET_ERR_INVALID, "null pointer");
    if (n < 1 || n >= (1ull << 31)) return ctx_fail(ctx, MDET_ERR_INVALID, "bad contig count");
    GraphPrep g;
    MDET_TRY(prep_sorted(ctx, d_tnf, d_log_size, n, false, &g));
    MDET_TRY(pair_scores(ctx, g, d_pairs, m, d_dist, d_prob));
    MDET_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return check_flag(ctx);
}

int mdet_tnf_max_prob_dev(mdet_ctx* ctx, const float* d_tnf, const double* d_log_size, uint64_t n,
                          const uint64_t* d_contigs, uint64_t m, int mode, double floor_prob, double* d_out) {
    if (!ctx) return MDET_ERR_INVALID;
    MDET_CUDA(ctx, cudaSetDevice(ctx->device));
    ctx->launches = 0;
    MDET_TRY(check_mode(ctx, mode));
    if (m > n) return ctx_fail(ctx, MDET_ERR_INVALID, "sample larger than the contig set");
    if (n >= (1ull << 31)) return ctx_fail(ctx, MDET_ERR_INVALID, "too many contigs");
    if (m == 0) return MDET_OK;
    if (!d_tnf || !d_log_size || !d_contigs || !d_out) return ctx_fail(ctx, MDET_ERR_INVALID, "null pointer");
    // Each sampled row's maximum comes from the exact stage over the
    // filter's candidates, so every filter form gives the same maxima; the
    // sample passes (sampled rows in the B role) use the BF16 filter when
    // TF32 is asked for.
    if (mode == MDET_MODE_TF32) mode = MDET_MODE_BF16;
    GraphPrep g;
    MDET_TRY(prep_sorted(ctx, d_tnf, d_log_size, n, mode != MDET_MODE_PLAIN, &g));
    MDET_TRY(maxprob_core(ctx, g, d_contigs, m, mode, floor_prob, d_out));
    return check_flag(ctx);
}

int mdet_tnf_max_prob(mdet_ctx* ctx, const float* tnf, const double* log_size, uint64_t n, const uint64_t* contigs,
                      uint64_t m, int mode, double floor_prob, double* out) {
    if (!ctx) return MDET_ERR_INVALID;
    MDET_CUDA(ctx, cudaSetDevice(ctx->device));
    if (m > n) return ctx_fail(ctx, MDET_ERR_INVALID, "sample larger than the contig set");
    if (m == 0) return MDET_OK;
    if (!tnf || !log_size || !contigs || !out) return ctx_fail(ctx, MDET_ERR_INVALID, "null pointer");
    for (uint64_t b = 0; b < m; ++b)
        if (contigs[b] >= n) return ctx_fail(ctx, MDET_ERR_INVALID, "contig index out of range");
    cudaStream_t s = ctx->stream;
    float* d_tnf = (float*)ctx_scratch(ctx, "io.gtnf", n * MDET_NTNF * 4);
    double* d_ls = (double*)ctx_scratch(ctx, "io.gls", n * 8);
    uint64_t* d_c = (uint64_t*)ctx_scratch(ctx, "io.contigs", m * 8);
    double* d_o = (double*)ctx_scratch(ctx, "io.mpout", m * 8);
    if (!d_tnf || !d_ls || !d_c || !d_o) return MDET_ERR_NOMEM;
    MDET_CUDA(ctx, cudaMemcpyAsync(d_tnf, tnf, n * MDET_NTNF * 4, cudaMemcpyHostToDevice, s));
    MDET_CUDA(ctx, cudaMemcpyAsync(d_ls, log_size, n * 8, cudaMemcpyHostToDevice, s));
    MDET_CUDA(ctx, cudaMemcpyAsync(d_c, contigs, m * 8, cudaMemcpyHostToDevice, s));
    MDET_TRY(mdet_tnf_max_prob_dev(ctx, d_tnf, d_ls, n, d_c, m, mode, floor_prob, d_o));
    MDET_CUDA(ctx, cudaMemcpyAsync(out, d_o, m * 8, cudaMemcpyDeviceToHost, s));
    MDET_CUDA(ctx, cudaStreamSynchronize(s));
    return MDET_OK;
}

// gen_tnf_graph_sample + driver (cuda/Cuda2.cu:972-1025, 1883-1904).
int mdet_tnf_ptnf_search_dev(mdet_ctx* ctx, const float* d_tnf, const double* d_log_size, uint64_t n,
                             double coverage, int mode, double* ptnf_out) {
    if (!ctx || !ptnf_out) return MDET_ERR_INVALID;
    MDET_CUDA(ctx, cudaSetDevice(ctx->device));
    ctx->launches = 0;
    MDET_TRY(check_mode(ctx, mode));
    if (n < 2) return ctx_fail(ctx, MDET_ERR_INVALID, "need at least two contigs");
    if (n >= (1ull << 31)) return ctx_fail(ctx, MDET_ERR_INVALID, "too many contigs");
    cudaStream_t s = ctx->stream;
    // the sample passes use the BF16 filter when TF32 is asked for (the
    // maxima are exact whatever the filter form; see mdet_tnf_max_prob_dev)
    if (mode == MDET_MODE_TF32) mode = MDET_MODE_BF16;
    GraphPrep g;
    MDET_TRY(prep_sorted(ctx, d_tnf, d_log_size, n, mode != MDET_MODE_PLAIN, &g));
    std::vector<uint64_t> idx(n);
    // sparse shuffle state: open addressing over positions (key ~0: empty)
    std::vector<uint64_t> mkey, mval;
    // ge[q]: how many sampled maxima are >= q / 1000. (q = 0..1000)
    std::vector<uint64_t> ge(1002);
    uint64_t* d_idx = (uint64_t*)ctx_scratch(ctx, "pt.idx", n * 8);
    double* d_mx = (double*)ctx_scratch(ctx, "pt.mx", n * 8);
    if (!d_idx || !d_mx) return MDET_ERR_NOMEM;
    // the search only compares maxima against cutoffs above 0.700
    const double floor_prob = 0.7;
    // first floor of a pass: just below the previous pass's cutoff, on a
    // 0.005 grid so that passes share a d* table
    double next_floor = 0.9;
    double lrange[2] = {NAN, NAN};  // log-size range of the sorted rows, found once
    auto sample = [&](bool full, double* p_out) -> int {
        uint64_t m = full ? n : std::min<uint64_t>(n, 2500);
        // random_unique (cuda/Cuda2.cu:500-511): a partial Fisher-Yates
        // shuffle of 0..n-1 whose first m entries are the sample; step p
        // swaps position p with p + rand() % (n - p)
        if (m == n) {
            std::iota(idx.begin(), idx.end(), (uint64_t)0);
            for (uint64_t p = 0; p < m; ++p) std::swap(idx[p], idx[p + (uint64_t)rand() % (n - p)]);
        } else {
            // the same draws on a sparse array (untouched positions hold their
            // own index), so a pass costs O(m) instead of O(n); the moved
            // positions live in a linear-probing table of >= 4m slots
            uint64_t cap = 16;
            while (cap < 4 * m) cap <<= 1;
            mkey.assign(cap, ~0ull);
            mval.resize(cap);
            auto slot = [&](uint64_t i) {
                uint64_t h = (i * 0x9E3779B97F4A7C15ull) >> 20;
                while (true) {
                    h &= cap - 1;
                    if (mkey[h] == i || mkey[h] == ~0ull) return h;
                    ++h;
                }
            };
            auto at = [&](uint64_t i) {
                const uint64_t h = slot(i);
                return mkey[h] == i ? mval[h] : i;
            };
            for (uint64_t p = 0; p < m; ++p) {
                const uint64_t r = p + (uint64_t)rand() % (n - p);
                const uint64_t vp = at(p), vr = at(r);
                idx[p] = vr;  // later steps only touch positions after p
                const uint64_t h = slot(r);
                mkey[h] = r;
                mval[h] = vp;
            }
        }
        // Maxima at floor f1 >= floor_prob first: a maximum at or above f1 is
        // exact (the pair that attains it is a candidate at that floor), so the
        // cuts the search makes at or above f1 see the same counts.  Samples
        // below f1 are scored again at floor_prob only if the search goes
        // below f1.  The result is the same for any f1; a higher f1 just
        // means fewer candidate pairs.
        const double f1 = full ? floor_prob : std::max(floor_prob, next_floor);
        auto maxima = [&](const uint64_t* ids, uint64_t k, double floor, double* out) -> int {
            MDET_CUDA(ctx, cudaMemcpyAsync(d_idx, ids, k * 8, cudaMemcpyHostToDevice, s));
            MDET_TRY(maxprob_core(ctx, g, d_idx, k, mode, floor, d_mx, lrange));
            MDET_CUDA(ctx, cudaMemcpyAsync(out, d_mx, k * 8, cudaMemcpyDeviceToHost, s));
            MDET_CUDA(ctx, cudaStreamSynchronize(s));
            return MDET_OK;
        };
        std::vector<double> raw(m);
        MDET_TRY(maxima(idx.data(), m, f1, raw.data()));
        std::vector<uint64_t> low;  // sample positions whose maximum is below f1
        if (f1 > floor_prob)
            for (uint64_t i = 0; i < m; ++i)
                if (!(raw[i] >= f1)) low.push_back(i);
        // counts of maxima at or above each cut q / 1000. (what walking the
        // maxima sorted in descending order gives, without the sort)
        auto count_cuts = [&]() {
            std::fill(ge.begin(), ge.end(), 0);
            for (uint64_t i = 0; i < m; ++i) {
                const double v = raw[i];
                if (!(v >= 0.)) continue;  // below every cut (or NaN)
                int q = v >= 1. ? 1000 : (int)(v * 1000.);
                while (q < 1000 && v >= (double)(q + 1) / 1000.) ++q;
                while (q > 0 && !(v >= (double)q / 1000.)) --q;
                ge[q]++;
            }
            for (int q = 999; q >= 0; --q) ge[q] += ge[q + 1];
        };
        count_cuts();
        uint64_t p = 999, pp = 1000, counton = 0;
        double cov = 0, pcov = 0;
        for (; p > 700;) {
            double cut = (double)p / 1000.;
            if (cut < f1 && !low.empty()) {
                // the exact maxima below f1 (all of them lie below f1, so the
                // first counton entries of the sorted list stay in place)
                std::vector<uint64_t> ids(low.size());
                std::vector<double> v(low.size());
                for (size_t i = 0; i < low.size(); ++i) ids[i] = idx[low[i]];
                MDET_TRY(maxima(ids.data(), ids.size(), floor_prob, v.data()));
                for (size_t i = 0; i < low.size(); ++i) raw[low[i]] = v[i];
                low.clear();
                count_cuts();
            }
            counton = ge[p];
            cov = (double)counton / m;
            if (cov >= coverage) {
                if (cov - coverage > coverage - pcov) {
                    p = pp;
                    cov = pcov;
                }
                break;
            }
            pp = p;
            pcov = cov;
            if (p > 990)
                p -= rand() % 3 + 1;
            else if (p > 900)
                p -= rand() % 3 + 3;
            else
                p -= rand() % 3 + 9;
        }
        *p_out = (double)p;
        return MDET_OK;
    };
    double ptnf = 0;
    if (n <= 25000) {
        MDET_TRY(sample(true, &ptnf));
    } else {
        for (int i = 0; i < 10; ++i) {
            double minp = 0;
            MDET_TRY(sample(false, &minp));
            next_floor = std::floor((minp - 10.) / 5.) * 5. / 1000.;
            if (minp < 701) minp = 700.;
            ptnf += minp;
            if (i == 1 && ptnf / 2 < 701) {
                ptnf = 700.;
                break;
            }
            if (i == 9) ptnf /= 10.;
        }
    }
    *ptnf_out = ptnf;
    return check_flag(ctx);
}

int mdet_tnf_ptnf_search(mdet_ctx* ctx, const float* tnf, const double* log_size, uint64_t n, double coverage,
                         int mode, double* ptnf_out) {
    if (!ctx || !ptnf_out) return MDET_ERR_INVALID;
    MDET_CUDA(ctx, cudaSetDevice(ctx->device));
    if (!tnf || !log_size) return ctx_fail(ctx, MDET_ERR_INVALID, "null pointer");
    if (n >= (1ull << 31)) return ctx_fail(ctx, MDET_ERR_INVALID, "too many contigs");
    cudaStream_t s = ctx->stream;
    float* d_tnf = (float*)ctx_scratch(ctx, "io.gtnf", n * MDET_NTNF * 4);
    double* d_ls = (double*)ctx_scratch(ctx, "io.gls", (n ? n : 1) * 8);
    if (!d_tnf || !d_ls) return MDET_ERR_NOMEM;
    MDET_CUDA(ctx, cudaMemcpyAsync(d_tnf, tnf, n * MDET_NTNF * 4, cudaMemcpyHostToDevice, s));
    MDET_CUDA(ctx, cudaMemcpyAsync(d_ls, log_size, n * 8, cudaMemcpyHostToDevice, s));
    return mdet_tnf_ptnf_search_dev(ctx, d_tnf, d_ls, n, coverage, mode, ptnf_out);
}

}  // extern "C"
