// graph_batch.cu -- mdet_tnf_graph_batched: the TNF graphs of many
// independent assemblies in one pass.  The reference builds one graph per
// run (gen_tnf_graph, cuda/Cuda2.cu:861-970); here every assembly's prepared
// rows are laid end to end (each padded to 256 rows, so no tile straddles two
// assemblies), one tile list covers the upper triangles of all of them, and
// a single filter launch, one exact-stage launch and one selection launch
// serve the whole batch.  Per-assembly cutoffs and max_edges ride along as
// per-block side tables; outputs go to each assembly's own buffers.
#include <cub/cub.cuh>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <vector>

#include "graph.cuh"

namespace {

struct BatchOut {
    uint64_t* from;
    uint64_t* to;
    double* stnf;
    unsigned long long out0;  // output offset of the assembly's first row
    uint32_t R, n;            // first row, contigs
    int emit;
    int pad;
};

// Block per row tile I: its column tiles [j0[I], j1[I]) as I * tcols + J.
__global__ void k_tile_list(const uint32_t* __restrict__ j0, const uint32_t* __restrict__ j1,
                            const unsigned long long* __restrict__ off, uint32_t tcols, uint32_t* __restrict__ list) {
    const uint32_t I = blockIdx.x;
    const uint32_t a = j0[I], b = j1[I];
    const unsigned long long o = off[I];
    for (uint32_t J = a + threadIdx.x; J < b; J += blockDim.x) list[o + (J - a)] = I * tcols + J;
}

// Log-size ranges (the prepared rows are ascending per assembly) and output
// offsets of every assembly.
__global__ void k_batch_ends(const double* __restrict__ ls, const unsigned long long* __restrict__ outptr,
                             const uint32_t* __restrict__ R, const uint32_t* __restrict__ n, uint32_t count,
                             double* __restrict__ range, unsigned long long* __restrict__ outs) {
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= count) return;
    if (n[k] == 0) {
        range[2 * k] = range[2 * k + 1] = 0;
        outs[2 * k] = outs[2 * k + 1] = 0;
        return;
    }
    range[2 * k] = ls[R[k]];
    range[2 * k + 1] = ls[R[k] + n[k] - 1];
    if (outptr) {
        outs[2 * k] = outptr[R[k]];
        outs[2 * k + 1] = outptr[R[k] + n[k]];
    }
}

// Warp per row o of the batch (original order, offset by its assembly's
// first row): the row's kept edges, already compacted and sorted by the
// selection, go to its assembly's outputs with local indices.
__global__ void k_emit_batch(const uint32_t* __restrict__ inv, const unsigned long long* __restrict__ rowptr,
                             const Ent* __restrict__ list, const unsigned long long* __restrict__ outptr,
                             const uint32_t* __restrict__ blk_asm, const BatchOut* __restrict__ outs, uint32_t N) {
    const uint32_t lane = threadIdx.x & 31;
    for (uint32_t o = blockIdx.x * (blockDim.x / 32) + (threadIdx.x >> 5); o < N; o += gridDim.x * (blockDim.x / 32)) {
        const BatchOut bo = outs[blk_asm[o >> 8]];
        if (!bo.emit || o - bo.R >= bo.n) continue;
        const uint32_t s = inv[o];
        const unsigned long long p0 = outptr[o];
        const uint32_t cnt = (uint32_t)(outptr[o + 1] - p0);
        const Ent* row = list + rowptr[s];
        for (uint32_t i = lane; i < cnt; i += 32) {
            const Ent x = row[i];
            const unsigned long long q = p0 - bo.out0 + i;
            bo.from[q] = o - bo.R;
            bo.to[q] = x.ocol - bo.R;
            bo.stnf[q] = x.sim;
        }
    }
}

}  // namespace

extern "C" int mdet_tnf_graph_batched(mdet_ctx* ctx, mdet_assembly* as, uint32_t count, int mode,
                                      mdet_graph_stats* stats) {
    if (!ctx) return MDET_ERR_INVALID;
    MDET_CUDA(ctx, cudaSetDevice(ctx->device));
    ctx->launches = 0;
    if (stats) memset(stats, 0, sizeof(*stats));
    if (count == 0) return MDET_OK;
    if (!as) return ctx_fail(ctx, MDET_ERR_INVALID, "null assembly array");
    if (mode != MDET_MODE_PLAIN && mode != MDET_MODE_BF16)
        return ctx_fail(ctx, MDET_ERR_UNSUPPORTED, "batched graphs take the plain or the BF16 form");
    MDET_TRY(check_mode(ctx, mode));
    const bool bf16 = mode == MDET_MODE_BF16;
    cudaStream_t s = ctx->stream;

    // layout: assemblies end to end, each padded to 256 rows
    std::vector<uint32_t> R(count), nn(count);
    uint64_t N = 0;
    uint32_t maxK = 1;
    for (uint32_t k = 0; k < count; ++k) {
        mdet_assembly& a = as[k];
        a.status = MDET_OK;
        a.n_edges = 0;
        if (!(a.cutoff > 0.0 && a.cutoff < 1.0))
            return ctx_fail(ctx, MDET_ERR_INVALID, "assembly %u: cutoff must lie in (0, 1)", k);
        if (a.max_edges == 0 || a.max_edges > 512)
            return ctx_fail(ctx, MDET_ERR_INVALID, "assembly %u: max_edges must be in [1, 512] in a batch", k);
        if (a.n >= 2 && (!a.d_tnf || !a.d_log_size))
            return ctx_fail(ctx, MDET_ERR_INVALID, "assembly %u: null input pointer", k);
        nn[k] = a.n >= 2 ? (uint32_t)std::min<uint64_t>(a.n, 0xFFFFFFFFull) : 0;
        if (a.n >= (1ull << 31)) return ctx_fail(ctx, MDET_ERR_INVALID, "assembly %u: too many contigs", k);
        R[k] = (uint32_t)N;
        N += (nn[k] + 255) / 256 * 256;
        maxK = std::max(maxK, a.max_edges);
    }
    if (N == 0) return MDET_OK;
    if (N >= (1ull << 31)) return ctx_fail(ctx, MDET_ERR_INVALID, "batch too large (%llu rows)", (unsigned long long)N);
    const uint32_t nblk256 = (uint32_t)(N / 256), nrt = (uint32_t)(N / 128);
    if ((uint64_t)nrt * nrt >= (1ull << 32)) return ctx_fail(ctx, MDET_ERR_INVALID, "batch too large for the tile list");

    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventRecord(e0, s);
    int rc = MDET_OK;
    auto body = [&]() -> int {
        // prepared rows of every assembly
        GraphPrep g;
        MDET_TRY(prep_alloc(ctx, "bt", N, bf16, &g));
        g.n = (uint32_t)N;
        g.npad = (uint32_t)N;
        for (uint32_t k = 0; k < count; ++k)
            if (nn[k]) MDET_TRY(prep_into(ctx, as[k].d_tnf, as[k].d_log_size, nn[k], bf16, g, R[k]));
        // per-assembly first rows and sizes; their log-size ranges
        uint32_t* dR = (uint32_t*)ctx_scratch(ctx, "bt.R", count * 4);
        uint32_t* dn = (uint32_t*)ctx_scratch(ctx, "bt.n", count * 4);
        double* drange = (double*)ctx_scratch(ctx, "bt.range", count * 16);
        unsigned long long* douts = (unsigned long long*)ctx_scratch(ctx, "bt.outs", count * 16);
        if (!dR || !dn || !drange || !douts) return MDET_ERR_NOMEM;
        MDET_CUDA(ctx, cudaMemcpyAsync(dR, R.data(), count * 4, cudaMemcpyHostToDevice, s));
        MDET_CUDA(ctx, cudaMemcpyAsync(dn, nn.data(), count * 4, cudaMemcpyHostToDevice, s));
        k_batch_ends<<<(count + 127) / 128, 128, 0, s>>>(g.ls, nullptr, dR, dn, count, drange, douts);
        MDET_LAUNCHED(ctx, "k_batch_ends");
        std::vector<double> range(2 * count);
        MDET_CUDA(ctx, cudaMemcpyAsync(range.data(), drange, count * 16, cudaMemcpyDeviceToHost, s));
        MDET_CUDA(ctx, cudaStreamSynchronize(s));
        double gmin = INFINITY, gmax = -INFINITY;
        for (uint32_t k = 0; k < count; ++k)
            if (nn[k]) {
                gmin = std::min(gmin, range[2 * k]);
                gmax = std::max(gmax, range[2 * k + 1]);
            }
        // one d* table per distinct cutoff, all over the batch's size range
        std::map<double, uint32_t> tab_of;
        for (uint32_t k = 0; k < count; ++k)
            if (nn[k] && !tab_of.count(as[k].cutoff)) {
                const uint32_t id = (uint32_t)tab_of.size();
                tab_of[as[k].cutoff] = id;
            }
        if (tab_of.size() > 255) return ctx_fail(ctx, MDET_ERR_INVALID, "more than 255 distinct cutoffs in a batch");
        float* st = (float*)ctx_scratch(ctx, "bt.tbl", tab_of.size() * MDET_TBL_FLOATS * 4);
        if (!st) return MDET_ERR_NOMEM;
        DstarTable tbl;
        for (auto& kv : tab_of)
            MDET_TRY(build_dstar_table_at(ctx, gmin, gmax, logit(kv.first), st + kv.second * MDET_TBL_FLOATS, &tbl));
        tbl.st = st;
        // per-block side tables
        std::vector<uint8_t> row_tbl(nrt, 0);
        std::vector<BlkCut> bcut(nblk256);
        std::vector<uint32_t> bK(nblk256, 1), bA(nblk256, 0);
        for (uint32_t k = 0; k < count; ++k) {
            const uint32_t npad = (nn[k] + 255) / 256 * 256;
            if (!npad) continue;
            const double L = logit(as[k].cutoff);
            BlkCut bc;
            bc.L.hi = (float)L;
            bc.L.lo = (float)(L - (double)bc.L.hi);
            bc.model2 = L < 2.1972245773362196 ? 1u : 0u;  // ln 9
            bc.pad = 0;
            for (uint32_t b = R[k] / 256; b < (R[k] + npad) / 256; ++b) {
                bcut[b] = bc;
                bK[b] = as[k].max_edges;
                bA[b] = k;
            }
            for (uint32_t i = 0; i < npad / 128; ++i) row_tbl[R[k] / 128 + i] = (uint8_t)tab_of[as[k].cutoff];
        }
        uint8_t* d_rtbl = (uint8_t*)ctx_scratch(ctx, "bt.rtbl", nrt);
        BlkCut* d_bcut = (BlkCut*)ctx_scratch(ctx, "bt.bcut", (uint64_t)nblk256 * sizeof(BlkCut));
        uint32_t* d_bK = (uint32_t*)ctx_scratch(ctx, "bt.bK", (uint64_t)nblk256 * 4);
        uint32_t* d_bA = (uint32_t*)ctx_scratch(ctx, "bt.bA", (uint64_t)nblk256 * 4);
        uint32_t* d_j0 = (uint32_t*)ctx_scratch(ctx, "bt.j0", (uint64_t)nrt * 4);
        uint32_t* d_j1 = (uint32_t*)ctx_scratch(ctx, "bt.j1", (uint64_t)nrt * 4);
        unsigned long long* d_off = (unsigned long long*)ctx_scratch(ctx, "bt.off", (uint64_t)nrt * 8);
        if (!d_rtbl || !d_bcut || !d_bK || !d_bA || !d_j0 || !d_j1 || !d_off) return MDET_ERR_NOMEM;
        MDET_CUDA(ctx, cudaMemcpyAsync(d_rtbl, row_tbl.data(), nrt, cudaMemcpyHostToDevice, s));
        MDET_CUDA(ctx, cudaMemcpyAsync(d_bcut, bcut.data(), nblk256 * sizeof(BlkCut), cudaMemcpyHostToDevice, s));
        MDET_CUDA(ctx, cudaMemcpyAsync(d_bK, bK.data(), nblk256 * 4, cudaMemcpyHostToDevice, s));
        MDET_CUDA(ctx, cudaMemcpyAsync(d_bA, bA.data(), nblk256 * 4, cudaMemcpyHostToDevice, s));

        // the tile list for column tiles of width w (upper triangle of every
        // assembly), then one filter launch over all of it
        uint64_t nlist = 0;
        std::vector<uint32_t> j0(nrt), j1(nrt);
        std::vector<unsigned long long> off(nrt + 1);
        uint2* cand = nullptr;
        unsigned long long ncand = 0;
        auto run = [&](int w) -> int {
            const uint32_t sh = w == 256 ? 1u : 0u;
            for (uint32_t k = 0; k < count; ++k) {
                const uint32_t npad = (nn[k] + 255) / 256 * 256;
                const uint32_t t0 = R[k] / 128;
                for (uint32_t i = 0; i < npad / 128; ++i) {
                    j0[t0 + i] = (R[k] / 128 + i) >> sh;
                    j1[t0 + i] = (R[k] + npad) / (uint32_t)w;
                }
            }
            off[0] = 0;
            for (uint32_t I = 0; I < nrt; ++I) off[I + 1] = off[I] + (j1[I] - j0[I]);
            nlist = off[nrt];
            uint32_t* d_list = (uint32_t*)ctx_scratch(ctx, "bt.list", std::max<uint64_t>(nlist, 1) * 4);
            if (!d_list) return MDET_ERR_NOMEM;
            MDET_CUDA(ctx, cudaMemcpyAsync(d_j0, j0.data(), nrt * 4, cudaMemcpyHostToDevice, s));
            MDET_CUDA(ctx, cudaMemcpyAsync(d_j1, j1.data(), nrt * 4, cudaMemcpyHostToDevice, s));
            MDET_CUDA(ctx, cudaMemcpyAsync(d_off, off.data(), nrt * 8, cudaMemcpyHostToDevice, s));
            k_tile_list<<<nrt, 128, 0, s>>>(d_j0, d_j1, d_off, (uint32_t)(N / w), d_list);
            MDET_LAUNCHED(ctx, "k_tile_list");
            return run_filter(ctx, mode, g, false, nullptr, nullptr, nullptr, 0, nullptr, nullptr, tbl, "bt", &cand,
                              &ncand, d_list, nlist, d_rtbl, MDET_TBL_FLOATS, w);
        };
        if (bf16)
            MDET_TRY(tc_autotune(ctx, tc_shape_key(false, true, N, N), run, true));
        else
            MDET_TRY(run(128));
        Edge* edges = nullptr;
        unsigned long long ne = 0;
        uint32_t* deg = nullptr;
        MDET_TRY(exact_graph(ctx, g, cand, ncand, 0.0, &edges, &ne, &deg, d_bcut));
        uint64_t total = 0;
        MDET_TRY(select_topk(ctx, g, edges, ne, deg, maxK, &total, d_bK));

        // per-assembly edge counts, capacities, outputs
        const unsigned long long* outptr = (const unsigned long long*)ctx->bufs["tk.outptr"].p;
        k_batch_ends<<<(count + 127) / 128, 128, 0, s>>>(g.ls, outptr, dR, dn, count, drange, douts);
        MDET_LAUNCHED(ctx, "k_batch_ends");
        std::vector<unsigned long long> outs(2 * count);
        MDET_CUDA(ctx, cudaMemcpyAsync(outs.data(), douts, count * 16, cudaMemcpyDeviceToHost, s));
        MDET_CUDA(ctx, cudaStreamSynchronize(s));
        std::vector<BatchOut> bo(count);
        int status = MDET_OK;
        for (uint32_t k = 0; k < count; ++k) {
            mdet_assembly& a = as[k];
            const uint64_t ek = nn[k] ? outs[2 * k + 1] - outs[2 * k] : 0;
            a.n_edges = ek;
            bo[k].from = a.d_from;
            bo[k].to = a.d_to;
            bo[k].stnf = a.d_stnf;
            bo[k].out0 = outs[2 * k];
            bo[k].R = R[k];
            bo[k].n = nn[k];
            bo[k].pad = 0;
            bo[k].emit = ek > 0;
            if (ek > a.capacity) {
                a.status = MDET_ERR_CAPACITY;
                bo[k].emit = 0;
                status = ctx_fail(ctx, MDET_ERR_CAPACITY, "assembly %u needs %llu edge entries, capacity %llu", k,
                                  (unsigned long long)ek, (unsigned long long)a.capacity);
            } else if (ek && (!a.d_from || !a.d_to || !a.d_stnf)) {
                a.status = MDET_ERR_INVALID;
                bo[k].emit = 0;
                status = ctx_fail(ctx, MDET_ERR_INVALID, "assembly %u: null output pointer", k);
            }
        }
        BatchOut* d_bo = (BatchOut*)ctx_scratch(ctx, "bt.bo", count * sizeof(BatchOut));
        if (!d_bo) return MDET_ERR_NOMEM;
        MDET_CUDA(ctx, cudaMemcpyAsync(d_bo, bo.data(), count * sizeof(BatchOut), cudaMemcpyHostToDevice, s));
        if (total) {
            const unsigned long long* rowptr = (const unsigned long long*)ctx->bufs["tk.rowptr"].p;
            const Ent* list = (const Ent*)ctx->bufs["tk.list"].p;
            const unsigned blocks = (unsigned)std::min<uint64_t>((N + 7) / 8, (uint64_t)ctx->num_sms * 32);
            k_emit_batch<<<blocks, 256, 0, s>>>(g.inv, rowptr, list, outptr, d_bA, d_bo, (uint32_t)N);
            MDET_LAUNCHED(ctx, "k_emit_batch");
        }
        if (stats) {
            stats->n_candidates = ncand;
            stats->n_above_cutoff = ne;
            stats->n_edges = total;
            stats->tiles_total = nlist;
            stats->tiles_computed = nlist;
            stats->tile_m_n = (uint32_t)ctx->last_tile_n;
        }
        return status;
    };
    rc = body();
    cudaEventRecord(e1, s);
    if (rc == MDET_OK || rc == MDET_ERR_CAPACITY) {
        const int frc = check_flag(ctx);
        if (frc != MDET_OK) rc = frc;
    }
    if (stats) {
        float ms = 0;
        cudaEventSynchronize(e1);
        cudaEventElapsedTime(&ms, e0, e1);
        stats->ms_total = ms;
        stats->gpu_launches = ctx->launches;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return rc;
}
