// graph_batch.cu -- mdet_tnf_graph_batched: the TNF graphs of many
// independent assemblies in one pass.  The reference builds one graph per
// run (gen_tnf_graph, cuda/Cuda2.cu:861-970); here every assembly's prepared
// rows are laid end to end (each padded to 256 rows, so no tile straddles two
// assemblies), one tile list covers the upper triangles of all of them, and
// a single persistent filter launch, one exact-stage launch and one selection
// launch serve the whole batch.  Per-assembly cutoffs and max_edges ride along
// as per-block side tables; outputs go to each assembly's own buffers.
//
// A batch that comes back with the same shapes and buffers is recorded once
// as a CUDA graph -- preparation, d* tables, filter, exact stage, selection
// and output, with every count kept on the device -- and later calls replay
// it with one launch.
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
    unsigned long long capacity;
    uint32_t R, n;  // first row, contigs
    int pad[2];
};

// Block per row tile I: its column tiles [j0[I], j1[I]) as I * tcols + J.
__global__ void k_tile_list(const uint32_t* __restrict__ j0, const uint32_t* __restrict__ j1,
                            const unsigned long long* __restrict__ off, uint32_t tcols, uint32_t* __restrict__ list) {
    const uint32_t I = blockIdx.x;
    const uint32_t a = j0[I], b = j1[I];
    const unsigned long long o = off[I];
    for (uint32_t J = a + threadIdx.x; J < b; J += blockDim.x) list[o + (J - a)] = I * tcols + J;
}

// Log-size ranges of every assembly (the prepared rows are ascending per
// assembly; empty assemblies give lo > hi) and, with outptr, the output range.
__global__ void k_batch_ends(const double* __restrict__ ls, const unsigned long long* __restrict__ outptr,
                             const uint32_t* __restrict__ R, const uint32_t* __restrict__ n, uint32_t count,
                             double* __restrict__ range, unsigned long long* __restrict__ outs) {
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= count) return;
    if (n[k] == 0) {
        range[2 * k] = 1.0;
        range[2 * k + 1] = 0.0;
        if (outptr) outs[2 * k] = outs[2 * k + 1] = 0;
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
// selection, go to its assembly's outputs with local indices -- unless the
// assembly's edges exceed its capacity, which its first row records.
__global__ void k_emit_batch(const uint32_t* __restrict__ inv, const unsigned long long* __restrict__ rowptr,
                             const Ent* __restrict__ list, const unsigned long long* __restrict__ outptr,
                             const uint32_t* __restrict__ blk_asm, const BatchOut* __restrict__ outs, uint32_t N,
                             int* __restrict__ status) {
    const uint32_t lane = threadIdx.x & 31;
    for (uint32_t o = blockIdx.x * (blockDim.x / 32) + (threadIdx.x >> 5); o < N; o += gridDim.x * (blockDim.x / 32)) {
        const uint32_t a = blk_asm[o >> 8];
        const BatchOut bo = outs[a];
        if (o - bo.R >= bo.n) continue;
        const unsigned long long base = outptr[bo.R];
        const unsigned long long total = outptr[bo.R + bo.n] - base;
        if (total > bo.capacity) {
            if (o == bo.R && lane == 0) status[a] = MDET_ERR_CAPACITY;
            continue;
        }
        const uint32_t s = inv[o];
        const unsigned long long p0 = outptr[o];
        const uint32_t cnt = (uint32_t)(outptr[o + 1] - p0);
        const Ent* row = list + rowptr[s];
        for (uint32_t i = lane; i < cnt; i += 32) {
            const Ent x = row[i];
            const unsigned long long q = p0 - base + i;
            bo.from[q] = o - bo.R;
            bo.to[q] = x.ocol - bo.R;
            bo.stnf[q] = x.sim;
        }
    }
}

// The shapes, pointers and options that a recorded batch depends on.
std::vector<uint64_t> batch_key(const mdet_assembly* as, uint32_t count, int mode) {
    std::vector<uint64_t> k;
    k.reserve(9 * count + 2);
    k.push_back((uint64_t)mode);
    k.push_back(count);
    for (uint32_t i = 0; i < count; ++i) {
        const mdet_assembly& a = as[i];
        uint64_t cut;
        memcpy(&cut, &a.cutoff, 8);
        k.push_back((uint64_t)(uintptr_t)a.d_tnf);
        k.push_back((uint64_t)(uintptr_t)a.d_log_size);
        k.push_back(a.n);
        k.push_back(cut);
        k.push_back(a.max_edges);
        k.push_back((uint64_t)(uintptr_t)a.d_from);
        k.push_back((uint64_t)(uintptr_t)a.d_to);
        k.push_back((uint64_t)(uintptr_t)a.d_stnf);
        k.push_back(a.capacity);
    }
    return k;
}

struct BatchPlan {
    std::vector<uint64_t> key;
    unsigned long long cand_cap = 0;
    int shape = 0;
    uint64_t scratch_gen = 0;
    cudaGraphExec_t exec = nullptr;
    uint32_t launches = 0;
    uint64_t nlist = 0;
};

void plan_free(void* p) {
    BatchPlan* bp = (BatchPlan*)p;
    if (!bp) return;
    if (bp->exec) cudaGraphExecDestroy(bp->exec);
    delete bp;
}

// Everything a pass needs that depends only on the batch's shapes.
struct Layout {
    uint32_t count = 0;
    std::vector<uint32_t> R, nn;
    uint64_t N = 0;
    uint32_t nblk256 = 0, nrt = 0, maxK = 1;
    std::map<double, uint32_t> tab_of;  // distinct cutoff -> table index
};

struct Dev {
    uint32_t *R, *n, *bK, *bA, *j0, *j1, *list;
    unsigned long long *off, *outs;
    double* range;
    uint8_t* rtbl;
    BlkCut* bcut;
    BatchOut* bo;
    int* status;
    float* tbl;
    TableGrid* grid;
};

// Side tables of a layout in scratch (uploaded from the host).
int upload_sides(mdet_ctx* ctx, const mdet_assembly* as, const Layout& L, Dev& d) {
    cudaStream_t s = ctx->stream;
    const uint32_t count = L.count;
    d.R = (uint32_t*)ctx_scratch(ctx, "bt.R", count * 4);
    d.n = (uint32_t*)ctx_scratch(ctx, "bt.n", count * 4);
    d.range = (double*)ctx_scratch(ctx, "bt.range", count * 16);
    d.outs = (unsigned long long*)ctx_scratch(ctx, "bt.outs", count * 16);
    d.rtbl = (uint8_t*)ctx_scratch(ctx, "bt.rtbl", L.nrt);
    d.bcut = (BlkCut*)ctx_scratch(ctx, "bt.bcut", (uint64_t)L.nblk256 * sizeof(BlkCut));
    d.bK = (uint32_t*)ctx_scratch(ctx, "bt.bK", (uint64_t)L.nblk256 * 4);
    d.bA = (uint32_t*)ctx_scratch(ctx, "bt.bA", (uint64_t)L.nblk256 * 4);
    d.j0 = (uint32_t*)ctx_scratch(ctx, "bt.j0", (uint64_t)L.nrt * 4);
    d.j1 = (uint32_t*)ctx_scratch(ctx, "bt.j1", (uint64_t)L.nrt * 4);
    d.off = (unsigned long long*)ctx_scratch(ctx, "bt.off", ((uint64_t)L.nrt + 1) * 8);
    d.bo = (BatchOut*)ctx_scratch(ctx, "bt.bo", count * sizeof(BatchOut));
    d.status = (int*)ctx_scratch(ctx, "bt.status", count * 4);
    d.tbl = (float*)ctx_scratch(ctx, "bt.tbl", L.tab_of.size() * MDET_TBL_FLOATS * 4);
    d.grid = (TableGrid*)ctx_scratch(ctx, "bt.grid", sizeof(TableGrid));
    if (!d.R || !d.n || !d.range || !d.outs || !d.rtbl || !d.bcut || !d.bK || !d.bA || !d.j0 || !d.j1 || !d.off ||
        !d.bo || !d.status || !d.tbl || !d.grid)
        return MDET_ERR_NOMEM;
    std::vector<uint8_t> row_tbl(L.nrt, 0);
    std::vector<BlkCut> bcut(L.nblk256);
    std::vector<uint32_t> bK(L.nblk256, 1), bA(L.nblk256, 0);
    std::vector<BatchOut> bo(count);
    for (uint32_t k = 0; k < count; ++k) {
        bo[k].from = as[k].d_from;
        bo[k].to = as[k].d_to;
        bo[k].stnf = as[k].d_stnf;
        bo[k].capacity = as[k].capacity;
        bo[k].R = L.R[k];
        bo[k].n = L.nn[k];
        bo[k].pad[0] = bo[k].pad[1] = 0;
        const uint32_t npad = (L.nn[k] + 255) / 256 * 256;
        if (!npad) continue;
        const double Lc = logit(as[k].cutoff);
        BlkCut bc;
        bc.L.hi = (float)Lc;
        bc.L.lo = (float)(Lc - (double)bc.L.hi);
        bc.model2 = Lc < 2.1972245773362196 ? 1u : 0u;  // ln 9
        bc.pad = 0;
        for (uint32_t b = L.R[k] / 256; b < (L.R[k] + npad) / 256; ++b) {
            bcut[b] = bc;
            bK[b] = as[k].max_edges;
            bA[b] = k;
        }
        const uint8_t t = (uint8_t)L.tab_of.at(as[k].cutoff);
        for (uint32_t i = 0; i < npad / 128; ++i) row_tbl[L.R[k] / 128 + i] = t;
    }
    MDET_CUDA(ctx, cudaMemcpyAsync(d.R, L.R.data(), count * 4, cudaMemcpyHostToDevice, s));
    MDET_CUDA(ctx, cudaMemcpyAsync(d.n, L.nn.data(), count * 4, cudaMemcpyHostToDevice, s));
    MDET_CUDA(ctx, cudaMemcpyAsync(d.rtbl, row_tbl.data(), L.nrt, cudaMemcpyHostToDevice, s));
    MDET_CUDA(ctx, cudaMemcpyAsync(d.bcut, bcut.data(), L.nblk256 * sizeof(BlkCut), cudaMemcpyHostToDevice, s));
    MDET_CUDA(ctx, cudaMemcpyAsync(d.bK, bK.data(), L.nblk256 * 4, cudaMemcpyHostToDevice, s));
    MDET_CUDA(ctx, cudaMemcpyAsync(d.bA, bA.data(), L.nblk256 * 4, cudaMemcpyHostToDevice, s));
    MDET_CUDA(ctx, cudaMemcpyAsync(d.bo, bo.data(), count * sizeof(BatchOut), cudaMemcpyHostToDevice, s));
    // the host vectors die here: wait for the copies
    MDET_CUDA(ctx, cudaStreamSynchronize(s));
    return MDET_OK;
}

// The tile list for column tiles of width w (upper triangle of every assembly).
int build_list(mdet_ctx* ctx, const Layout& L, Dev& d, int w, uint64_t* nlist) {
    cudaStream_t s = ctx->stream;
    std::vector<uint32_t> j0(L.nrt), j1(L.nrt);
    std::vector<unsigned long long> off(L.nrt + 1);
    const uint32_t sh = w == 256 ? 1u : 0u;
    for (uint32_t k = 0; k < L.count; ++k) {
        const uint32_t npad = (L.nn[k] + 255) / 256 * 256;
        const uint32_t t0 = L.R[k] / 128;
        for (uint32_t i = 0; i < npad / 128; ++i) {
            j0[t0 + i] = (t0 + i) >> sh;
            j1[t0 + i] = (L.R[k] + npad) / (uint32_t)w;
        }
    }
    off[0] = 0;
    for (uint32_t I = 0; I < L.nrt; ++I) off[I + 1] = off[I] + (j1[I] - j0[I]);
    *nlist = off[L.nrt];
    d.list = (uint32_t*)ctx_scratch(ctx, "bt.list", std::max<uint64_t>(*nlist, 1) * 4);
    if (!d.list) return MDET_ERR_NOMEM;
    MDET_CUDA(ctx, cudaMemcpyAsync(d.j0, j0.data(), L.nrt * 4, cudaMemcpyHostToDevice, s));
    MDET_CUDA(ctx, cudaMemcpyAsync(d.j1, j1.data(), L.nrt * 4, cudaMemcpyHostToDevice, s));
    MDET_CUDA(ctx, cudaMemcpyAsync(d.off, off.data(), ((uint64_t)L.nrt + 1) * 8, cudaMemcpyHostToDevice, s));
    k_tile_list<<<L.nrt, 128, 0, s>>>(d.j0, d.j1, d.off, (uint32_t)(L.N / w), d.list);
    MDET_LAUNCHED(ctx, "k_tile_list");
    MDET_CUDA(ctx, cudaStreamSynchronize(s));  // the host arrays die here
    return MDET_OK;
}

// Preparation and d* tables of every assembly; no host synchronisation.
int prep_and_tables(mdet_ctx* ctx, const mdet_assembly* as, const Layout& L, bool bf16, Dev& d, GraphPrep& g,
                    DstarTable* tbl) {
    MDET_TRY(prep_alloc(ctx, "bt", L.N, bf16, &g));
    g.n = (uint32_t)L.N;
    g.npad = (uint32_t)L.N;
    for (uint32_t k = 0; k < L.count; ++k)
        if (L.nn[k]) MDET_TRY(prep_into(ctx, as[k].d_tnf, as[k].d_log_size, L.nn[k], bf16, g, L.R[k]));
    k_batch_ends<<<(L.count + 127) / 128, 128, 0, ctx->stream>>>(g.ls, nullptr, d.R, d.n, L.count, d.range, d.outs);
    MDET_LAUNCHED(ctx, "k_batch_ends");
    MDET_TRY(grid_from_ranges(ctx, d.range, L.count, d.grid));
    for (auto& kv : L.tab_of)
        MDET_TRY(build_dstar_table_dev(ctx, d.grid, logit(kv.first), d.tbl + kv.second * MDET_TBL_FLOATS, tbl));
    tbl->st = d.tbl;
    return MDET_OK;
}

// Outputs of the pass: per-assembly output ranges, statuses, and the edges.
int emit_pass(mdet_ctx* ctx, const Layout& L, Dev& d, const GraphPrep& g) {
    cudaStream_t s = ctx->stream;
    const unsigned long long* outptr = (const unsigned long long*)ctx->bufs["tk.outptr"].p;
    const unsigned long long* rowptr = (const unsigned long long*)ctx->bufs["tk.rowptr"].p;
    const Ent* list = (const Ent*)ctx->bufs["tk.list"].p;
    k_batch_ends<<<(L.count + 127) / 128, 128, 0, s>>>(g.ls, outptr, d.R, d.n, L.count, d.range, d.outs);
    MDET_LAUNCHED(ctx, "k_batch_ends");
    MDET_CUDA(ctx, cudaMemsetAsync(d.status, 0, L.count * 4, s));
    const unsigned blocks = (unsigned)std::min<uint64_t>((L.N + 7) / 8, (uint64_t)ctx->num_sms * 32);
    k_emit_batch<<<blocks, 256, 0, s>>>(g.inv, rowptr, list, outptr, d.bA, d.bo, (uint32_t)L.N, d.status);
    MDET_LAUNCHED(ctx, "k_emit_batch");
    return MDET_OK;
}

// The whole batch with every count on the device: what a CUDA graph records.
int device_pass(mdet_ctx* ctx, const mdet_assembly* as, const Layout& L, int mode, Dev& d, uint64_t nlist, int shape,
                unsigned long long cap) {
    GraphPrep g;
    DstarTable tbl;
    MDET_TRY(prep_and_tables(ctx, as, L, mode == MDET_MODE_BF16, d, g, &tbl));
    uint2* cand = nullptr;
    unsigned long long ncap = 0, *ncand_dev = nullptr, *ne_dev = nullptr;
    MDET_TRY(run_filter(ctx, mode, g, false, nullptr, nullptr, nullptr, 0, nullptr, nullptr, tbl, "bt", &cand, &ncap,
                        d.list, nlist, d.rtbl, MDET_TBL_FLOATS, shape, cap, &ncand_dev, d.off));
    Edge* edges = nullptr;
    unsigned long long ecap = 0;
    uint32_t* deg = nullptr;
    MDET_TRY(exact_graph(ctx, g, cand, cap, 0.0, &edges, &ecap, &deg, d.bcut, ncand_dev, &ne_dev));
    uint64_t total = 0;
    MDET_TRY(select_topk(ctx, g, edges, ecap, deg, L.maxK, &total, d.bK, ne_dev));
    return emit_pass(ctx, L, d, g);
}

// Sizing run, then recording, of a batch; returns the plan or null.
BatchPlan* record(mdet_ctx* ctx, const mdet_assembly* as, const Layout& L, int mode, Dev& d, int shape,
                  unsigned long long ncand, const std::vector<uint64_t>& key) {
    cudaStream_t s = ctx->stream;
    uint64_t nlist = 0;
    if (build_list(ctx, L, d, shape ? shape : 128, &nlist) != MDET_OK) return nullptr;
    BatchPlan* np = new BatchPlan();
    np->key = key;
    np->cand_cap = ncand + ncand / 4 + 65536;
    np->shape = shape;
    np->nlist = nlist;
    int exact = 8;
    auto ex = ctx->exact_shape.find(tc_shape_key(false, false, ncand, L.N));
    if (ex != ctx->exact_shape.end()) exact = ex->second;
    const int saved_exact = ctx->forced_exact;
    const bool saved_timing = ctx->timing;
    ctx->forced_exact = exact;
    ctx->timing = false;
    // every buffer reaches its final size outside the recording
    int rc = device_pass(ctx, as, L, mode, d, nlist, shape, np->cand_cap);
    if (rc == MDET_OK) rc = ctx_cuda(ctx, cudaStreamSynchronize(s), "sizing pass");
    cudaGraph_t graph = nullptr;
    // the recording is captured on the context's own capture stream: the
    // caller's stream may be the legacy default stream, which cannot be
    // captured; the graph is launched on the caller's stream later
    if (rc == MDET_OK && !ctx->cap_stream)
        rc = ctx_cuda(ctx, cudaStreamCreateWithFlags(&ctx->cap_stream, cudaStreamNonBlocking), "capture stream");
    if (rc == MDET_OK) {
        const uint32_t l0 = ctx->launches;
        const cudaStream_t cs = ctx->cap_stream;
        rc = ctx_cuda(ctx, cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal), "begin capture");
        if (rc == MDET_OK) {
            ctx->capturing = true;
            ctx->stream = cs;
            const int crc = device_pass(ctx, as, L, mode, d, nlist, shape, np->cand_cap);
            ctx->stream = s;
            ctx->capturing = false;
            const cudaError_t ce = cudaStreamEndCapture(cs, &graph);
            if (crc == MDET_OK && ce == cudaSuccess && graph) {
                rc = ctx_cuda(ctx, cudaGraphInstantiate(&np->exec, graph, 0), "graph instantiate");
                np->launches = ctx->launches - l0;
            } else {
                cudaGetLastError();
                rc = MDET_ERR_CUDA;
            }
        }
    }
    if (graph) cudaGraphDestroy(graph);
    ctx->forced_exact = saved_exact;
    ctx->timing = saved_timing;
    if (rc != MDET_OK || !np->exec) {
        plan_free(np);
        return nullptr;
    }
    np->scratch_gen = ctx->scratch_gen;
    return np;
}

}  // namespace

extern "C" int mdet_ctx_set_graph_capture(mdet_ctx* ctx, int enable) {
    if (!ctx) return MDET_ERR_INVALID;
    ctx->graph_capture = enable != 0;
    if (!ctx->graph_capture && ctx->batch_plan) {
        plan_free(ctx->batch_plan);
        ctx->batch_plan = nullptr;
    }
    return MDET_OK;
}

extern "C" uint64_t mdet_ctx_graph_replays(mdet_ctx* ctx) { return ctx ? ctx->graph_replays : 0; }

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
    Layout L;
    L.count = count;
    L.R.resize(count);
    L.nn.resize(count);
    for (uint32_t k = 0; k < count; ++k) {
        mdet_assembly& a = as[k];
        a.status = MDET_OK;
        a.n_edges = 0;
        if (!(a.cutoff > 0.0 && a.cutoff < 1.0))
            return ctx_fail(ctx, MDET_ERR_INVALID, "assembly %u: cutoff must lie in (0, 1)", k);
        if (a.max_edges == 0 || a.max_edges > 512)
            return ctx_fail(ctx, MDET_ERR_INVALID, "assembly %u: max_edges must be in [1, 512] in a batch", k);
        if (a.n >= (1ull << 31)) return ctx_fail(ctx, MDET_ERR_INVALID, "assembly %u: too many contigs", k);
        if (a.n >= 2 && (!a.d_tnf || !a.d_log_size))
            return ctx_fail(ctx, MDET_ERR_INVALID, "assembly %u: null input pointer", k);
        if (a.n >= 2 && a.capacity && (!a.d_from || !a.d_to || !a.d_stnf))
            return ctx_fail(ctx, MDET_ERR_INVALID, "assembly %u: null output pointer", k);
        L.nn[k] = a.n >= 2 ? (uint32_t)a.n : 0;
        L.R[k] = (uint32_t)L.N;
        L.N += (L.nn[k] + 255) / 256 * 256;
        L.maxK = std::max(L.maxK, a.max_edges);
        if (L.nn[k] && !L.tab_of.count(a.cutoff)) {
            const uint32_t id = (uint32_t)L.tab_of.size();
            L.tab_of[a.cutoff] = id;
        }
    }
    if (L.N == 0) return MDET_OK;
    if (L.N >= (1ull << 31))
        return ctx_fail(ctx, MDET_ERR_INVALID, "batch too large (%llu rows)", (unsigned long long)L.N);
    if (L.tab_of.size() > 255) return ctx_fail(ctx, MDET_ERR_INVALID, "more than 255 distinct cutoffs in a batch");
    L.nblk256 = (uint32_t)(L.N / 256);
    L.nrt = (uint32_t)(L.N / 128);
    if ((uint64_t)L.nrt * L.nrt >= (1ull << 32))
        return ctx_fail(ctx, MDET_ERR_INVALID, "batch too large for the tile list");

    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventRecord(e0, s);
    std::vector<uint64_t> key;
    if (ctx->graph_capture) key = batch_key(as, count, mode);
    BatchPlan* plan = (BatchPlan*)ctx->batch_plan;
    Dev d;
    memset(&d, 0, sizeof(d));

    // per-assembly results from the device: output ranges and capacities
    auto collect = [&](unsigned long long ncand, unsigned long long ne) -> int {
        std::vector<unsigned long long> outs(2 * count);
        MDET_CUDA(ctx, cudaMemcpyAsync(outs.data(), d.outs, count * 16, cudaMemcpyDeviceToHost, s));
        MDET_CUDA(ctx, cudaStreamSynchronize(s));
        int status = MDET_OK;
        uint64_t total = 0;
        for (uint32_t k = 0; k < count; ++k) {
            const uint64_t ek = L.nn[k] ? outs[2 * k + 1] - outs[2 * k] : 0;
            as[k].n_edges = ek;
            total += ek;
            if (ek > as[k].capacity) {
                as[k].status = MDET_ERR_CAPACITY;
                status = ctx_fail(ctx, MDET_ERR_CAPACITY, "assembly %u needs %llu edge entries, capacity %llu", k,
                                  (unsigned long long)ek, (unsigned long long)as[k].capacity);
            }
        }
        if (stats) {
            stats->n_candidates = ncand;
            stats->n_above_cutoff = ne;
            stats->n_edges = total;
        }
        return status;
    };

    int rc = MDET_OK;
    bool done = false;
    // replay of a recorded batch
    if (ctx->graph_capture && plan && plan->key == key && plan->scratch_gen == ctx->scratch_gen) {
        MDET_CUDA(ctx, cudaGraphLaunch(plan->exec, s));
        ctx->graph_replays++;
        ctx->launches += plan->launches;
        ctx->total_launches += plan->launches;
        unsigned long long cnt[2] = {0, 0};
        MDET_CUDA(ctx, cudaMemcpyAsync(&cnt[0], ctx->bufs["flt.cnt"].p, 8, cudaMemcpyDeviceToHost, s));
        MDET_CUDA(ctx, cudaMemcpyAsync(&cnt[1], ctx->bufs["ex.cnt"].p, 8, cudaMemcpyDeviceToHost, s));
        MDET_CUDA(ctx, cudaStreamSynchronize(s));
        if (cnt[0] <= plan->cand_cap) {
            d.outs = (unsigned long long*)ctx->bufs["bt.outs"].p;
            rc = collect(cnt[0], cnt[1]);
            if (stats) {
                stats->tiles_total = stats->tiles_computed = plan->nlist;
                stats->tile_m_n = plan->shape == 128 ? 128128 : 128256;
            }
            done = true;
        } else {  // more candidates than the recording holds: the sized path below, recorded again
            plan_free(plan);
            ctx->batch_plan = plan = nullptr;
        }
    }

    if (!done) {
        // the side tables in scratch are about to change: a recording of another batch is stale
        if (ctx->batch_plan) {
            plan_free(ctx->batch_plan);
            ctx->batch_plan = plan = nullptr;
        }
        auto body = [&]() -> int {
            MDET_TRY(upload_sides(ctx, as, L, d));
            GraphPrep g;
            DstarTable tbl;
            MDET_TRY(prep_and_tables(ctx, as, L, bf16, d, g, &tbl));
            // one filter launch over every assembly's tiles, one exact stage, one selection
            uint64_t nlist = 0;
            uint2* cand = nullptr;
            unsigned long long ncand = 0;
            auto run = [&](int w) -> int {
                MDET_TRY(build_list(ctx, L, d, w, &nlist));
                return run_filter(ctx, mode, g, false, nullptr, nullptr, nullptr, 0, nullptr, nullptr, tbl, "bt",
                                  &cand, &ncand, d.list, nlist, d.rtbl, MDET_TBL_FLOATS, w, 0, nullptr, d.off);
            };
            if (bf16)
                MDET_TRY(tc_autotune(ctx, tc_shape_key(false, true, L.N, L.N), run, true));
            else
                MDET_TRY(run(128));
            Edge* edges = nullptr;
            unsigned long long ne = 0;
            uint32_t* deg = nullptr;
            MDET_TRY(exact_graph(ctx, g, cand, ncand, 0.0, &edges, &ne, &deg, d.bcut));
            uint64_t total = 0;
            MDET_TRY(select_topk(ctx, g, edges, ne, deg, L.maxK, &total, d.bK));
            MDET_TRY(emit_pass(ctx, L, d, g));
            const int status = collect(ncand, ne);
            if (stats) {
                stats->tiles_total = nlist;
                stats->tiles_computed = nlist;
                stats->tile_m_n = (uint32_t)ctx->last_tile_n;
            }
            if (status != MDET_OK && status != MDET_ERR_CAPACITY) return status;
            // record the batch for later calls with the same shapes and buffers;
            // recording is an optimisation, the results above stand either way
            if (ctx->graph_capture) {
                const std::string err = ctx->err;
                int shape = 0;
                if (bf16) {
                    const int t = ctx->last_tile_n;  // the shape of the pass whose output stands
                    auto it = ctx->tc_shape.find(tc_shape_key(false, true, L.N, L.N));
                    shape = it != ctx->tc_shape.end() ? it->second : (t == 128128 ? 128 : 256);
                }
                BatchPlan* np = record(ctx, as, L, mode, d, shape, ncand, key);
                ctx->err = err;
                if (np) {
                    if (ctx->batch_plan) plan_free(ctx->batch_plan);
                    ctx->batch_plan = np;
                    ctx->batch_plan_free = plan_free;
                }
            }
            return status;
        };
        rc = body();
    }
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
