// ctx.cu -- context lifetime, scratch arena, status handling, canonical
// tables and the split form of the MetaBAT2 logistic model.
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <limits>

#include "common.cuh"

// ------------------------------------------------------------ status ------

int ctx_fail(mdet_ctx* ctx, int code, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    if (ctx) ctx->err = buf;
    return code;
}

int ctx_cuda(mdet_ctx* ctx, cudaError_t e, const char* what) {
    if (e == cudaSuccess) return MDET_OK;
    cudaGetLastError();  // clear a non-sticky error
    return ctx_fail(ctx, e == cudaErrorMemoryAllocation ? MDET_ERR_NOMEM : MDET_ERR_CUDA, "%s: %s", what,
                    cudaGetErrorString(e));
}

int ctx_check_launch(mdet_ctx* ctx, const char* what) { return ctx_cuda(ctx, cudaGetLastError(), what); }

void ctx_timer_begin(mdet_ctx* ctx, const char* kernel) {
    if (!ctx->timing) return;
    cudaEvent_t a, b;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    cudaEventRecord(a, ctx->stream);
    ctx->timers[kernel].ev.push_back({a, b});
}

void ctx_timer_end(mdet_ctx* ctx, const char* kernel) {
    if (!ctx->timing) return;
    auto it = ctx->timers.find(kernel);
    if (it == ctx->timers.end() || it->second.ev.empty()) return;
    cudaEventRecord(it->second.ev.back().second, ctx->stream);
}

static void timers_clear(mdet_ctx* ctx) {
    for (auto& kv : ctx->timers)
        for (auto& e : kv.second.ev) {
            cudaEventDestroy(e.first);
            cudaEventDestroy(e.second);
        }
    ctx->timers.clear();
}

void* ctx_scratch(mdet_ctx* ctx, const char* name, size_t bytes, bool zero_on_grow) {
    if (bytes == 0) bytes = 16;
    DevBuf& b = ctx->bufs[name];
    if (b.cap >= bytes) return b.p;
    if (ctx->capturing) {  // a captured pass must not move its buffers
        ctx_fail(ctx, MDET_ERR_NOMEM, "scratch %s would grow while a pass is captured", name);
        return nullptr;
    }
    ++ctx->scratch_gen;  // captured passes that used the old buffer are stale now
    if (b.p) {
        cudaStreamSynchronize(ctx->stream);
        cudaFree(b.p);
        b.p = nullptr;
        b.cap = 0;
    }
    size_t cap = bytes + bytes / 8;  // headroom so slowly growing inputs do not thrash
    cap = (cap + 4095) & ~(size_t)4095;
    if (cudaMalloc(&b.p, cap) != cudaSuccess) {
        cudaGetLastError();
        if (cudaMalloc(&b.p, bytes) != cudaSuccess) {
            cudaGetLastError();
            b.p = nullptr;
            ctx_fail(ctx, MDET_ERR_NOMEM, "device allocation of %zu bytes for %s failed", bytes, name);
            return nullptr;
        }
        cap = bytes;
    }
    b.cap = cap;
    if (zero_on_grow) cudaMemsetAsync(b.p, 0, cap, ctx->stream);
    return b.p;
}

void* ctx_pinned(mdet_ctx* ctx, size_t bytes) {
    if (ctx->pinned_cap >= bytes) return ctx->pinned;
    if (ctx->pinned) {
        cudaStreamSynchronize(ctx->stream);
        cudaFreeHost(ctx->pinned);
        ctx->pinned = nullptr;
        ctx->pinned_cap = 0;
    }
    if (cudaMallocHost(&ctx->pinned, bytes) != cudaSuccess) {
        cudaGetLastError();
        ctx->pinned = nullptr;
        ctx_fail(ctx, MDET_ERR_NOMEM, "pinned host allocation of %zu bytes failed", bytes);
        return nullptr;
    }
    ctx->pinned_cap = bytes;
    return ctx->pinned;
}

// ------------------------------------------------------------ tables ------

namespace {
// Column order of the canonical tetranucleotides: the TNF.bin layout of the
// reference (openmp/TNF.cpp:14-24); kept because it is the output format.
const char kTnOrder[] =
    "GGTAAGCCAAAAACATAGTCACGACATACGAAAAGTCAAACCAGGGACATTAGATCCCTCCTAAACTAAGGCGCAACCGCCGCCAAAC"
    "ACTCATCCGACCGAGAATAGATCACAGAAGTAATGAAAATTTAATATAAGTGAGCTCCACGGCCACCCGGGAGCGCATACCTGATAGA"
    "ATATGTCACTCCACAAACCTTAAAAACGCGAGAGGGATCGACGCTCAACTACCTCAGACAGGAACTTCGCCCCTGCTGCAGGCACACG"
    "GAGCAACTCATGAATTACAGAGATATAACATCGCCATCGACACACAACAAGGAGCAATGGATTCGTGAACCGGATAGCTACGTCCCCG"
    "AAGCCGTAGTACAGGAAATGCACCCAGCCGGCACACCCGGCCGACCCCTGAAAACAAGAGCCCACGGATACAACCAACGTGAACGTAA"
    "ATGCGTTATCCACAGGACTGAAAGAAGACAAGGCGAAACCACGGCCAACTTAAGACAGCGGAAAAATCATTGGCACCCTACGACCTAG"
    "AGAACGCACGCGAATA";

int base_of(char c) {
    switch (c) {
        case 'A': return 0;
        case 'C': return 1;
        case 'T': return 2;
        default: return 3;  // 'G'
    }
}
int comp_code(int b) { return b == 0 ? 2 : b == 2 ? 0 : b == 1 ? 3 : 1; }  // A<->T, C<->G

TnTables build_tables() {
    TnTables t;
    for (int col = 0; col < MDET_NTNF; ++col) {
        int fw = 0, rc = 0;
        for (int p = 0; p < 4; ++p) fw = (fw << 2) | base_of(kTnOrder[4 * col + p]);
        for (int p = 3; p >= 0; --p) rc = (rc << 2) | comp_code(base_of(kTnOrder[4 * col + p]));
        t.col_fw[col] = (uint8_t)fw;
        t.col_rc[col] = (uint8_t)rc;
    }
    for (int code = 0; code < 256; ++code) t.raw_to_col[code] = 255;
    for (int col = 0; col < MDET_NTNF; ++col) {
        t.raw_to_col[t.col_fw[col]] = (uint8_t)col;
        t.raw_to_col[t.col_rc[col]] = (uint8_t)col;
    }
    return t;
}
}  // namespace

const TnTables& tn_tables() {
    static TnTables t = build_tables();
    return t;
}

// ------------------------------------------------------------ model ------

namespace {
// MetaBAT2 logistic-model coefficients (cuda/Cuda2.cu:170-188); they are the
// model's parameters, identical by necessity.
const double kB1[18] = {46349.1624324381,  -76092.3748553155, -639.918334183,  53873.3933743949, -156.6547554844,
                        -21263.6010657275, 64.7719132839,     5003.2646455284, -8.5014386744,    -700.5825500292,
                        0.3968284526,      54.037542743,      -1.7713972342,   474.0850141891,   -23.966597785,
                        0.7800219061,      -0.0138723693,     0.0001027543};
const double kC1[18] = {-443565.465710869, 718862.10804858, 5114.1630934534,   -501588.206183097, 784.4442123743,
                        194712.394138513,  -377.9645994741, -45088.7863182741, 50.5960513287,     6220.3310639927,
                        -2.3670776453,     -473.269785487,  15.3213264134,     -3282.8510348085,  164.0438603974,
                        -5.2778800755,     0.0929379305,    -0.0006826817};
const double kB2[17] = {6770.9351457442, -5933.7589419767, -2976.2879986855, 3279.7524685865, 1602.7544794819,
                        -967.2906583423, -462.0149190219,  159.8317289682,   74.4884405822,   -14.0267151808,
                        -6.3644917671,   0.5108811613,     0.2252455343,     0.965040193,     -0.0546309127,
                        0.0012917084,    -1.14383e-05};
const double kC2[19] = {39406.5712626297,  -77863.1741143294, 9586.8761567725, 55360.1701572325, -5825.2491611377,
                        -21887.8400068324, 1751.6803621934,   5158.3764225203, -290.1765894829,  -724.0348081819,
                        25.364646181,      56.0522105105,     -0.9172073892,   -1.8470088417,    449.4660736502,
                        -24.4141920625,    0.8465834103,      -0.0158943762,   0.0001235384};

// Regroup each polynomial by variable: x-only monomials into F, y-only into
// G, (x*y)^k into H.  The monomial of every coefficient follows the lw[]
// indices of cuda/Cuda2.cu:202-236.
ModelSplit build_split() {
    ModelSplit s;
    memset(&s, 0, sizeof(s));
    // b1 / c1: 1, x, y, x2, y2, x3, y3, x4, y4, x5, y5, x6, x7, xy, (xy)^2..(xy)^5
    const int fx1[18] = {0, 1, -1, 2, -1, 3, -1, 4, -1, 5, -1, 6, 7, -1, -1, -1, -1, -1};
    const int gy1[18] = {-1, -1, 1, -1, 2, -1, 3, -1, 4, -1, 5, -1, -1, -1, -1, -1, -1, -1};
    const int ht1[18] = {-1, -1, -1, -1, -1, -1, -1, -1, -1, -1, -1, -1, -1, 1, 2, 3, 4, 5};
    for (int k = 0; k < 18; ++k) {
        if (fx1[k] >= 0) { s.F[0][fx1[k]] += kB1[k]; s.F[1][fx1[k]] += kC1[k]; }
        if (gy1[k] >= 0) { s.G[0][gy1[k]] += kB1[k]; s.G[1][gy1[k]] += kC1[k]; }
        if (ht1[k] >= 0) { s.H[0][ht1[k]] += kB1[k]; s.H[1][ht1[k]] += kC1[k]; }
    }
    // b2: 1, x, y, x2, y2, x3, y3, x4, y4, x5, y5, x6, y6, (xy)^2..(xy)^5
    const int fx2[17] = {0, 1, -1, 2, -1, 3, -1, 4, -1, 5, -1, 6, -1, -1, -1, -1, -1};
    const int gy2[17] = {-1, -1, 1, -1, 2, -1, 3, -1, 4, -1, 5, -1, 6, -1, -1, -1, -1};
    const int ht2[17] = {-1, -1, -1, -1, -1, -1, -1, -1, -1, -1, -1, -1, -1, 2, 3, 4, 5};
    for (int k = 0; k < 17; ++k) {
        if (fx2[k] >= 0) s.F[2][fx2[k]] += kB2[k];
        if (gy2[k] >= 0) s.G[2][gy2[k]] += kB2[k];
        if (ht2[k] >= 0) s.H[2][ht2[k]] += kB2[k];
    }
    // c2: 1, x, y, x2, y2, x3, y3, x4, y4, x5, y5, x6, y6, x7, xy, (xy)^2..(xy)^5
    const int fx3[19] = {0, 1, -1, 2, -1, 3, -1, 4, -1, 5, -1, 6, -1, 7, -1, -1, -1, -1, -1};
    const int gy3[19] = {-1, -1, 1, -1, 2, -1, 3, -1, 4, -1, 5, -1, 6, -1, -1, -1, -1, -1, -1};
    const int ht3[19] = {-1, -1, -1, -1, -1, -1, -1, -1, -1, -1, -1, -1, -1, -1, 1, 2, 3, 4, 5};
    for (int k = 0; k < 19; ++k) {
        if (fx3[k] >= 0) s.F[3][fx3[k]] += kC2[k];
        if (gy3[k] >= 0) s.G[3][gy3[k]] += kC2[k];
        if (ht3[k] >= 0) s.H[3][ht3[k]] += kC2[k];
    }
    return s;
}

double poly_at(const double* c, int deg, double v) {
    double r = c[deg];
    for (int k = deg - 1; k >= 0; --k) r = r * v + c[k];
    return r;
}
}  // namespace

const ModelSplit& model_split() {
    static ModelSplit s = build_split();
    return s;
}

static void host_coefs(double x, double y, double out[4]) {
    const ModelSplit& s = model_split();
    double t = x * y;
    for (int m = 0; m < 4; ++m) {
        double g[7] = {0, s.G[m][1], s.G[m][2], s.G[m][3], s.G[m][4], s.G[m][5], s.G[m][6]};
        double h[6] = {0, s.H[m][1], s.H[m][2], s.H[m][3], s.H[m][4], s.H[m][5]};
        out[m] = poly_at(s.F[m], 7, x) + poly_at(g, 6, y) + poly_at(h, 5, t);
    }
}

double host_dstar(double x, double y, double logit_cut) {
    const double ln9 = 2.1972245773362196;
    double c[4];
    host_coefs(x, y, c);
    const double inf = std::numeric_limits<double>::infinity();
    if (!(c[1] > 0)) return inf;
    if (logit_cut >= ln9) return (-logit_cut - c[0]) / c[1];
    if (!(c[3] > 0)) return inf;
    double d1 = (-ln9 - c[0]) / c[1];
    double d2 = (-logit_cut - c[2]) / c[3];
    return d1 > d2 ? d1 : d2;
}

// ------------------------------------------------------------ C ABI ------

extern "C" {

const char* mdet_version(void) { return "mdet_tnf 0.1 sm_103a (tcgen05/TMA)"; }

int mdet_ctx_create(int device, mdet_ctx** out) {
    if (!out) return MDET_ERR_INVALID;
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return MDET_ERR_CUDA;
    }
    if (device < 0 || device >= ndev) return MDET_ERR_INVALID;
    mdet_ctx* c = new mdet_ctx();
    c->device = device;
    if (cudaSetDevice(device) != cudaSuccess) {
        delete c;
        return MDET_ERR_CUDA;
    }
    cudaDeviceProp prop;
    cudaGetDeviceProperties(&prop, device);
    c->num_sms = prop.multiProcessorCount;
    c->cc_major = prop.major;
    c->cc_minor = prop.minor;
    if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess) {
        delete c;
        return MDET_ERR_CUDA;
    }
    c->own_stream = true;
    if (cudaMalloc(&c->d_flag, sizeof(int)) != cudaSuccess) {
        cudaStreamDestroy(c->stream);
        delete c;
        return MDET_ERR_NOMEM;
    }
    cudaMemset(c->d_flag, 0, sizeof(int));
    *out = c;
    return MDET_OK;
}

int mdet_ctx_destroy(mdet_ctx* ctx) {
    if (!ctx) return MDET_OK;
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    timers_clear(ctx);
    if (ctx->batch_plan_free) ctx->batch_plan_free(ctx->batch_plan);
    for (auto& kv : ctx->bufs)
        if (kv.second.p) cudaFree(kv.second.p);
    if (ctx->pinned) cudaFreeHost(ctx->pinned);
    if (ctx->d_flag) cudaFree(ctx->d_flag);
    if (ctx->own_stream) cudaStreamDestroy(ctx->stream);
    if (ctx->io_in) cudaStreamDestroy(ctx->io_in);
    if (ctx->io_out) cudaStreamDestroy(ctx->io_out);
    if (ctx->cap_stream) cudaStreamDestroy(ctx->cap_stream);
    if (ctx->cap_stream2) cudaStreamDestroy(ctx->cap_stream2);
    if (ctx->cap_fork) cudaEventDestroy(ctx->cap_fork);
    if (ctx->cap_join) cudaEventDestroy(ctx->cap_join);
    delete ctx;
    return MDET_OK;
}

const char* mdet_last_error(const mdet_ctx* ctx) { return ctx ? ctx->err.c_str() : "null context"; }

int mdet_ctx_set_stream(mdet_ctx* ctx, void* stream) {
    if (!ctx) return MDET_ERR_INVALID;
    if (ctx->own_stream) {
        cudaStreamSynchronize(ctx->stream);
        cudaStreamDestroy(ctx->stream);
        ctx->own_stream = false;
    }
    ctx->stream = (cudaStream_t)stream;
    return MDET_OK;
}

int mdet_ctx_set_autotune(mdet_ctx* ctx, int mode) {
    if (!ctx) return MDET_ERR_INVALID;
    if (mode == 0 || mode == 1) {
        ctx->autotune = mode == 1;
        ctx->forced_shape = 0;
        return MDET_OK;
    }
    if (mode != 128256 && mode != 128128 && mode != 256128)
        return ctx_fail(ctx, MDET_ERR_INVALID, "unknown tile shape %d", mode);
    ctx->forced_shape = mode;
    return MDET_OK;
}

}  // extern "C"

int check_flag(mdet_ctx* ctx);  // graph.cu: reads and clears the device error flag

namespace {
// One thread waits, with the library's bounded wait, on an mbarrier that no
// thread ever arrives on; the wait runs out after `budget` cycles, raises the
// context's error flag and the kernel returns.  Nothing else is in flight.
__global__ void k_wait_probe(int* flag, unsigned long long budget) {
    __shared__ uint64_t bar;
    if (threadIdx.x == 0) {
        mbar_init(&bar, 1);
        mbar_fence_init();
        mbar_wait(&bar, 0, flag, budget);
    }
}
}  // namespace

extern "C" {

int mdet_ctx_check_wait(mdet_ctx* ctx, uint64_t budget_cycles) {
    if (!ctx) return MDET_ERR_INVALID;
    if (budget_cycles > MDET_SPIN_CYCLES) return ctx_fail(ctx, MDET_ERR_INVALID, "budget above the library's");
    MDET_CUDA(ctx, cudaSetDevice(ctx->device));
    ctx->launches = 0;
    k_wait_probe<<<1, 32, 0, ctx->stream>>>(ctx->d_flag, budget_cycles);
    MDET_LAUNCHED(ctx, "k_wait_probe");
    return check_flag(ctx);
}

int mdet_ctx_set_timing(mdet_ctx* ctx, int enable) {
    if (!ctx) return MDET_ERR_INVALID;
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    timers_clear(ctx);
    ctx->timing = enable != 0;
    return MDET_OK;
}

int mdet_ctx_kernel_ms(mdet_ctx* ctx, const char* kernel, double* ms, uint32_t* launches) {
    if (!ctx || !kernel || !ms) return MDET_ERR_INVALID;
    *ms = 0;
    if (launches) *launches = 0;
    auto it = ctx->timers.find(kernel);
    if (it == ctx->timers.end()) return MDET_OK;
    KernelTimer& t = it->second;
    for (auto& e : t.ev) {
        float f = 0;
        if (cudaEventSynchronize(e.second) != cudaSuccess) return ctx_cuda(ctx, cudaGetLastError(), "event");
        cudaEventElapsedTime(&f, e.first, e.second);
        t.ms += f;
        t.launches++;
        cudaEventDestroy(e.first);
        cudaEventDestroy(e.second);
    }
    t.ev.clear();
    *ms = t.ms;
    if (launches) *launches = t.launches;
    return MDET_OK;
}

uint64_t mdet_ctx_launch_count(const mdet_ctx* ctx) { return ctx ? ctx->total_launches : 0; }

}  // extern "C"

extern "C" {

int mdet_host_alloc(uint64_t bytes, void** out) {
    if (!out) return MDET_ERR_INVALID;
    *out = nullptr;
    if (cudaMallocHost(out, bytes ? bytes : 1) != cudaSuccess) {
        cudaGetLastError();
        *out = nullptr;
        return MDET_ERR_NOMEM;
    }
    return MDET_OK;
}

int mdet_host_free(void* p) {
    if (p && cudaFreeHost(p) != cudaSuccess) {
        cudaGetLastError();
        return MDET_ERR_CUDA;
    }
    return MDET_OK;
}

}  // extern "C"
