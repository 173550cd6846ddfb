// common.cuh -- shared internals of libmdet_tnf: the context, its scratch
// arena, status handling, PTX wrappers (mbarrier, bulk copies, tcgen05) and
// the MetaBAT2 logistic-model coefficients.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <map>
#include <string>
#include <unordered_map>
#include <utility>
#include <vector>

#include "../../include/mdet_tnf.h"

#define MDET_NTNF 136

// ---------------------------------------------------------------- context --

struct DevBuf {
    void* p = nullptr;
    size_t cap = 0;
};

struct KernelTimer {
    std::vector<std::pair<cudaEvent_t, cudaEvent_t>> ev;  // pending and finished launches
    double ms = 0;
    uint32_t launches = 0;
};

struct mdet_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    int num_sms = 0;
    int cc_major = 0, cc_minor = 0;
    std::string err;
    std::unordered_map<std::string, DevBuf> bufs;  // named grow-only device scratch
    void* pinned = nullptr;                        // pinned host staging
    size_t pinned_cap = 0;
    int* d_flag = nullptr;     // device error flag (bounded waits that ran out)
    uint32_t launches = 0;     // kernels launched by the current call
    void* encode_tiled = nullptr;  // cuTensorMapEncodeTiled entry point
    bool count_scratch_dirty = false;
    uint64_t total_launches = 0;
    // keys of the d* tables held in scratch "tbl.st0".."tbl.st3" (least
    // recently used one is rebuilt on a miss)
    struct TblSlot {
        bool valid = false;
        double L = 0, lmin = 0, lmax = 0;
        uint64_t used = 0;
    } tbl[4];
    uint64_t tbl_clock = 0;
    bool timing = false;
    std::unordered_map<std::string, KernelTimer> timers;
    const struct mdet_mlp* mlp = nullptr;          // network of MDET_MODE_LEARNED
    mdet_learned_report* learned_report = nullptr;  // optional caller-owned report
    // tile-shape autotuner of the tensor-core filter: chosen column-tile
    // width per shape class, whether to tune, and the width of the last launch
    std::map<uint64_t, int> tc_shape;
    std::map<uint64_t, int> exact_shape;  // blocks per SM of the exact stage
    bool autotune = true;
    int forced_shape = 0;  // tile-shape code forced by mdet_ctx_set_autotune (0: none)
    int forced_exact = 0;  // exact-stage blocks per SM forced while a pass is captured (0: none)
    int last_tile_n = 0;
    // CUDA-graph capture of repeated batched passes
    bool graph_capture = true;
    bool capturing = false;
    uint64_t scratch_gen = 0;  // bumped whenever a scratch buffer is (re)allocated
    uint64_t graph_replays = 0;
    void* batch_plan = nullptr;
    void (*batch_plan_free)(void*) = nullptr;
    // The last size-sorted preparation ("pre" buffers): which inputs it was
    // made from (pointers, n, BF16 part, a hash of their contents) and which
    // buffers hold it.  Counting invalidates it (new TNF rows).
    struct PrepCache {
        bool valid = false;
        const void* tnf = nullptr;
        const void* ls = nullptr;
        uint64_t n = 0;
        int tck = 0;  // reduced-precision rows made (0 none, 1 BF16, 2 TF32)
        unsigned long long hash = 0;
        const void* x32 = nullptr;
        const void* xa = nullptr;
        const void* ta = nullptr;
        uint64_t gen = 0;  // scratch_gen when it was made (no buffer moved since)
    } prep_cache;
    // copy streams of the host-buffer entry points (created on first use)
    cudaStream_t io_in = nullptr, io_out = nullptr;
    // stream CUDA-graph recordings are captured on (the caller's stream may be
    // the legacy default stream, which cannot be captured)
    cudaStream_t cap_stream = nullptr;
    // a second capture stream and the events that fork work onto it and join
    // it back, for recordings with independent branches
    cudaStream_t cap_stream2 = nullptr;
    cudaEvent_t cap_fork = nullptr, cap_join = nullptr;
    // abundance set by mdet_ctx_set_abundance: contigs and samples (the
    // matrices and per-contig low flags live in scratch "abd.m", "abd.v",
    // "abd.low"); nabd == 0: none
    uint64_t abd_n = 0;
    uint32_t abd_nabd = 0;
};

// Event pair around one launch of a named kernel when timing is enabled.
void ctx_timer_begin(mdet_ctx* ctx, const char* kernel);
void ctx_timer_end(mdet_ctx* ctx, const char* kernel);

// Returns a device buffer of at least `bytes` named `name`, growing it if
// needed.  zero_on_grow: freshly grown buffers are memset to 0.
void* ctx_scratch(mdet_ctx* ctx, const char* name, size_t bytes, bool zero_on_grow = false);
void* ctx_pinned(mdet_ctx* ctx, size_t bytes);
int ctx_fail(mdet_ctx* ctx, int code, const char* fmt, ...);
int ctx_cuda(mdet_ctx* ctx, cudaError_t e, const char* what);
int ctx_check_launch(mdet_ctx* ctx, const char* what);

#define MDET_TRY(call)                     \
    do {                                   \
        int _rc = (call);                  \
        if (_rc != MDET_OK) return _rc;    \
    } while (0)
#define MDET_CUDA(ctx, call) MDET_TRY(ctx_cuda((ctx), (call), #call))
#define MDET_LAUNCHED(ctx, what)                   \
    do {                                           \
        (ctx)->launches++;                         \
        (ctx)->total_launches++;                   \
        MDET_TRY(ctx_check_launch((ctx), (what))); \
    } while (0)

// Device-wide bounded-wait budget: ~2 s at 2 GHz.
#define MDET_SPIN_CYCLES (4000000000ull)
#define MDET_FLAG_TIMEOUT 1

// ------------------------------------------------------ canonical tables --

// 8-bit raw 4-mer code (base codes A=0,C=1,T=2,G=3, oldest base in the high
// bits) -> canonical TNF column; and per column its forward and
// reverse-complement raw codes.  Built on the host from the column order.
struct TnTables {
    uint8_t raw_to_col[256];
    uint8_t col_fw[MDET_NTNF];
    uint8_t col_rc[MDET_NTNF];
};
const TnTables& tn_tables();

// Uploads the canonical tables to __constant__ memory once per device.
int ensure_constants(mdet_ctx* ctx);

// ------------------------------------------------------- model pieces ----
// b(x,y) and c(x,y) of both logistic models split as F(x) + G(y) + H(x*y)
// with x = min log size, y = max log size (cuda/Cuda2.cu:199-236).
struct ModelSplit {
    // F coefficients: powers x^0..x^7; G: y^1..y^6; H: t^1..t^5 (t = x*y)
    double F[4][8];
    double G[4][7];
    double H[4][6];
};
const ModelSplit& model_split();

// Host FP64 evaluation of the largest distance d* with pre-probability above
// logit_cut for log sizes (x <= y); returns +inf where the model is not
// decreasing in d.
double host_dstar(double x, double y, double logit_cut);

// ------------------------------------------------------------ PTX helpers --

static __device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

static __device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

static __device__ __forceinline__ void mbar_fence_init() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

static __device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

static __device__ __forceinline__ void mbar_arrive_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}

static __device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// try_wait with a suspend-time hint (ns): the thread sleeps until the phase
// completes or the hint runs out instead of polling, so waiting warps leave
// their issue slots to the working ones.
static __device__ __forceinline__ bool mbar_try_wait_suspend(uint64_t* bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity), "r"(1000000u)
        : "memory");
    return ok != 0;
}

// Bounded wait: returns false (and raises the device flag) when the budget
// (SM clock cycles) runs out, so no wait in this library can spin forever.
static __device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, int* flag,
                                                 unsigned long long budget = MDET_SPIN_CYCLES) {
    if (mbar_try_wait(bar, parity)) return true;
    long long t0 = clock64();
    while (true) {
        if (mbar_try_wait_suspend(bar, parity)) return true;
        if ((unsigned long long)(clock64() - t0) > budget) {
            if (flag) atomicOr(flag, MDET_FLAG_TIMEOUT);
            return false;
        }
        if (flag && *(volatile int*)flag) return false;
    }
}

// 1-D bulk copy global -> shared (TMA engine), completion on an mbarrier.
static __device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_u32(dst)),
        "l"(src), "r"(bytes), "r"(smem_u32(bar))
        : "memory");
}

static __device__ __forceinline__ void fence_proxy_async_smem() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

static __device__ __forceinline__ uint32_t lane_id() {
    uint32_t l;
    asm volatile("mov.u32 %0, %%laneid;" : "=r"(l));
    return l;
}
