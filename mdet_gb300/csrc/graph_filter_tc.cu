// graph_filter_tc.cu -- tensor-core distance filter (tcgen05, sm_103a).
//
// The pairwise stage restructured as ||a||^2 + ||b||^2 - 2 a.b over centred
// BF16 rows: a.b is a 128 x 256 x 144 tile GEMM per (row tile, column tile)
// issued by one thread with tcgen05.mma (kind::f16, BF16 x BF16 -> FP32),
// operands staged in shared memory by TMA (cp.async.bulk.tensor, 128-byte
// swizzle for K 0..127, 32-byte swizzle for K 128..143), accumulators in TMEM
// (two 256-column buffers, so the epilogue of one tile overlaps the MMA of
// the next).  The epilogue reads TMEM with tcgen05.ld and keeps pairs with
//     dot > (||a~||^2 - R^2)/2 + ||b~||^2/2,
// R = d*_tile + e_a + e_b + slack, where d*_tile bounds the model's distance
// threshold over the tile's sizes and e_a, e_b bound the BF16 rounding of the
// rows (||a~ - a||).  By the triangle inequality no pair whose exact
// distance is below d* is dropped; the exact stage re-scores every kept pair,
// so the edge set equals the plain form's.  Nothing n x n leaves the SM.
//
// Warp roles (10 warps): 0 = TMA producer, 1 = MMA issuer + TMEM owner,
// 2..9 = epilogue (TMEM lane quarter = warp % 4, column half = (warp-2)/4).
// Every CTA walks a contiguous range of the row-major tile list, so the A
// tile (128 rows) is loaded once per row tile and B tiles stream through a
// two-stage ring.  All waits are bounded.
#include <cudaTypedefs.h>

#include "graph.cuh"

namespace {

constexpr int kBM = 128, kBN = 256;
constexpr uint32_t kAChunk = kBM * 128;           // 16 KB, 64 bf16 per row
constexpr uint32_t kATail = kBM * 32;             // 4 KB, 16 bf16 per row
constexpr uint32_t kABytes = 2 * kAChunk + kATail;  // 36 KB
constexpr uint32_t kBChunk = kBN * 128;           // 32 KB
constexpr uint32_t kBTail = kBN * 32;             // 8 KB
constexpr uint32_t kBBytes = 2 * kBChunk + kBTail;  // 72 KB
constexpr int kEpiWarps = 8;
constexpr int kThreads = (2 + kEpiWarps) * 32;
constexpr int kQueue = 512;                       // candidate queue per epilogue warp
constexpr uint32_t kTmemCols = 512;
constexpr uint32_t kSmemBytes = kABytes + 2 * kBBytes + 1024;  // + alignment slack

struct TcArgs {
    uint32_t na, nb, ta, tb;
    int triangular;
    const float* a_nsq;
    const float* b_nsq;
    const BlockMeta* ameta;
    const BlockMeta* bmeta;
    DstarTable tbl;
    CandBuf out;
    unsigned long long ntiles;
    int* flag;
};

struct __align__(8) Ctl {
    uint64_t a_full, a_empty;
    uint64_t b_full[2], b_empty[2];
    uint64_t acc_full[2], acc_empty[2];
    uint32_t tmem_base;
    uint32_t qcount[kEpiWarps];
};

// ---------------------------------------------------------------- PTX --

__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, int x, int y, uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
            smem_u32(dst)),
        "l"(map), "r"(x), "r"(y), "r"(smem_u32(bar))
        : "memory");
}

__device__ __forceinline__ void tma_prefetch_desc(const CUtensorMap* map) {
    asm volatile("prefetch.tensormap [%0];" ::"l"(map) : "memory");
}

// K-major shared-memory matrix descriptor (version 1 for tcgen05).
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t layout, uint32_t sbo) {
    uint64_t d = 0;
    d |= (uint64_t)((saddr & 0x3FFFFu) >> 4);
    d |= (uint64_t)1 << 16;                  // leading byte offset (unused for swizzled K-major)
    d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
    d |= (uint64_t)1 << 46;                  // descriptor version
    d |= (uint64_t)layout << 61;
    return d;
}
constexpr uint32_t kLayoutSW128 = 2, kLayoutSW32 = 6;

// BF16 x BF16 -> FP32, M = 128, N = 256, A and B K-major.
constexpr uint32_t kIdesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(kBN >> 3) << 17) |
                            ((uint32_t)(kBM >> 4) << 24);

__device__ __forceinline__ void mma_bf16(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t accumulate) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem_d),
        "l"(adesc), "l"(bdesc), "r"(kIdesc), "r"(accumulate)
        : "memory");
}

__device__ __forceinline__ void mma_commit(uint64_t* bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
                 : "memory");
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float (&v)[32]) {
    uint32_t r[32];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
        "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];\n"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
          "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
          "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int k = 0; k < 32; ++k) v[k] = __uint_as_float(r[k]);
}

// ------------------------------------------------------------ schedule --

// Tiles before row tile I in the row-major list (column tiles J >= I/2 in
// the triangular schedule, all J otherwise).
__device__ __forceinline__ unsigned long long row_start(const TcArgs& p, unsigned long long I) {
    if (!p.triangular) return I * p.tb;
    unsigned long long m = I >> 1;
    unsigned long long f = (I & 1) ? m * m : m * (m - (m ? 1 : 0));
    if (!(I & 1) && m == 0) f = 0;
    return I * p.tb - f;
}

__device__ __forceinline__ uint32_t j_start(const TcArgs& p, uint32_t I) { return p.triangular ? (I >> 1) : 0u; }

struct Cursor {
    uint32_t I, J;
    unsigned long long t, t1;
};

__device__ __forceinline__ Cursor cursor_at(const TcArgs& p, unsigned long long t0, unsigned long long t1) {
    // largest I with row_start(I) <= t0
    uint32_t lo = 0, hi = p.ta;  // row_start(ta) = ntiles > t0
    while (hi - lo > 1) {
        uint32_t mid = (lo + hi) >> 1;
        if (row_start(p, mid) <= t0)
            lo = mid;
        else
            hi = mid;
    }
    Cursor c;
    c.I = lo;
    c.J = j_start(p, lo) + (uint32_t)(t0 - row_start(p, lo));
    c.t = t0;
    c.t1 = t1;
    return c;
}

__device__ __forceinline__ void advance(const TcArgs& p, Cursor& c) {
    ++c.t;
    if (++c.J >= p.tb) {
        ++c.I;
        c.J = j_start(p, c.I);
    }
}

// -------------------------------------------------------------- kernel --

__global__ void __launch_bounds__(kThreads, 1)
    k_filter_tc(const __grid_constant__ CUtensorMap tmA128, const __grid_constant__ CUtensorMap tmA32,
                const __grid_constant__ CUtensorMap tmB128, const __grid_constant__ CUtensorMap tmB32, TcArgs p) {
    extern __shared__ unsigned char smem_raw[];
    __shared__ Ctl ctl;
    __shared__ uint2 queue[kEpiWarps][kQueue];
    unsigned char* smem = (unsigned char*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    unsigned char* sA = smem;
    unsigned char* sB = smem + kABytes;
    const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

    const unsigned long long G = gridDim.x;
    const unsigned long long t0 = p.ntiles * blockIdx.x / G, t1 = p.ntiles * (blockIdx.x + 1) / G;

    if (threadIdx.x == 0) {
        mbar_init(&ctl.a_full, 1);
        mbar_init(&ctl.a_empty, 1);
        for (int s = 0; s < 2; ++s) {
            mbar_init(&ctl.b_full[s], 1);
            mbar_init(&ctl.b_empty[s], 1);
            mbar_init(&ctl.acc_full[s], 1);
            mbar_init(&ctl.acc_empty[s], kEpiWarps * 32);
        }
        for (int w = 0; w < kEpiWarps; ++w) ctl.qcount[w] = 0;
        mbar_fence_init();
    }
    if (warp == 0 && lane == 0) {
        tma_prefetch_desc(&tmA128);
        tma_prefetch_desc(&tmA32);
        tma_prefetch_desc(&tmB128);
        tma_prefetch_desc(&tmB32);
    }
    if (warp == 1) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&ctl.tmem_base)),
                     "r"(kTmemCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = ctl.tmem_base;

    if (t0 < t1) {
        if (warp == 0) {
            // ------------------------------------------------ TMA producer
            if (lane == 0) {
                Cursor c = cursor_at(p, t0, t1);
                uint32_t a_e_ph = 0, b_e_ph[2] = {0, 0};
                uint32_t curI = 0xFFFFFFFFu;
                for (uint32_t lt = 0; c.t < c.t1; ++lt, advance(p, c)) {
                    if (c.I != curI) {
                        if (!mbar_wait(&ctl.a_empty, a_e_ph ^ 1, p.flag)) break;
                        a_e_ph ^= 1;
                        mbar_arrive_tx(&ctl.a_full, kABytes);
                        const int y = (int)(c.I * kBM);
                        tma_load_2d(sA, &tmA128, 0, y, &ctl.a_full);
                        tma_load_2d(sA + kAChunk, &tmA128, 64, y, &ctl.a_full);
                        tma_load_2d(sA + 2 * kAChunk, &tmA32, 128, y, &ctl.a_full);
                        curI = c.I;
                    }
                    const uint32_t bs = lt & 1;
                    if (!mbar_wait(&ctl.b_empty[bs], b_e_ph[bs] ^ 1, p.flag)) break;
                    b_e_ph[bs] ^= 1;
                    unsigned char* dst = sB + bs * kBBytes;
                    mbar_arrive_tx(&ctl.b_full[bs], kBBytes);
                    const int y = (int)(c.J * kBN);
                    tma_load_2d(dst, &tmB128, 0, y, &ctl.b_full[bs]);
                    tma_load_2d(dst + kBChunk, &tmB128, 64, y, &ctl.b_full[bs]);
                    tma_load_2d(dst + 2 * kBChunk, &tmB32, 128, y, &ctl.b_full[bs]);
                }
            }
        } else if (warp == 1) {
            // -------------------------------------------------- MMA issuer
            if (lane == 0) {
                Cursor c = cursor_at(p, t0, t1);
                uint32_t a_ph = 0, b_ph[2] = {0, 0}, e_ph[2] = {0, 0};
                uint32_t curI = 0xFFFFFFFFu;
                const uint32_t a_base = smem_u32(sA), b_base = smem_u32(sB);
                for (uint32_t lt = 0; c.t < c.t1; ++lt) {
                    if (c.I != curI) {
                        if (!mbar_wait(&ctl.a_full, a_ph, p.flag)) break;
                        a_ph ^= 1;
                        curI = c.I;
                    }
                    const uint32_t s = lt & 1;
                    if (!mbar_wait(&ctl.acc_empty[s], e_ph[s] ^ 1, p.flag)) break;
                    e_ph[s] ^= 1;
                    if (!mbar_wait(&ctl.b_full[s], b_ph[s], p.flag)) break;
                    b_ph[s] ^= 1;
                    tc_fence_after();
                    const uint32_t d = tmem + s * kBN;
                    const uint32_t bb = b_base + s * kBBytes;
#pragma unroll
                    for (int k = 0; k < 9; ++k) {
                        uint64_t ad, bd;
                        if (k < 8) {
                            const uint32_t ch = k >> 2, ko = (k & 3) * 32;
                            ad = smem_desc(a_base + ch * kAChunk + ko, kLayoutSW128, 1024);
                            bd = smem_desc(bb + ch * kBChunk + ko, kLayoutSW128, 1024);
                        } else {
                            ad = smem_desc(a_base + 2 * kAChunk, kLayoutSW32, 256);
                            bd = smem_desc(bb + 2 * kBChunk, kLayoutSW32, 256);
                        }
                        mma_bf16(d, ad, bd, k > 0 ? 1u : 0u);
                    }
                    mma_commit(&ctl.b_empty[s]);
                    mma_commit(&ctl.acc_full[s]);
                    Cursor nx = c;
                    advance(p, nx);
                    if (nx.t >= nx.t1 || nx.I != c.I) mma_commit(&ctl.a_empty);
                    c = nx;
                }
            }
        } else {
            // ---------------------------------------------------- epilogue
            const uint32_t ew = warp - 2;           // 0..7
            const uint32_t quarter = warp & 3;      // TMEM lanes 32*quarter ..
            const uint32_t half = ew >> 2;          // column half of the 256-wide tile
            uint32_t* qc = &ctl.qcount[ew];
            uint2* q = queue[ew];
            Cursor c = cursor_at(p, t0, t1);
            uint32_t f_ph[2] = {0, 0};
            for (uint32_t lt = 0; c.t < c.t1; ++lt, advance(p, c)) {
                const uint32_t s = lt & 1;
                const uint32_t row = c.I * kBM + quarter * 32 + lane;
                // tile threshold
                const BlockMeta ma = p.ameta[c.I];
                const BlockMeta mb0 = p.bmeta[2 * c.J], mb1 = p.bmeta[2 * c.J + 1];
                const float blo = fminf(mb0.lo, mb1.lo), bhi = fmaxf(mb0.hi, mb1.hi);
                const float T = tile_dstar(p.tbl, ma.lo, ma.hi, blo, bhi);
                const float E = ma.emax + fmaxf(mb0.emax, mb1.emax);
                const float N2 = ma.nmax * fmaxf(mb0.nmax, mb1.nmax);
                const float R = T * (1.f + 2e-5f) + 1e-6f + E;
                float R2 = R * R + 4e-5f * N2 + 1e-7f;
                if (!(R2 < 1e30f)) R2 = __int_as_float(0x7f800000);
                const float hr = 0.5f * (__ldg(p.a_nsq + row) - R2);
                const bool diag = p.triangular && (c.J * kBN < c.I * kBM + kBM);
                const bool ok = mbar_wait(&ctl.acc_full[s], f_ph[s], p.flag);
                if (!__all_sync(0xffffffffu, ok)) break;  // warp-uniform, so tcgen05.ld stays converged
                f_ph[s] ^= 1;
                tc_fence_after();
#pragma unroll 1
                for (uint32_t ch = 0; ch < 4; ++ch) {
                    const uint32_t col0 = half * 128 + ch * 32;
                    float v[32];
                    tmem_ld32(tmem + ((quarter * 32) << 16) + s * kBN + col0, v);
                    const uint32_t gc0 = c.J * kBN + col0;
                    const float4* hcp = reinterpret_cast<const float4*>(p.b_nsq + gc0);
                    float m0 = -__int_as_float(0x7f800000), m1 = m0, m2 = m0, m3 = m0;
#pragma unroll
                    for (int k4 = 0; k4 < 8; ++k4) {
                        const float4 h = __ldg(hcp + k4);
                        v[4 * k4 + 0] = fmaf(-0.5f, h.x, v[4 * k4 + 0]);
                        v[4 * k4 + 1] = fmaf(-0.5f, h.y, v[4 * k4 + 1]);
                        v[4 * k4 + 2] = fmaf(-0.5f, h.z, v[4 * k4 + 2]);
                        v[4 * k4 + 3] = fmaf(-0.5f, h.w, v[4 * k4 + 3]);
                        m0 = fmaxf(m0, v[4 * k4 + 0]);
                        m1 = fmaxf(m1, v[4 * k4 + 1]);
                        m2 = fmaxf(m2, v[4 * k4 + 2]);
                        m3 = fmaxf(m3, v[4 * k4 + 3]);
                    }
                    const float m = fmaxf(fmaxf(m0, m1), fmaxf(m2, m3));
                    if (m > hr) {
                        uint32_t mask = 0;
#pragma unroll
                        for (int k = 0; k < 32; ++k) mask |= (v[k] > hr ? 1u : 0u) << k;
                        while (mask) {
                            const int k = __ffs(mask) - 1;
                            mask &= mask - 1;
                            const uint32_t col = gc0 + k;
                            if (col < p.nb && row < p.na && (!diag || col > row)) {
                                uint32_t slot = atomicAdd(qc, 1u);
                                if (slot < (uint32_t)kQueue) {
                                    q[slot] = make_uint2(row, col);
                                } else {
                                    unsigned long long pos = atomicAdd(p.out.count, 1ull);
                                    if (pos < p.out.cap) p.out.cand[pos] = make_uint2(row, col);
                                }
                            }
                        }
                    }
                }
                tc_fence_before();
                mbar_arrive(&ctl.acc_empty[s]);
                // flush this warp's queue when it is half full
                __syncwarp();
                uint32_t cnt = *(volatile uint32_t*)qc;
                if (cnt >= kQueue / 2) {
                    cnt = cnt < (uint32_t)kQueue ? cnt : (uint32_t)kQueue;
                    unsigned long long base = 0;
                    if (lane == 0) base = atomicAdd(p.out.count, (unsigned long long)cnt);
                    base = __shfl_sync(0xffffffffu, base, 0);
                    for (uint32_t i = lane; i < cnt; i += 32)
                        if (base + i < p.out.cap) p.out.cand[base + i] = q[i];
                    __syncwarp();
                    if (lane == 0) *(volatile uint32_t*)qc = 0;
                    __syncwarp();
                }
            }
            // final flush
            __syncwarp();
            uint32_t cnt = *(volatile uint32_t*)qc;
            cnt = cnt < (uint32_t)kQueue ? cnt : (uint32_t)kQueue;
            if (cnt) {
                unsigned long long base = 0;
                if (lane == 0) base = atomicAdd(p.out.count, (unsigned long long)cnt);
                base = __shfl_sync(0xffffffffu, base, 0);
                for (uint32_t i = lane; i < cnt; i += 32)
                    if (base + i < p.out.cap) p.out.cand[base + i] = q[i];
            }
        }
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (warp == 1) {
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmemCols) : "memory");
    }
}

// ---------------------------------------------------------------- host --

PFN_cuTensorMapEncodeTiled_v12000 get_encode(mdet_ctx* ctx) {
    if (!ctx->encode_tiled) {
        void* fn = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) !=
                cudaSuccess ||
            q != cudaDriverEntryPointSuccess)
            return nullptr;
        ctx->encode_tiled = fn;
    }
    return (PFN_cuTensorMapEncodeTiled_v12000)ctx->encode_tiled;
}

int make_map(mdet_ctx* ctx, CUtensorMap* map, const uint16_t* base, uint64_t rows, uint32_t box_k, uint32_t box_rows,
             CUtensorMapSwizzle sw) {
    auto enc = get_encode(ctx);
    if (!enc) return ctx_fail(ctx, MDET_ERR_CUDA, "cuTensorMapEncodeTiled unavailable");
    cuuint64_t dims[2] = {MDET_KPAD, rows};
    cuuint64_t strides[1] = {MDET_KPAD * 2};
    cuuint32_t box[2] = {box_k, box_rows};
    cuuint32_t es[2] = {1, 1};
    CUresult r = enc(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, (void*)base, dims, strides, box, es,
                     CU_TENSOR_MAP_INTERLEAVE_NONE, sw, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                     CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return ctx_fail(ctx, MDET_ERR_CUDA, "cuTensorMapEncodeTiled failed (%d)", (int)r);
    return MDET_OK;
}

}  // namespace

int filter_tc(mdet_ctx* ctx, const uint16_t* a, const float* a_nsq, uint32_t na, const BlockMeta* ameta,
              const uint16_t* b, const float* b_nsq, uint32_t nb, const BlockMeta* bmeta, bool triangular,
              const DstarTable& tbl, CandBuf out) {
    if (na == 0 || nb == 0) return MDET_OK;
    const uint64_t na_pad = (na + 255) / 256 * 256, nb_pad = (nb + 255) / 256 * 256;
    CUtensorMap mA128, mA32, mB128, mB32;
    MDET_TRY(make_map(ctx, &mA128, a, na_pad, 64, kBM, CU_TENSOR_MAP_SWIZZLE_128B));
    MDET_TRY(make_map(ctx, &mA32, a, na_pad, 16, kBM, CU_TENSOR_MAP_SWIZZLE_32B));
    MDET_TRY(make_map(ctx, &mB128, b, nb_pad, 64, kBN, CU_TENSOR_MAP_SWIZZLE_128B));
    MDET_TRY(make_map(ctx, &mB32, b, nb_pad, 16, kBN, CU_TENSOR_MAP_SWIZZLE_32B));
    TcArgs p;
    p.na = na;
    p.nb = nb;
    p.ta = (na + kBM - 1) / kBM;
    p.tb = (nb + kBN - 1) / kBN;
    p.triangular = triangular ? 1 : 0;
    p.a_nsq = a_nsq;
    p.b_nsq = b_nsq;
    p.ameta = ameta;
    p.bmeta = bmeta;
    p.tbl = tbl;
    p.out = out;
    p.flag = ctx->d_flag;
    unsigned long long total = (unsigned long long)p.ta * p.tb;
    if (triangular) {
        unsigned long long m = p.ta >> 1;
        unsigned long long f = (p.ta & 1) ? m * m : (m ? m * (m - 1) : 0);
        total -= f;
    }
    p.ntiles = total;
    static bool attr[64] = {false};
    if (!attr[ctx->device & 63]) {
        MDET_CUDA(ctx, cudaFuncSetAttribute(k_filter_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmemBytes));
        attr[ctx->device & 63] = true;
    }
    unsigned grid = (unsigned)std::min<unsigned long long>((unsigned long long)ctx->num_sms, total);
    ctx_timer_begin(ctx, "k_filter_tc");
    k_filter_tc<<<grid, kThreads, kSmemBytes, ctx->stream>>>(mA128, mA32, mB128, mB32, p);
    ctx_timer_end(ctx, "k_filter_tc");
    MDET_LAUNCHED(ctx, "k_filter_tc");
    return MDET_OK;
}
