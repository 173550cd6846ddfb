// mlp_tc.cu -- the embedding network's inference on the tensor cores: the
// three layers of 136 -> 256 -> 128 -> 64 (GELU) fused in one persistent
// kernel, a CTA per 128-row tile at a time.  Each layer is one run of
// tcgen05.mma (kind::f16, BF16 x BF16 -> FP32 in TMEM, M = 128, N = 256 / 128
// / 64, K in steps of 16) issued by one thread: the tile's activations are
// the A operand and the layer's weights the B operand, both K-major in
// shared memory in the 128-byte-swizzled layout (8 rows x 128 bytes per
// 1 KB atom, the 16-byte granule g of row r stored at g ^ (r mod 8)).
// The weights are laid out in that image once per call (k_mlp_wimage) and
// copied into shared memory with one bulk copy per layer; the input rows
// are centred, scaled and rounded to BF16 by the CTA's threads as they are
// staged.  Each thread owns one TMEM lane (a row of the tile): the epilogue
// of a layer reads its row of the accumulator (tcgen05.ld), adds the bias,
// applies GELU, rounds to BF16 and writes the row into the next layer's A
// operand; the last layer's row goes to global memory in FP32.  Numerics:
// BF16 weights and activations, FP32 accumulation (the SIMT training path
// keeps FP32 activations).  All waits are bounded.
#include <cuda_bf16.h>

#include <algorithm>

#include "mlp.cuh"

namespace {

constexpr int kRows = 128;                 // rows per tile = TMEM lanes
constexpr int kThreads = 128;
constexpr uint32_t kChunkA = kRows * 128;  // one 64-element K chunk of a 128-row operand
// K chunks (64 elements) of each layer's input; 136 is padded to 192
constexpr int kKc1 = 3, kKc2 = MLP_H1 / 64, kKc3 = MLP_H2 / 64;
// weight images: N rows x KC chunks x 128 bytes
constexpr uint32_t kW1Bytes = MLP_H1 * kKc1 * 128;   // 96 KB
constexpr uint32_t kW2Bytes = MLP_H2 * kKc2 * 128;   // 64 KB
constexpr uint32_t kW3Bytes = MLP_OUT * kKc3 * 128;  // 16 KB
constexpr uint32_t kActBytes = kRows * kKc2 * 128;   // 64 KB (the widest input, H1)
constexpr uint32_t kSmem = kActBytes + kW1Bytes + 1024;
constexpr uint32_t kTmemCols = 512;                  // layer outputs at columns 0, 256, 384
constexpr uint32_t kLayoutSW128 = 2;

// byte offset of element (r, k) in a K-major SW128 operand of `rows` rows
__host__ __device__ __forceinline__ uint32_t swz(uint32_t rows, uint32_t r, uint32_t k) {
    return (k >> 6) * rows * 128 + r * 128 + ((((k & 63) >> 3) ^ (r & 7)) << 4) + (k & 7) * 2;
}

__device__ __forceinline__ uint64_t desc_sw128(uint32_t saddr) {
    uint64_t d = 0;
    d |= (uint64_t)((saddr & 0x3FFFFu) >> 4);
    d |= (uint64_t)1 << 16;
    d |= (uint64_t)(1024 >> 4) << 32;  // 8-row atoms 1 KB apart
    d |= (uint64_t)1 << 46;
    d |= (uint64_t)kLayoutSW128 << 61;
    return d;
}

// BF16 x BF16 -> FP32, M = 128, N = n, A and B K-major
__host__ __device__ constexpr uint32_t idesc(uint32_t n) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((n >> 3) << 17) | ((128u >> 4) << 24);
}

__device__ __forceinline__ void mma_bf16(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t id,
                                         uint32_t accumulate) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem_d),
        "l"(adesc), "l"(bdesc), "r"(id), "r"(accumulate)
        : "memory");
}

__device__ __forceinline__ void mma_commit(uint64_t* bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
                 : "memory");
}

__device__ __forceinline__ void fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// 32 consecutive FP32 columns of this thread's TMEM lane
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float (&v)[32]) {
    uint32_t r[32];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
        "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];\n"
        "tcgen05.wait::ld.sync.aligned;\n"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
          "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
          "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr)
        : "memory");
#pragma unroll
    for (int k = 0; k < 32; ++k) v[k] = __uint_as_float(r[k]);
}

__device__ __forceinline__ float gelu(float z) { return 0.5f * z * (1.f + erff(z * 0.70710678118654752f)); }

__device__ __forceinline__ uint32_t pack2(float a, float b) {
    const __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
    return *reinterpret_cast<const uint32_t*>(&h);
}

// The weight images of the three layers, one after another: element (n, k)
// of layer l is BF16(W_l[n][k]) (0 in the K padding).
__global__ void k_mlp_wimage(const float* __restrict__ P, unsigned char* __restrict__ img) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;  // one element
    const uint32_t n1 = MLP_H1 * kKc1 * 64, n2 = MLP_H2 * kKc2 * 64, n3 = MLP_OUT * kKc3 * 64;
    uint32_t rows, kin, kc, e;
    const float* W;
    unsigned char* base;
    if (i < n1) {
        e = i, rows = MLP_H1, kin = MLP_IN, kc = kKc1, W = P + MLP_W1, base = img;
    } else if (i < n1 + n2) {
        e = i - n1, rows = MLP_H2, kin = MLP_H1, kc = kKc2, W = P + MLP_W2, base = img + kW1Bytes;
    } else if (i < n1 + n2 + n3) {
        e = i - n1 - n2, rows = MLP_OUT, kin = MLP_H2, kc = kKc3, W = P + MLP_W3, base = img + kW1Bytes + kW2Bytes;
    } else {
        return;
    }
    const uint32_t r = e / (kc * 64), k = e % (kc * 64);
    const float w = k < kin ? W[r * kin + k] : 0.f;
    *reinterpret_cast<__nv_bfloat16*>(base + swz(rows, r, k)) = __float2bfloat16_rn(w);
}

struct __align__(8) MlpCtl {
    uint64_t w_full, mma_done;
    uint32_t tmem_base;
};

// One layer's epilogue for this thread's row: columns [c0, c0 + 32 * nq) of
// the accumulator, + bias, GELU, BF16 into the next A operand.
template <int NQ>
__device__ __forceinline__ void epi_hidden(uint32_t tmem_row, uint32_t col0, const float* __restrict__ bias,
                                           unsigned char* act, uint32_t r) {
#pragma unroll 1
    for (int q = 0; q < NQ; ++q) {
        float v[32];
        tmem_ld32(tmem_row + col0 + 32 * q, v);
#pragma unroll
        for (int g = 0; g < 4; ++g) {  // 16-byte granules of 8 columns
            uint4 u;
            const int c = 32 * q + 8 * g;
            u.x = pack2(gelu(v[8 * g + 0] + __ldg(bias + c + 0)), gelu(v[8 * g + 1] + __ldg(bias + c + 1)));
            u.y = pack2(gelu(v[8 * g + 2] + __ldg(bias + c + 2)), gelu(v[8 * g + 3] + __ldg(bias + c + 3)));
            u.z = pack2(gelu(v[8 * g + 4] + __ldg(bias + c + 4)), gelu(v[8 * g + 5] + __ldg(bias + c + 5)));
            u.w = pack2(gelu(v[8 * g + 6] + __ldg(bias + c + 6)), gelu(v[8 * g + 7] + __ldg(bias + c + 7)));
            *reinterpret_cast<uint4*>(act + swz(kRows, r, (uint32_t)c)) = u;
        }
    }
}

__global__ void __launch_bounds__(kThreads, 1) k_mlp_fwd_tc(const float* __restrict__ tnf, uint64_t n,
                                                             const float* __restrict__ P,
                                                             const unsigned char* __restrict__ wimg,
                                                             float* __restrict__ z, int* flag) {
    extern __shared__ unsigned char smem_raw[];
    __shared__ MlpCtl ctl;
    __shared__ float mu[MLP_IN];
    unsigned char* smem = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    unsigned char* act = smem;               // A operand: X (3 chunks), H1 (4), H2 (2)
    unsigned char* wsm = smem + kActBytes;   // B operand: W1, W2 or W3
    const uint32_t t = threadIdx.x, warp = t >> 5;
    if (t == 0) {
        mbar_init(&ctl.w_full, 1);
        mbar_init(&ctl.mma_done, 1);
        mbar_fence_init();
    }
    for (uint32_t k = t; k < MLP_IN; k += kThreads) mu[k] = P[MLP_MU + k];
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&ctl.tmem_base)),
                     "r"(kTmemCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    fence_before();
    __syncthreads();
    fence_after();
    const uint32_t tmem = ctl.tmem_base;
    const uint32_t tmem_row = tmem + ((warp * 32) << 16);
    const float scale = P[MLP_SCALE];
    const uint32_t sa = smem_u32(act), sw = smem_u32(wsm);
    uint32_t ph_w = 0, ph_m = 0;
    const uint64_t tiles = (n + kRows - 1) / kRows;

    // thread 0: a layer's weights into shared memory, then its MMAs; every
    // thread then waits for them.  The result is block-uniform: a timeout
    // anywhere ends every thread's loop at the same point.
    auto run_layer = [&](uint32_t wbytes, const unsigned char* src, int kc, uint32_t ncols, uint32_t col,
                         uint32_t rows_b) -> bool {
        if (t == 0) {
            mbar_arrive_tx(&ctl.w_full, wbytes);
            bulk_g2s(wsm, src, wbytes, &ctl.w_full);
        }
        fence_proxy_async_smem();  // this thread's activation stores, before the MMAs read them
        fence_before();
        __syncthreads();
        fence_after();
        bool issued = true;
        if (t == 0) {
            issued = mbar_wait(&ctl.w_full, ph_w, flag);
            if (issued) {
                fence_after();
                for (int s = 0; s < 4 * kc; ++s) {
                    const uint32_t c = s >> 2, off = (s & 3) * 32;  // 16 K elements = 32 bytes of a row
                    mma_bf16(tmem + col, desc_sw128(sa + c * kChunkA + off), desc_sw128(sw + c * rows_b * 128 + off),
                             idesc(ncols), s > 0 ? 1u : 0u);
                }
                mma_commit(&ctl.mma_done);
            }
        }
        ph_w ^= 1;
        // no commit means no completion: skip the wait rather than time out
        if (__syncthreads_or(!issued)) return false;
        const bool ok = mbar_wait(&ctl.mma_done, ph_m, flag);
        ph_m ^= 1;
        fence_after();
        return !__syncthreads_or(!ok);
    };

    for (uint64_t tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
        const uint64_t r0 = tile * kRows;
        // stage the tile's rows: centred, scaled, BF16, K padded to 192
        for (uint32_t g = t; g < kRows * kKc1 * 8; g += kThreads) {  // 16-byte granules
            const uint32_t r = g / (kKc1 * 8), k = (g % (kKc1 * 8)) * 8;
            uint4 u = make_uint4(0, 0, 0, 0);
            if (r0 + r < n && k < MLP_IN) {
                const float4* src = reinterpret_cast<const float4*>(tnf + (r0 + r) * MLP_IN + k);
                const float4 a = __ldg(src), b = __ldg(src + 1);
                u.x = pack2((a.x - mu[k + 0]) * scale, (a.y - mu[k + 1]) * scale);
                u.y = pack2((a.z - mu[k + 2]) * scale, (a.w - mu[k + 3]) * scale);
                u.z = pack2((b.x - mu[k + 4]) * scale, (b.y - mu[k + 5]) * scale);
                u.w = pack2((b.z - mu[k + 6]) * scale, (b.w - mu[k + 7]) * scale);
            }
            *reinterpret_cast<uint4*>(act + swz(kRows, r, k)) = u;
        }
        if (!run_layer(kW1Bytes, wimg, kKc1, MLP_H1, 0, MLP_H1)) break;
        epi_hidden<MLP_H1 / 32>(tmem_row, 0, P + MLP_B1, act, t);
        if (!run_layer(kW2Bytes, wimg + kW1Bytes, kKc2, MLP_H2, 256, MLP_H2)) break;
        epi_hidden<MLP_H2 / 32>(tmem_row, 256, P + MLP_B2, act, t);
        if (!run_layer(kW3Bytes, wimg + kW1Bytes + kW2Bytes, kKc3, MLP_OUT, 384, MLP_OUT)) break;
        // the embedding: + b3, FP32 to global
        const uint64_t row = r0 + t;
#pragma unroll
        for (int q = 0; q < MLP_OUT / 32; ++q) {
            float v[32];
            tmem_ld32(tmem_row + 384 + 32 * q, v);
            if (row < n) {
                float4* dst = reinterpret_cast<float4*>(z + row * MLP_OUT + 32 * q);
#pragma unroll
                for (int g = 0; g < 8; ++g) {
                    const int c = 32 * q + 4 * g;
                    dst[g] = make_float4(v[4 * g] + __ldg(P + MLP_B3 + c), v[4 * g + 1] + __ldg(P + MLP_B3 + c + 1),
                                         v[4 * g + 2] + __ldg(P + MLP_B3 + c + 2),
                                         v[4 * g + 3] + __ldg(P + MLP_B3 + c + 3));
                }
            }
        }
        fence_before();
        __syncthreads();  // the next tile overwrites the A operand and the accumulators
        fence_after();
    }
    fence_before();
    __syncthreads();
    fence_after();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmemCols) : "memory");
}

}  // namespace

// Embeddings of n rows on the tensor cores (sm_103 devices): z (n x 64).
int mlp_embed_tc(mdet_ctx* ctx, const float* P, const float* tnf, uint64_t n, float* z) {
    if (n == 0) return MDET_OK;
    cudaStream_t s = ctx->stream;
    unsigned char* img = (unsigned char*)ctx_scratch(ctx, "mlptc.wimg", kW1Bytes + kW2Bytes + kW3Bytes);
    if (!img) return MDET_ERR_NOMEM;
    const uint32_t nel = (kW1Bytes + kW2Bytes + kW3Bytes) / 2;
    k_mlp_wimage<<<(nel + 255) / 256, 256, 0, s>>>(P, img);
    MDET_LAUNCHED(ctx, "k_mlp_wimage");
    static bool attr[64] = {false};
    if (!attr[ctx->device & 63]) {
        MDET_CUDA(ctx, cudaFuncSetAttribute(k_mlp_fwd_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmem));
        attr[ctx->device & 63] = true;
    }
    const uint64_t tiles = (n + kRows - 1) / kRows;
    const unsigned grid = (unsigned)std::min<uint64_t>(tiles, (uint64_t)ctx->num_sms);
    ctx_timer_begin(ctx, "k_mlp_fwd_tc");
    k_mlp_fwd_tc<<<grid, kThreads, kSmem, s>>>(tnf, n, P, img, z, ctx->d_flag);
    MDET_LAUNCHED(ctx, "k_mlp_fwd_tc");
    ctx_timer_end(ctx, "k_mlp_fwd_tc");
    return MDET_OK;
}
