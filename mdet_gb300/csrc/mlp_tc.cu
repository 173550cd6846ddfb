// mlp_tc.cu -- the embedding network on the tensor cores: inference and the
// GEMMs of training.  The network is 136 -> 256 -> 128 -> 64 (GELU).
//
// Forward (k_mlp_fwd_tc): the three layers fused in one persistent kernel, a
// CTA per 128-row tile at a time.  Each layer is one run of tcgen05.mma
// (kind::f16, BF16 x BF16 -> FP32 in TMEM, M = 128, N = 256 / 128 / 64, K in
// steps of 16) issued by one thread: the tile's activations are the A operand
// and the layer's weights the B operand, both K-major in shared memory in the
// 128-byte-swizzled layout (8 rows x 128 bytes per 1 KB atom, the 16-byte
// granule g of row r stored at g ^ (r mod 8)).  The weights are laid out in
// that image once per call (k_mlp_wimage) and copied into shared memory with
// one bulk copy per layer; the input rows are centred, scaled and rounded to
// BF16 by the CTA's threads as they are staged.  Each thread owns one TMEM
// lane (a row of the tile): a layer's epilogue reads its row of the
// accumulator (tcgen05.ld), adds the bias, applies GELU, rounds to BF16 and
// writes the row into the next layer's A operand; the last layer's row goes to
// global memory in FP32.  For training the forward pass also keeps the
// pre-activations (FP32) and the BF16 layer inputs transposed (feature-major),
// the operands of the weight gradients.
//
// Backward (k_mlp_bwd_tc): per 128-row tile, dH2 = dZ3 W3 and dH1 = dZ2 W2 as
// the same fused two-layer scheme (B operands: the transposed weight images),
// each epilogue multiplying by GELU' of the saved pre-activation and writing
// dZ in FP32 (bias gradients) and transposed BF16.  Weight gradients
// (k_mlp_dw_tc): dW = dZ^T H with K = the batch's rows, split over CTAs, the
// A and B tiles staged from the transposed arrays, partial sums added into
// the FP32 gradient.  Numerics: BF16 GEMM operands, FP32 accumulation.  All
// waits are bounded.
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
// backward images: W3^T (128 rows, K = 64) and W2^T (256 rows, K = 128)
constexpr uint32_t kW3tBytes = MLP_H2 * 1 * 128;      // 16 KB
constexpr uint32_t kW2tBytes = MLP_H1 * 2 * 128;      // 64 KB
constexpr uint32_t kImgBytes = kW1Bytes + kW2Bytes + kW3Bytes + kW3tBytes + kW2tBytes;
// the backward kernel's operands take 96 KB; 120 KB keeps it at one CTA per
// SM, so that its 512 TMEM columns are never contended
constexpr uint32_t kSmemBwd = 120 * 1024;
// weight gradients: an A chunk (128 x 64) and a B chunk (up to 256 x 64);
// 100 KB allows two CTAs per SM, whose 256 TMEM columns each fit together
constexpr uint32_t kSmemDw = 100 * 1024;
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

__device__ __forceinline__ float gelu_grad(float z) {
    const float cdf = 0.5f * (1.f + erff(z * 0.70710678118654752f));
    const float pdf = 0.39894228040143268f * expf(-0.5f * z * z);
    return cdf + z * pdf;
}

__device__ __forceinline__ __nv_bfloat16 bf(float v) { return __float2bfloat16_rn(v); }

__device__ __forceinline__ uint32_t pack2(float a, float b) {
    const __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
    return *reinterpret_cast<const uint32_t*>(&h);
}

// The weight images, one after another: W1, W2, W3 (element (n, k) =
// BF16(W[n][k]), 0 in the K padding), then W3^T and W2^T (element (n, k) =
// BF16(W[k][n])), the B operands of the backward pass.
__global__ void k_mlp_wimage(const float* __restrict__ P, unsigned char* __restrict__ img) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;  // one element
    const uint32_t n1 = MLP_H1 * kKc1 * 64, n2 = MLP_H2 * kKc2 * 64, n3 = MLP_OUT * kKc3 * 64;
    const uint32_t n4 = MLP_H2 * 64, n5 = MLP_H1 * 128;
    uint32_t rows, kin, kc, e;
    bool tr = false;
    const float* W;
    unsigned char* base;
    if (i < n1) {
        e = i, rows = MLP_H1, kin = MLP_IN, kc = kKc1, W = P + MLP_W1, base = img;
    } else if (i < n1 + n2) {
        e = i - n1, rows = MLP_H2, kin = MLP_H1, kc = kKc2, W = P + MLP_W2, base = img + kW1Bytes;
    } else if (i < n1 + n2 + n3) {
        e = i - n1 - n2, rows = MLP_OUT, kin = MLP_H2, kc = kKc3, W = P + MLP_W3, base = img + kW1Bytes + kW2Bytes;
    } else if (i < n1 + n2 + n3 + n4) {  // W3^T: rows = h2 units, K = output units
        e = i - n1 - n2 - n3, rows = MLP_H2, kin = MLP_OUT, kc = 1, W = P + MLP_W3, tr = true;
        base = img + kW1Bytes + kW2Bytes + kW3Bytes;
    } else if (i < n1 + n2 + n3 + n4 + n5) {  // W2^T: rows = h1 units, K = h2 units
        e = i - n1 - n2 - n3 - n4, rows = MLP_H1, kin = MLP_H2, kc = 2, W = P + MLP_W2, tr = true;
        base = img + kW1Bytes + kW2Bytes + kW3Bytes + kW3tBytes;
    } else {
        return;
    }
    const uint32_t r = e / (kc * 64), k = e % (kc * 64);
    float w = 0.f;
    if (k < kin) w = tr ? W[k * rows + r] : W[r * kin + k];
    *reinterpret_cast<__nv_bfloat16*>(base + swz(rows, r, k)) = __float2bfloat16_rn(w);
}

struct __align__(8) MlpCtl {
    uint64_t w_full, mma_done;
    uint32_t tmem_base;
};

// The per-CTA machinery of a fused layer chain: 128 threads, one TMEM lane
// each, an A operand (act) written by the threads and a B operand (wsm)
// bulk-copied from a weight image.
struct Chain {
    MlpCtl* ctl;
    unsigned char* act;
    unsigned char* wsm;
    uint32_t tmem, sa, sw, ph_w, ph_m;
    int* flag;

    __device__ void init(MlpCtl* c, unsigned char* smem, uint32_t act_bytes, uint32_t tmem_cols, int* f) {
        ctl = c;
        act = smem;
        wsm = smem + act_bytes;
        flag = f;
        ph_w = ph_m = 0;
        if (threadIdx.x == 0) {
            mbar_init(&ctl->w_full, 1);
            mbar_init(&ctl->mma_done, 1);
            mbar_fence_init();
        }
        if (threadIdx.x < 32) {
            asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                             smem_u32(&ctl->tmem_base)),
                         "r"(tmem_cols)
                         : "memory");
            asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
        }
        fence_before();
        __syncthreads();
        fence_after();
        tmem = ctl->tmem_base;
        sa = smem_u32(act);
        sw = smem_u32(wsm);
    }
    __device__ void finish(uint32_t tmem_cols) {
        fence_before();
        __syncthreads();
        fence_after();
        if (threadIdx.x < 32)
            asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(tmem_cols)
                         : "memory");
    }
    // thread 0: the layer's weights into shared memory, then its MMAs (A: kc
    // K chunks of the 128-row act operand, B: rows_b rows); every thread
    // then waits for them.  Block-uniform result: a timeout anywhere ends
    // every thread's loop at the same point.
    __device__ bool layer(uint32_t wbytes, const unsigned char* src, int kc, uint32_t ncols, uint32_t col,
                          uint32_t rows_b) {
        const uint32_t t = threadIdx.x;
        if (t == 0) {
            mbar_arrive_tx(&ctl->w_full, wbytes);
            bulk_g2s(wsm, src, wbytes, &ctl->w_full);
        }
        fence_proxy_async_smem();  // this thread's operand stores, before the MMAs read them
        fence_before();
        __syncthreads();
        fence_after();
        bool issued = true;
        if (t == 0) {
            issued = mbar_wait(&ctl->w_full, ph_w, flag);
            if (issued) {
                fence_after();
                for (int s = 0; s < 4 * kc; ++s) {
                    const uint32_t c = s >> 2, off = (s & 3) * 32;  // 16 K elements = 32 bytes of a row
                    mma_bf16(tmem + col, desc_sw128(sa + c * kChunkA + off), desc_sw128(sw + c * rows_b * 128 + off),
                             idesc(ncols), s > 0 ? 1u : 0u);
                }
                mma_commit(&ctl->mma_done);
            }
        }
        ph_w ^= 1;
        // no commit means no completion: skip the wait rather than time out
        if (__syncthreads_or(!issued)) return false;
        const bool ok = mbar_wait(&ctl->mma_done, ph_m, flag);
        ph_m ^= 1;
        fence_after();
        return !__syncthreads_or(!ok);
    }
};

// Outputs the training pass keeps (null in inference): FP32 pre-activations
// [rows][256] and [rows][128]; BF16 layer inputs transposed, [192][ld],
// [256][ld] and [128][ld] (ld = the padded row count).
struct FwdKeep {
    float* z1;
    float* z2;
    __nv_bfloat16* xT;
    __nv_bfloat16* h1T;
    __nv_bfloat16* h2T;
    uint64_t ld;
};

// A hidden layer's epilogue for this thread's row r (global row g, kept when
// g < n): columns [col0, col0 + 32 * NQ) of the accumulator, + bias, GELU,
// BF16 into the next A operand; the training pass also keeps z and h^T.
template <int NQ>
__device__ __forceinline__ void epi_hidden(uint32_t tmem_row, uint32_t col0, const float* __restrict__ bias,
                                           unsigned char* act, uint32_t r, float* zkeep, __nv_bfloat16* hT,
                                           uint64_t ld, uint64_t g, bool keep) {
#pragma unroll 1
    for (int q = 0; q < NQ; ++q) {
        float v[32];
        tmem_ld32(tmem_row + col0 + 32 * q, v);
#pragma unroll
        for (int j = 0; j < 32; ++j) v[j] += __ldg(bias + 32 * q + j);
        if (zkeep && keep) {
            float4* zd = reinterpret_cast<float4*>(zkeep + g * (NQ * 32) + 32 * q);
#pragma unroll
            for (int j = 0; j < 8; ++j) zd[j] = make_float4(v[4 * j], v[4 * j + 1], v[4 * j + 2], v[4 * j + 3]);
        }
#pragma unroll
        for (int j = 0; j < 32; ++j) v[j] = gelu(v[j]);
        if (hT) {
#pragma unroll
            for (int j = 0; j < 32; ++j) hT[(uint64_t)(32 * q + j) * ld + g] = bf(keep ? v[j] : 0.f);
        }
#pragma unroll
        for (int c8 = 0; c8 < 4; ++c8) {  // 16-byte granules of 8 columns
            uint4 u;
            u.x = pack2(v[8 * c8 + 0], v[8 * c8 + 1]);
            u.y = pack2(v[8 * c8 + 2], v[8 * c8 + 3]);
            u.z = pack2(v[8 * c8 + 4], v[8 * c8 + 5]);
            u.w = pack2(v[8 * c8 + 6], v[8 * c8 + 7]);
            *reinterpret_cast<uint4*>(act + swz(kRows, r, (uint32_t)(32 * q + 8 * c8))) = u;
        }
    }
}

// Forward pass over n rows (row i is tnf row idx[i], or i without idx): the
// embedding into z (FP32 [n][64]); with keep, the training outputs too.
__global__ void __launch_bounds__(kThreads, 1) k_mlp_fwd_tc(const float* __restrict__ tnf,
                                                             const uint32_t* __restrict__ idx, uint64_t n,
                                                             const float* __restrict__ P,
                                                             const unsigned char* __restrict__ wimg,
                                                             float* __restrict__ z, FwdKeep keep, int* flag) {
    extern __shared__ unsigned char smem_raw[];
    __shared__ MlpCtl ctl;
    __shared__ float mu[MLP_IN];
    unsigned char* smem = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    const uint32_t t = threadIdx.x, warp = t >> 5;
    for (uint32_t k = t; k < MLP_IN; k += kThreads) mu[k] = P[MLP_MU + k];
    Chain ch;
    ch.init(&ctl, smem, kActBytes, kTmemCols, flag);
    const uint32_t tmem_row = ch.tmem + ((warp * 32) << 16);
    const float scale = P[MLP_SCALE];
    const uint64_t tiles = (n + kRows - 1) / kRows;
    const bool train = keep.xT != nullptr;

    for (uint64_t tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
        const uint64_t r0 = tile * kRows;
        // stage the tile's rows: centred, scaled, BF16, K padded to 192
        // (granule g: row g % 128, K columns 8 * (g / 128) .. + 7)
        for (uint32_t gi = t; gi < kRows * kKc1 * 8; gi += kThreads) {
            const uint32_t r = gi % kRows, k = (gi / kRows) * 8;
            float e[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
            if (r0 + r < n && k < MLP_IN) {
                const uint64_t src_row = idx ? idx[r0 + r] : r0 + r;
                const float4* src = reinterpret_cast<const float4*>(tnf + src_row * MLP_IN + k);
                const float4 a = __ldg(src), b = __ldg(src + 1);
                e[0] = (a.x - mu[k + 0]) * scale;
                e[1] = (a.y - mu[k + 1]) * scale;
                e[2] = (a.z - mu[k + 2]) * scale;
                e[3] = (a.w - mu[k + 3]) * scale;
                e[4] = (b.x - mu[k + 4]) * scale;
                e[5] = (b.y - mu[k + 5]) * scale;
                e[6] = (b.z - mu[k + 6]) * scale;
                e[7] = (b.w - mu[k + 7]) * scale;
            }
            uint4 u;
            u.x = pack2(e[0], e[1]);
            u.y = pack2(e[2], e[3]);
            u.z = pack2(e[4], e[5]);
            u.w = pack2(e[6], e[7]);
            *reinterpret_cast<uint4*>(ch.act + swz(kRows, r, k)) = u;
            if (train)
#pragma unroll
                for (int j = 0; j < 8; ++j) keep.xT[(uint64_t)(k + j) * keep.ld + r0 + r] = bf(e[j]);
        }
        const uint64_t g = r0 + t;
        const bool valid = g < n;
        if (!ch.layer(kW1Bytes, wimg, kKc1, MLP_H1, 0, MLP_H1)) break;
        epi_hidden<MLP_H1 / 32>(tmem_row, 0, P + MLP_B1, ch.act, t, keep.z1, keep.h1T, keep.ld, g, valid);
        if (!ch.layer(kW2Bytes, wimg + kW1Bytes, kKc2, MLP_H2, 256, MLP_H2)) break;
        epi_hidden<MLP_H2 / 32>(tmem_row, 256, P + MLP_B2, ch.act, t, keep.z2, keep.h2T, keep.ld, g, valid);
        if (!ch.layer(kW3Bytes, wimg + kW1Bytes + kW2Bytes, kKc3, MLP_OUT, 384, MLP_OUT)) break;
        // the embedding: + b3, FP32 to global
#pragma unroll
        for (int q = 0; q < MLP_OUT / 32; ++q) {
            float v[32];
            tmem_ld32(tmem_row + 384 + 32 * q, v);
            if (valid) {
                float4* dst = reinterpret_cast<float4*>(z + g * MLP_OUT + 32 * q);
#pragma unroll
                for (int j = 0; j < 8; ++j) {
                    const int c = 32 * q + 4 * j;
                    dst[j] = make_float4(v[4 * j] + __ldg(P + MLP_B3 + c), v[4 * j + 1] + __ldg(P + MLP_B3 + c + 1),
                                         v[4 * j + 2] + __ldg(P + MLP_B3 + c + 2),
                                         v[4 * j + 3] + __ldg(P + MLP_B3 + c + 3));
                }
            }
        }
        fence_before();
        __syncthreads();  // the next tile overwrites the A operand and the accumulators
        fence_after();
    }
    ch.finish(kTmemCols);
}

// A backward layer's epilogue for this thread's row: columns [col0, col0 +
// 32 * NQ) of dH, times GELU' of the saved pre-activation zs (FP32 row) ->
// dZ: FP32 into dout (bias gradients), BF16 transposed into dT (weight
// gradients), and BF16 into the next A operand when act is non-null.  Rows
// at or past n give zeros.
template <int NQ>
__device__ __forceinline__ void epi_back(uint32_t tmem_row, uint32_t col0, const float* zs, float* dout,
                                         __nv_bfloat16* dT, uint64_t ld, unsigned char* act, uint32_t r, uint64_t g,
                                         bool valid) {
#pragma unroll 1
    for (int q = 0; q < NQ; ++q) {
        float v[32];
        tmem_ld32(tmem_row + col0 + 32 * q, v);
        if (valid) {
            const float4* zr = reinterpret_cast<const float4*>(zs + g * (NQ * 32) + 32 * q);
#pragma unroll
            for (int j = 0; j < 8; ++j) {
                const float4 zz = zr[j];
                v[4 * j] *= gelu_grad(zz.x);
                v[4 * j + 1] *= gelu_grad(zz.y);
                v[4 * j + 2] *= gelu_grad(zz.z);
                v[4 * j + 3] *= gelu_grad(zz.w);
            }
            float4* dd = reinterpret_cast<float4*>(dout + g * (NQ * 32) + 32 * q);
#pragma unroll
            for (int j = 0; j < 8; ++j) dd[j] = make_float4(v[4 * j], v[4 * j + 1], v[4 * j + 2], v[4 * j + 3]);
        } else {
#pragma unroll
            for (int j = 0; j < 32; ++j) v[j] = 0.f;
        }
#pragma unroll
        for (int j = 0; j < 32; ++j) dT[(uint64_t)(32 * q + j) * ld + g] = bf(v[j]);
        if (act) {
#pragma unroll
            for (int c8 = 0; c8 < 4; ++c8) {
                uint4 u;
                u.x = pack2(v[8 * c8 + 0], v[8 * c8 + 1]);
                u.y = pack2(v[8 * c8 + 2], v[8 * c8 + 3]);
                u.z = pack2(v[8 * c8 + 4], v[8 * c8 + 5]);
                u.w = pack2(v[8 * c8 + 6], v[8 * c8 + 7]);
                *reinterpret_cast<uint4*>(act + swz(kRows, r, (uint32_t)(32 * q + 8 * c8))) = u;
            }
        }
    }
}

// Backward of the two upper layers over ld rows (n of them real): from
// dZ3 (FP32 [ld][64]) to dZ2 and dZ1 (FP32, and BF16 transposed), dZ3^T too.
__global__ void __launch_bounds__(kThreads, 1) k_mlp_bwd_tc(const float* __restrict__ d3, uint64_t n, uint64_t ld,
                                                             const float* __restrict__ z1,
                                                             const float* __restrict__ z2,
                                                             const unsigned char* __restrict__ wimg,
                                                             float* __restrict__ d2, float* __restrict__ d1,
                                                             __nv_bfloat16* __restrict__ d3T,
                                                             __nv_bfloat16* __restrict__ d2T,
                                                             __nv_bfloat16* __restrict__ d1T, int* flag) {
    extern __shared__ unsigned char smem_raw[];
    __shared__ MlpCtl ctl;
    unsigned char* smem = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    const uint32_t t = threadIdx.x, warp = t >> 5;
    Chain ch;
    ch.init(&ctl, smem, kRows * 2 * 128, kTmemCols, flag);  // A: up to 128 K (dZ2)
    const uint32_t tmem_row = ch.tmem + ((warp * 32) << 16);
    const unsigned char* w3t = wimg + kW1Bytes + kW2Bytes + kW3Bytes;
    const unsigned char* w2t = w3t + kW3tBytes;
    const uint64_t tiles = (ld + kRows - 1) / kRows;
    for (uint64_t tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
        const uint64_t r0 = tile * kRows;
        // stage dZ3 as BF16 (K = 64), and dZ3^T
        for (uint32_t gi = t; gi < kRows * 8; gi += kThreads) {
            const uint32_t r = gi % kRows, k = (gi / kRows) * 8;
            float e[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
            if (r0 + r < n) {
                const float4* src = reinterpret_cast<const float4*>(d3 + (r0 + r) * MLP_OUT + k);
                const float4 a = src[0], b = src[1];
                e[0] = a.x, e[1] = a.y, e[2] = a.z, e[3] = a.w, e[4] = b.x, e[5] = b.y, e[6] = b.z, e[7] = b.w;
            }
            uint4 u;
            u.x = pack2(e[0], e[1]);
            u.y = pack2(e[2], e[3]);
            u.z = pack2(e[4], e[5]);
            u.w = pack2(e[6], e[7]);
            *reinterpret_cast<uint4*>(ch.act + swz(kRows, r, k)) = u;
#pragma unroll
            for (int j = 0; j < 8; ++j) d3T[(uint64_t)(k + j) * ld + r0 + r] = bf(e[j]);
        }
        const uint64_t g = r0 + t;
        const bool valid = g < n;
        // dH2 = dZ3 W3 (N = 128, K = 64)
        if (!ch.layer(kW3tBytes, w3t, 1, MLP_H2, 0, MLP_H2)) break;
        epi_back<MLP_H2 / 32>(tmem_row, 0, z2, d2, d2T, ld, ch.act, t, g, valid);
        // dH1 = dZ2 W2 (N = 256, K = 128)
        if (!ch.layer(kW2tBytes, w2t, 2, MLP_H1, 256, MLP_H1)) break;
        epi_back<MLP_H1 / 32>(tmem_row, 256, z1, d1, d1T, ld, nullptr, t, g, valid);
        fence_before();
        __syncthreads();
        fence_after();
    }
    ch.finish(kTmemCols);
}

// Weight gradient dW[m][c] += sum_k A[m][k] B[c][k] for m < M, c < nout:
// A = dZ^T ([M][ld] BF16), B = H^T ([nb][ld] BF16, rows nb .. nn - 1 read as
// zeros), over this CTA's K range [k0, k0 + kspan) of the ld rows; a 128-row
// block of dW per blockIdx.x (M = 64 fills the block's lower half, the rest
// zeros), nn (a multiple of 16, <= 256) accumulator columns.
__global__ void __launch_bounds__(kThreads, 1) k_mlp_dw_tc(const __nv_bfloat16* __restrict__ A, uint32_t M,
                                                            const __nv_bfloat16* __restrict__ B, uint32_t nb,
                                                            uint32_t nn, uint32_t nout, uint64_t ld, uint64_t kspan,
                                                            float* __restrict__ dW, int* flag) {
    extern __shared__ unsigned char smem_raw[];
    __shared__ MlpCtl ctl;
    unsigned char* smem = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    unsigned char* sA = smem;                 // 128 rows x 64 K
    unsigned char* sB = smem + kChunkA;       // nn rows x 64 K
    const uint32_t t = threadIdx.x, warp = t >> 5;
    if (t == 0) {
        mbar_init(&ctl.mma_done, 1);
        mbar_fence_init();
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&ctl.tmem_base)),
                     "r"(256u)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    fence_before();
    __syncthreads();
    fence_after();
    const uint32_t tmem = ctl.tmem_base;
    const uint32_t m0 = blockIdx.x * kRows;
    const uint64_t k0 = blockIdx.y * kspan, k1 = min(ld, k0 + kspan);
    const uint32_t sa = smem_u32(sA), sb = smem_u32(sB);
    uint32_t ph = 0;
    bool ok = true, any = false;
    for (uint64_t kc = k0; kc < k1; kc += 64) {
        // stage the K chunk [kc, kc + 64) of A's 128 rows and B's nn rows
        for (uint32_t gi = t; gi < (kRows + nn) * 8; gi += kThreads) {
            const uint32_t row = gi >> 3, kg = (gi & 7) * 8;
            uint4 u = make_uint4(0, 0, 0, 0);
            if (row < kRows) {
                if (m0 + row < M && kc + kg < k1)
                    u = *reinterpret_cast<const uint4*>(A + (uint64_t)(m0 + row) * ld + kc + kg);
                *reinterpret_cast<uint4*>(sA + swz(kRows, row, kg)) = u;
            } else {
                const uint32_t c = row - kRows;
                if (c < nb && kc + kg < k1) u = *reinterpret_cast<const uint4*>(B + (uint64_t)c * ld + kc + kg);
                *reinterpret_cast<uint4*>(sB + swz(nn, c, kg)) = u;
            }
        }
        fence_proxy_async_smem();
        fence_before();
        __syncthreads();
        fence_after();
        if (t == 0) {
            for (int s = 0; s < 4; ++s)
                mma_bf16(tmem, desc_sw128(sa + s * 32), desc_sw128(sb + s * 32), idesc(nn), (any || s > 0) ? 1u : 0u);
            mma_commit(&ctl.mma_done);
        }
        any = true;
        const bool w = mbar_wait(&ctl.mma_done, ph, flag);
        ph ^= 1;
        fence_after();
        if (__syncthreads_or(!w)) {
            ok = false;
            break;
        }
    }
    if (ok && any) {
        const uint32_t tmem_row = tmem + ((warp * 32) << 16);
        const uint32_t m = m0 + t;
#pragma unroll 1
        for (uint32_t q = 0; q * 32 < nn; ++q) {
            float v[32];
            tmem_ld32(tmem_row + 32 * q, v);
            if (m < M)
#pragma unroll
                for (int j = 0; j < 32; ++j) {
                    const uint32_t c = 32 * q + j;
                    if (c < nout) atomicAdd(dW + (uint64_t)m * nout + c, v[j]);
                }
        }
    }
    fence_before();
    __syncthreads();
    fence_after();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(256u) : "memory");
}

__global__ void k_colsum_tc(const float* __restrict__ d, uint64_t rows, int cols, float* __restrict__ g) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= cols) return;
    const uint64_t r0 = blockIdx.y * 256ull, r1 = min(rows, r0 + 256);
    float s = 0.f;
    for (uint64_t r = r0; r < r1; ++r) s += d[r * cols + c];
    atomicAdd(&g[c], s);
}

int weight_images(mdet_ctx* ctx, const float* P, unsigned char** img) {
    *img = (unsigned char*)ctx_scratch(ctx, "mlptc.wimg", kImgBytes);
    if (!*img) return MDET_ERR_NOMEM;
    const uint32_t nel = kImgBytes / 2;
    k_mlp_wimage<<<(nel + 255) / 256, 256, 0, ctx->stream>>>(P, *img);
    MDET_LAUNCHED(ctx, "k_mlp_wimage");
    return MDET_OK;
}

int set_attrs(mdet_ctx* ctx) {
    static bool attr[64] = {false};
    if (!attr[ctx->device & 63]) {
        MDET_CUDA(ctx, cudaFuncSetAttribute(k_mlp_fwd_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmem));
        MDET_CUDA(ctx, cudaFuncSetAttribute(k_mlp_bwd_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmemBwd));
        MDET_CUDA(ctx, cudaFuncSetAttribute(k_mlp_dw_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmemDw));
        attr[ctx->device & 63] = true;
    }
    return MDET_OK;
}

int fwd_launch(mdet_ctx* ctx, const float* P, const unsigned char* img, const float* tnf, const uint32_t* idx,
               uint64_t n, float* z, const FwdKeep& keep) {
    const uint64_t tiles = (n + kRows - 1) / kRows;
    const unsigned grid = (unsigned)std::min<uint64_t>(tiles, (uint64_t)ctx->num_sms);
    ctx_timer_begin(ctx, "k_mlp_fwd_tc");
    k_mlp_fwd_tc<<<grid, kThreads, kSmem, ctx->stream>>>(tnf, idx, n, P, img, z, keep, ctx->d_flag);
    MDET_LAUNCHED(ctx, "k_mlp_fwd_tc");
    ctx_timer_end(ctx, "k_mlp_fwd_tc");
    return MDET_OK;
}

}  // namespace

// Embeddings of n rows on the tensor cores (rows idx[i] of tnf when idx is
// non-null): z (n x 64).
int mlp_embed_tc(mdet_ctx* ctx, const float* P, const float* tnf, uint64_t n, float* z, const uint32_t* idx) {
    if (n == 0) return MDET_OK;
    MDET_TRY(set_attrs(ctx));
    unsigned char* img = nullptr;
    MDET_TRY(weight_images(ctx, P, &img));
    return fwd_launch(ctx, P, img, tnf, idx, n, z, FwdKeep{nullptr, nullptr, nullptr, nullptr, nullptr, 0});
}

int mlp_tc_alloc(mdet_ctx* ctx, const char* tag, uint64_t rows, MlpTcActs* a) {
    const uint64_t ld = (rows + kRows - 1) / kRows * kRows;
    std::string t(tag);
    auto f = [&](const char* nm, uint64_t cols) { return (float*)ctx_scratch(ctx, (t + nm).c_str(), ld * cols * 4); };
    auto h = [&](const char* nm, uint64_t feats) {
        return (__nv_bfloat16*)ctx_scratch(ctx, (t + nm).c_str(), ld * feats * 2);
    };
    a->ld = ld;
    a->z1 = f(".z1", MLP_H1);
    a->z2 = f(".z2", MLP_H2);
    a->z3 = f(".z3", MLP_OUT);
    a->d3 = f(".d3", MLP_OUT);
    a->d2 = f(".d2", MLP_H2);
    a->d1 = f(".d1", MLP_H1);
    a->xT = h(".xT", 64 * kKc1);
    a->h1T = h(".h1T", MLP_H1);
    a->h2T = h(".h2T", MLP_H2);
    a->d3T = h(".d3T", MLP_OUT);
    a->d2T = h(".d2T", MLP_H2);
    a->d1T = h(".d1T", MLP_H1);
    return (a->z1 && a->z2 && a->z3 && a->d3 && a->d2 && a->d1 && a->xT && a->h1T && a->h2T && a->d3T && a->d2T &&
            a->d1T)
               ? MDET_OK
               : MDET_ERR_NOMEM;
}

int mlp_forward_tc(mdet_ctx* ctx, const float* P, const float* tnf, const uint32_t* idx, uint64_t rows,
                   const MlpTcActs& a) {
    if (rows == 0) return MDET_OK;
    MDET_TRY(set_attrs(ctx));
    unsigned char* img = nullptr;
    MDET_TRY(weight_images(ctx, P, &img));
    return fwd_launch(ctx, P, img, tnf, idx, rows, a.z3, FwdKeep{a.z1, a.z2, a.xT, a.h1T, a.h2T, a.ld});
}

int mlp_backward_tc(mdet_ctx* ctx, const float* P, const MlpTcActs& a, uint64_t np, const float* labels, float m_pos,
                    float m_neg, float* grad, double* loss_sum) {
    cudaStream_t s = ctx->stream;
    const uint64_t rows = 2 * np, ld = a.ld;
    if (np == 0) return MDET_OK;
    MDET_TRY(set_attrs(ctx));
    const unsigned char* img = (const unsigned char*)ctx_scratch(ctx, "mlptc.wimg", kImgBytes);  // from the forward
    MDET_CUDA(ctx, cudaMemsetAsync(grad, 0, MLP_NTRAIN * 4, s));
    MDET_CUDA(ctx, cudaMemsetAsync(a.d3, 0, ld * MLP_OUT * 4, s));
    MDET_TRY(mlp_pair_loss(ctx, a.z3, np, labels, m_pos, m_neg, a.d3, loss_sum));
    const uint64_t tiles = ld / kRows;
    const unsigned grid = (unsigned)std::min<uint64_t>(tiles, (uint64_t)ctx->num_sms);
    k_mlp_bwd_tc<<<grid, kThreads, kSmemBwd, s>>>(a.d3, rows, ld, a.z1, a.z2, img, a.d2, a.d1, a.d3T, a.d2T, a.d1T,
                                                   ctx->d_flag);
    MDET_LAUNCHED(ctx, "k_mlp_bwd_tc");
    // weight gradients: K = the ld rows in spans of 512 rows per CTA
    const uint64_t kspan = 512;
    const unsigned ks = (unsigned)((ld + kspan - 1) / kspan);
    struct Dw {
        const __nv_bfloat16* A;
        uint32_t M;
        const __nv_bfloat16* B;
        uint32_t nb, nn, nout;
        float* out;
    } dws[3] = {
        {a.d3T, MLP_OUT, a.h2T, MLP_H2, MLP_H2, MLP_H2, grad + MLP_W3},
        {a.d2T, MLP_H2, a.h1T, MLP_H1, MLP_H1, MLP_H1, grad + MLP_W2},
        {a.d1T, MLP_H1, a.xT, 64 * kKc1, 144, MLP_IN, grad + MLP_W1},  // K = 136 padded to 144 columns
    };
    for (const Dw& d : dws) {
        dim3 g((d.M + kRows - 1) / kRows, ks);
        k_mlp_dw_tc<<<g, kThreads, kSmemDw, s>>>(d.A, d.M, d.B, d.nb, d.nn, d.nout, ld, kspan, d.out, ctx->d_flag);
        MDET_LAUNCHED(ctx, "k_mlp_dw_tc");
    }
    // bias gradients: column sums of the FP32 output gradients
    const dim3 cg(1, (unsigned)((rows + 255) / 256));
    k_colsum_tc<<<cg, MLP_OUT, 0, s>>>(a.d3, rows, MLP_OUT, grad + MLP_B3);
    MDET_LAUNCHED(ctx, "k_colsum_tc");
    k_colsum_tc<<<cg, MLP_H2, 0, s>>>(a.d2, rows, MLP_H2, grad + MLP_B2);
    MDET_LAUNCHED(ctx, "k_colsum_tc");
    k_colsum_tc<<<cg, MLP_H1, 0, s>>>(a.d1, rows, MLP_H1, grad + MLP_B1);
    MDET_LAUNCHED(ctx, "k_colsum_tc");
    return MDET_OK;
}
