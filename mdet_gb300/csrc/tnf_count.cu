// tnf_count.cu -- K1: per-contig tetranucleotide counting + normalisation.
//
// Semantics of the reference host loop (cuda/Cuda2.cu:1825-1853, next_contig
// and get_tn at 317-339): a window of the last four non-newline characters
// slides over the sequence view; a window is counted when all four are
// A/C/G/T (either case); the counted raw 4-mer (A=0,C=1,T=2,G=3, oldest base
// in the high bits) is folded onto one of 136 canonical columns.  Counts are
// exact integers; TNF = float(c / sqrt(sum float(c*c))).
//
// GB300 layout: the sequence bytes sit in HBM exactly as the FASTA reader
// left them (newlines included).  Work is cut into pieces of <= 64 KB of
// one contig; each warp takes pieces from a global counter, and each lane
// walks a contiguous 1/32 of the piece with its own rolling state
// (16-byte loads, the next one in flight), warmed up on the bytes just
// before its run, so no lane depends on another while it counts.  The
// 16-byte chunks at the two ends of a lane's run are clipped by turning the
// bytes outside the run into newlines (no state change, nothing counted), so
// every chunk goes through the same branch-free 16-byte step.  Windows go
// into the warp's 256-bin shared histogram of raw 8-bit codes, folded onto
// the 136 canonical columns per piece.  A contig cut into several pieces
// accumulates into a per-contig scratch row and the last piece to finish
// normalises it (and clears the scratch row).  Normalisation runs in FP32
// (float-float square root and reciprocal of the exact integer square sum):
// no FP64 on the counting path.
#include <cub/cub.cuh>

#include <mutex>
#include <vector>

#include "common.cuh"

namespace {

constexpr int kWarps = 8;
constexpr uint64_t kPiece = 65536;  // bytes per piece
constexpr uint32_t kPoison = 0xFF00u;

struct FoldTables {
    uint8_t fw[MDET_NTNF];
    uint8_t rc[MDET_NTNF];
};

// Pieces per contig, checked before anything is sized from them: a view
// outside [0, nbytes) counts in status[1] (and gets one piece, so nothing
// downstream grows from garbage lengths), and status[0] receives the 64-bit
// piece total, which the host compares with its limits before the uint32 scan
// of npieces is used.  status must be zero on entry.
__global__ void k_piece_counts(const uint64_t* __restrict__ off, const uint64_t* __restrict__ len, uint64_t n,
                               uint64_t nbytes, uint32_t* __restrict__ npieces,
                               unsigned long long* __restrict__ status) {
    uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    uint64_t np = 0, bad = 0;
    if (i < n) {
        const uint64_t L = len[i], o = off[i];
        if (o > nbytes || L > nbytes - o) {
            bad = 1;
            np = 1;
        } else {
            np = L == 0 ? 1 : L / kPiece + (L % kPiece != 0);  // <= 2^48: no overflow
        }
        npieces[i] = (uint32_t)min(np, (uint64_t)0xFFFFFFFFu);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        np += __shfl_xor_sync(0xffffffffu, np, o);
        bad += __shfl_xor_sync(0xffffffffu, bad, o);
    }
    if ((threadIdx.x & 31) == 0 && np) {
        atomicAdd(&status[0], (unsigned long long)np);
        if (bad) atomicAdd(&status[1], (unsigned long long)bad);
    }
}

__global__ void k_piece_map(const uint32_t* __restrict__ npieces, const uint32_t* __restrict__ start, uint64_t n,
                            uint32_t* __restrict__ piece_contig) {
    uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    uint32_t s = start[i], np = npieces[i];
    for (uint32_t k = 0; k < np; ++k) piece_contig[s + k] = (uint32_t)i;
}

__device__ __forceinline__ uint64_t warp_sum_u64(uint64_t v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// 1/sqrt(s) of an exact integer s < 2^53 as a float-float pair ih + il
// (about 46 significant bits) from FP32 arithmetic alone: one Newton step on
// the square root from sqrtf of its leading float, then one on the
// reciprocal, with the residuals formed exactly by FMA.
__device__ __forceinline__ void inv_sqrt_ff(uint64_t s, float& ih, float& il) {
    const float sh = __ull2float_rn(s);
    const float sl = (float)(long long)(s - (unsigned long long)sh);  // s - sh, exact to ~2^-24 of itself
    const float r0 = __fsqrt_rn(sh);
    const float ph = __fmul_rn(r0, r0), pl = __fmaf_rn(r0, r0, -ph);
    const float res = __fadd_rn(__fadd_rn(__fsub_rn(sh, ph), -pl), sl);  // s - r0^2
    const float r1 = __fdiv_rn(res, __fmul_rn(2.0f, r0));              // r = r0 + r1
    const float q0 = __fdiv_rn(1.0f, r0);
    const float e = __fsub_rn(__fmaf_rn(-r0, q0, 1.0f), __fmul_rn(r1, q0));  // 1 - r q0
    ih = q0;
    il = __fmul_rn(q0, e);
}

// Writes one finished contig row from per-lane canonical counts: counts, then
// float(c / sqrt(sum float(c*c))).  The square sum is exact (integers
// < 2^53); c * (ih + il) is formed in float-float and rounded once to float.
__device__ __forceinline__ void finish_row(uint32_t lane, const uint32_t (&v)[5], uint64_t c,
                                           uint32_t* __restrict__ counts, float* __restrict__ tnf) {
    uint64_t s = 0;
#pragma unroll
    for (int j = 0; j < 5; ++j) {
        uint32_t col = lane + 32 * j;
        if (col < MDET_NTNF) {
            float f = (float)v[j];
            float sq = __fmul_rn(f, f);  // the reference squares in float
            s += (uint64_t)sq;           // integers < 2^53: exact in any order
        }
    }
    s = warp_sum_u64(s);
    float ih = 0.f, il = 0.f;
    if (s) inv_sqrt_ff(s, ih, il);
#pragma unroll
    for (int j = 0; j < 5; ++j) {
        uint32_t col = lane + 32 * j;
        if (col < MDET_NTNF) {
            const float f = (float)v[j];
            const float p = __fmul_rn(f, ih);
            const float e = __fmaf_rn(f, il, __fmaf_rn(f, ih, -p));
            counts[c * MDET_NTNF + col] = v[j];
            tnf[c * MDET_NTNF + col] = s ? __fadd_rn(p, e) : __int_as_float(0x7fffffff);
        }
    }
}

// One byte of the rolling state.  x: codes of the last four non-newline
// characters (2 bits each, newest lowest) in bits 0-7 and their poison bits
// (not a base) in bits 8-15; u = lut[byte].  A newline leaves x unchanged
// (the reference overwrites the window's oldest slot instead of shifting, so
// the window spanning a line break is still counted); t >= 256 marks a
// window that is not counted (poisoned, or the newline itself).
__device__ __forceinline__ uint32_t roll(uint32_t x, uint32_t u, uint32_t& t) {
    t = ((x << 2) & 0xFCFCu) | u;
    return u >= 0x8000u ? x : t;
}

__device__ __forceinline__ uint32_t byte_of(const uint4& v, int b) {
    const uint32_t w = b < 4 ? v.x : (b < 8 ? v.y : (b < 12 ? v.z : v.w));
    return __byte_perm(w, 0u, 0x4440u | (uint32_t)(b & 3));
}

// Bytes of the 16-byte chunk at q that lie outside [a, b) become '\n': a
// newline leaves the rolling state alone and counts nowhere, so a run starts
// from its warm-up state at a and stops counting at b.
__device__ __forceinline__ void clip_chunk(uint4& v, uint64_t q, uint64_t a, uint64_t b) {
    const uint32_t lo = q < a ? (uint32_t)(a - q) : 0u;
    const uint32_t hi = q >= b ? 0u : (q + 16 <= b ? 16u : (uint32_t)(b - q));
    const uint32_t keep = hi > lo ? (((1u << hi) - 1u) & ~((1u << lo) - 1u)) : 0u;
    uint32_t* w = reinterpret_cast<uint32_t*>(&v);
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        const uint32_t bits = (keep >> (4 * j)) & 0xFu;
        const uint32_t bm = ((bits * 0x00204081u) & 0x01010101u) * 0xFFu;  // 4 bits -> 4 byte masks
        w[j] = (w[j] & bm) | (0x0A0A0A0Au & ~bm);
    }
}

// Warp per piece (<= 64 KB of one contig, taken from a global counter);
// lane l walks its 1/32 of the piece in order with its own rolling state,
// warmed up on the bytes just before its run, and counts each window that
// ends in its run into the warp's shared histogram of raw 8-bit codes.  No
// lane waits on another until the piece is folded.
__global__ void __launch_bounds__(kWarps * 32) k_count(const unsigned char* __restrict__ bytes,
                                                      const uint64_t* __restrict__ off,
                                                      const uint64_t* __restrict__ len, uint64_t n,
                                                      const uint32_t* __restrict__ piece_start,
                                                      const uint32_t* __restrict__ npieces,
                                                      const uint32_t* __restrict__ piece_contig, uint32_t total,
                                                      uint32_t* __restrict__ work, uint32_t* __restrict__ acc,
                                                      uint32_t* __restrict__ done, uint32_t* __restrict__ counts,
                                                      float* __restrict__ tnf, FoldTables tabs, int* flag) {
    __shared__ uint32_t hist_all[kWarps][257];  // 256 raw 4-mer codes + a bin for windows not counted
    // byte -> update word: 2-bit base code | 0x300 when not a base | 0x8000 for '\n'
    __shared__ uint16_t lut[256];
    const uint32_t w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    uint32_t* hist = hist_all[w];
    for (uint32_t c = threadIdx.x; c < 256; c += blockDim.x) {
        const uint32_t u = (c | 0x20u) - 0x61u;
        const uint32_t valid = (u < 20u) ? ((0x80045u >> u) & 1u) : 0u;
        lut[c] = (uint16_t)(c == '\n' ? 0x8000u : (((c >> 1) & 3u) | (valid ? 0u : 0x300u)));
    }
    __syncthreads();

    while (true) {
        // the next piece (lane 0) and the abort flag (lane 1) load side by side
        uint32_t p = 0;
        int stop = 0;
        if (lane == 0) p = atomicAdd(work, 1u);
        else if (lane == 1) stop = *(volatile int*)flag;
        p = __shfl_sync(0xffffffffu, p, 0);
        stop = __shfl_sync(0xffffffffu, stop, 1);
        if (p >= total || stop) break;
        const uint64_t c = piece_contig[p];
        const uint32_t k = p - piece_start[c];
        const uint64_t s0 = off[c], L = len[c];
        const uint64_t p0 = s0 + (uint64_t)k * kPiece;
        const uint64_t p1 = min(s0 + L, p0 + kPiece);

        for (int i = lane; i < 257; i += 32) hist[i] = 0;
        __syncwarp();

        // the piece is split evenly over the 32 lanes in runs of whole 16-byte
        // chunks (so every lane's run starts at the same offset mod 16)
        const uint64_t run = max((uint64_t)16, (((p1 - p0) + 31) / 32 + 15) & ~(uint64_t)15);
        const uint64_t seg0 = p0 + (uint64_t)lane * run;
        const uint64_t seg1 = min(p1, seg0 + run);
        if (seg0 < seg1) {
            // warm-up: the state after the last three non-newline bytes before
            // seg0 (none before s0).  Fast case: the four bytes before seg0
            // hold at most one newline; else walk back byte by byte.
            uint32_t x = kPoison, t;
            bool warm = false;
            if (seg0 >= s0 + 4) {
                const uint64_t q = seg0 - 4;
                const uint32_t* wp = reinterpret_cast<const uint32_t*>(bytes + (q & ~(uint64_t)3));
                const uint32_t four = __funnelshift_r(__ldg(wp), __ldg(wp + 1), 8u * (uint32_t)(q & 3));
                const uint32_t z = four ^ 0x0A0A0A0Au;
                const uint32_t nl = ~(((z & 0x7F7F7F7Fu) + 0x7F7F7F7Fu) | z) & 0x80808080u;
                if (__popc(nl) <= 1) {
#pragma unroll
                    for (int b = 0; b < 4; ++b) x = roll(x, lut[(four >> (8 * b)) & 0xFFu], t);
                    warm = true;
                }
            }
            if (!warm) {
                uint64_t ws = seg0;
                int need = 3;
                while (need > 0 && ws > s0) {
                    --ws;
                    if (bytes[ws] != '\n') --need;
                }
                for (uint64_t q = ws; q < seg0; ++q) x = roll(x, lut[bytes[q]], t);
            }
            // counting pass over aligned 16-byte chunks, the next one in
            // flight; chunks at the ends of the run are clipped to it
            const uint64_t a0 = seg0 & ~(uint64_t)15;
            const uint32_t nch = (uint32_t)((seg1 - a0 + 15) >> 4);
            const unsigned char* ptr = bytes + a0;
            uint4 nxt = __ldg(reinterpret_cast<const uint4*>(ptr));
            for (uint32_t i = 0; i < nch; ++i) {
                uint4 v = nxt;
                if (i + 1 < nch) nxt = __ldg(reinterpret_cast<const uint4*>(ptr + 16 * (i + 1)));
                const uint64_t q = a0 + 16ull * i;
                if (q < seg0 || q + 16 > seg1) clip_chunk(v, q, seg0, seg1);
#pragma unroll
                for (int b = 0; b < 16; ++b) {
                    x = roll(x, lut[byte_of(v, b)], t);
                    atomicAdd(&hist[min(t, 256u)], 1u);  // bin 256 takes the windows not counted
                }
            }
        }
        __syncwarp();
        uint32_t v[5];
#pragma unroll
        for (int j = 0; j < 5; ++j) {
            uint32_t col = lane + 32 * j;
            v[j] = 0;
            if (col < MDET_NTNF) {
                uint32_t f = tabs.fw[col], r = tabs.rc[col];
                v[j] = hist[f] + (r != f ? hist[r] : 0u);
            }
        }
        const uint32_t np = npieces[c];
        if (np == 1) {
            finish_row(lane, v, c, counts, tnf);
        } else {
#pragma unroll
            for (int j = 0; j < 5; ++j) {
                uint32_t col = lane + 32 * j;
                if (col < MDET_NTNF && v[j]) atomicAdd(&acc[c * MDET_NTNF + col], v[j]);
            }
            __threadfence();
            __syncwarp();
            uint32_t prev = 0;
            if (lane == 0) prev = atomicAdd(&done[c], 1u);
            prev = __shfl_sync(0xffffffffu, prev, 0);
            if (prev == np - 1) {
                __threadfence();
#pragma unroll
                for (int j = 0; j < 5; ++j) {
                    uint32_t col = lane + 32 * j;
                    if (col < MDET_NTNF) {
                        v[j] = __ldcg(&acc[c * MDET_NTNF + col]);
                        acc[c * MDET_NTNF + col] = 0;
                    }
                }
                if (lane == 0) done[c] = 0;
                finish_row(lane, v, c, counts, tnf);
            }
        }
        __syncwarp();
    }
}

}  // namespace

// Device scratch of one count.
struct CountScratch {
    uint32_t *npieces, *start, *pmap, *work, *acc, *done;
    unsigned long long* status;  // [0] piece total, [1] views outside the buffer
    void* cub_tmp;
    size_t cub_bytes;
};

static size_t count_cub_bytes(uint64_t n, cudaStream_t s) {
    size_t a = 0;
    cub::DeviceScan::ExclusiveSum(nullptr, a, (uint32_t*)nullptr, (uint32_t*)nullptr, (int)n, s);
    return a;
}

// Phase 1 of a count: pieces per contig and the view check (status), piece
// starts; the caller reads status back and checks it before phase 2.
static cudaError_t count_phase1(const CountScratch& S, const uint64_t* d_off, const uint64_t* d_len, uint64_t n,
                                uint64_t nbytes, cudaStream_t s) {
    cudaError_t e = cudaMemsetAsync(S.status, 0, 16, s);
    if (e != cudaSuccess) return e;
    const unsigned blocks = (unsigned)((n + 255) / 256);
    k_piece_counts<<<blocks, 256, 0, s>>>(d_off, d_len, n, nbytes, S.npieces, S.status);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    size_t tb = S.cub_bytes;
    return cub::DeviceScan::ExclusiveSum(S.cub_tmp, tb, S.npieces, S.start, (int)n, s);
}

// Phase 2: piece map and the counting kernel.
static cudaError_t count_phase2(const CountScratch& S, const unsigned char* d_bytes, const uint64_t* d_off,
                                const uint64_t* d_len, uint64_t n, uint32_t total, uint32_t* d_counts, float* d_tnf,
                                int* flag, int grid, cudaStream_t s) {
    const unsigned blocks = (unsigned)((n + 255) / 256);
    k_piece_map<<<blocks, 256, 0, s>>>(S.npieces, S.start, n, S.pmap);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    if ((e = cudaMemsetAsync(S.work, 0, 4, s)) != cudaSuccess) return e;
    FoldTables tabs;
    const TnTables& t = tn_tables();
    memcpy(tabs.fw, t.col_fw, MDET_NTNF);
    memcpy(tabs.rc, t.col_rc, MDET_NTNF);
    k_count<<<grid, kWarps * 32, 0, s>>>(d_bytes, d_off, d_len, n, S.start, S.npieces, S.pmap, total, S.work, S.acc,
                                         S.done, d_counts, d_tnf, tabs, flag);
    return cudaGetLastError();
}

static int k_count_grid(int num_sms) {
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_count, kWarps * 32, 0);
    return num_sms * (per_sm < 1 ? 1 : per_sm);
}

static int count_impl(mdet_ctx* ctx, const char* d_bytes, uint64_t nbytes, const uint64_t* d_off,
                      const uint64_t* d_len, uint64_t n, uint32_t* d_counts, float* d_tnf) {
    if (n == 0) return MDET_OK;
    if (n >= 0xFFFFFFFFull) return ctx_fail(ctx, MDET_ERR_INVALID, "too many contigs (%llu)", (unsigned long long)n);
    ctx->prep_cache.valid = false;  // new TNF rows: no preparation carries over past a count
    if (((uintptr_t)d_bytes & 15) != 0)
        return ctx_fail(ctx, MDET_ERR_INVALID, "sequence buffer must be 16-byte aligned");
    cudaStream_t s = ctx->stream;
    CountScratch S{};
    S.npieces = (uint32_t*)ctx_scratch(ctx, "cnt.np", n * 4);
    S.start = (uint32_t*)ctx_scratch(ctx, "cnt.start", n * 4);
    S.work = (uint32_t*)ctx_scratch(ctx, "cnt.work", 32);  // piece counter; status (2 x u64) at +8
    // per-contig accumulators for multi-piece contigs: zero when grown, and
    // every finishing warp clears its row again, so they stay zero between calls
    if (ctx->count_scratch_dirty) {
        ctx->bufs.erase("cnt.acc");
        ctx->bufs.erase("cnt.done");
        ctx->count_scratch_dirty = false;
    }
    S.acc = (uint32_t*)ctx_scratch(ctx, "cnt.acc", n * MDET_NTNF * 4, true);
    S.done = (uint32_t*)ctx_scratch(ctx, "cnt.done", n * 4, true);
    if (!S.npieces || !S.start || !S.work || !S.acc || !S.done) return MDET_ERR_NOMEM;
    S.status = (unsigned long long*)(S.work + 2);
    S.cub_bytes = count_cub_bytes(n, s);
    S.cub_tmp = ctx_scratch(ctx, "cnt.cubtmp", S.cub_bytes);
    if (!S.cub_tmp) return MDET_ERR_NOMEM;
    MDET_CUDA(ctx, count_phase1(S, d_off, d_len, n, nbytes, s));
    MDET_LAUNCHED(ctx, "k_piece_counts");
    // exact piece total in 64 bits (contig views may overlap, so it is not
    // bounded by nbytes) and the number of views outside the buffer
    unsigned long long st[2] = {0, 0};
    MDET_CUDA(ctx, cudaMemcpyAsync(st, S.status, 16, cudaMemcpyDeviceToHost, s));
    MDET_CUDA(ctx, cudaStreamSynchronize(s));
    if (st[1]) return ctx_fail(ctx, MDET_ERR_INVALID, "%llu contig view(s) lie outside the byte buffer", st[1]);
    if (st[0] > 0xFFFFFFFFull)
        return ctx_fail(ctx, MDET_ERR_CAPACITY, "%llu 64-KB pieces of sequence (views overlap too much)", st[0]);
    S.pmap = (uint32_t*)ctx_scratch(ctx, "cnt.pmap", (size_t)st[0] * 4);
    if (!S.pmap) return MDET_ERR_NOMEM;
    ctx_timer_begin(ctx, "k_count");
    MDET_CUDA(ctx, count_phase2(S, (const unsigned char*)d_bytes, d_off, d_len, n, (uint32_t)st[0], d_counts, d_tnf,
                                ctx->d_flag, k_count_grid(ctx->num_sms), s));
    ctx_timer_end(ctx, "k_count");
    MDET_LAUNCHED(ctx, "k_count");
    return MDET_OK;
}

static int check_flag(mdet_ctx* ctx) {
    int h = 0;
    MDET_CUDA(ctx, cudaMemcpyAsync(&h, ctx->d_flag, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    MDET_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    if (h) {
        cudaMemsetAsync(ctx->d_flag, 0, sizeof(int), ctx->stream);
        ctx->count_scratch_dirty = true;
        return ctx_fail(ctx, MDET_ERR_TIMEOUT, "a bounded device wait ran out (flag %d)", h);
    }
    return MDET_OK;
}

extern "C" {

int mdet_tnf_count_dev(mdet_ctx* ctx, const char* d_bytes, uint64_t nbytes, const uint64_t* d_off,
                       const uint64_t* d_len, uint64_t n, uint32_t* d_counts, float* d_tnf) {
    if (!ctx) return MDET_ERR_INVALID;
    if (n && (!d_bytes || !d_off || !d_len || !d_counts || !d_tnf))
        return ctx_fail(ctx, MDET_ERR_INVALID, "null pointer");
    MDET_CUDA(ctx, cudaSetDevice(ctx->device));
    ctx->launches = 0;
    int rc = count_impl(ctx, d_bytes, nbytes, d_off, d_len, n, d_counts, d_tnf);
    if (rc != MDET_OK) {
        ctx->count_scratch_dirty = true;
        return rc;
    }
    return check_flag(ctx);
}

// Chunked host-buffer path of mdet_tnf_count (file-order views, see there).
static int count_chunked(mdet_ctx* ctx, const char* bytes, uint64_t nbytes, const uint64_t* off, const uint64_t* len,
                         uint64_t n, uint32_t* counts, float* tnf, char* d_bytes, const uint64_t* d_off,
                         const uint64_t* d_len, uint32_t* d_counts, float* d_tnf) {
    cudaStream_t s = ctx->stream;
    if (!ctx->io_in) MDET_CUDA(ctx, cudaStreamCreateWithFlags(&ctx->io_in, cudaStreamNonBlocking));
    if (!ctx->io_out) MDET_CUDA(ctx, cudaStreamCreateWithFlags(&ctx->io_out, cudaStreamNonBlocking));
    const uint64_t target = (uint64_t)1 << 30;
    // chunk k: contigs [cs[k], cs[k+1]), bytes [bs[k], bs[k+1]) (the chunks tile the buffer)
    std::vector<uint64_t> cs{0}, bs{0};
    for (uint64_t i = 0; i < n; ++i) {
        const uint64_t end = off[i] + len[i];
        if (end - bs.back() >= target && i + 1 < n) {
            cs.push_back(i + 1);
            bs.push_back(end);
        }
    }
    cs.push_back(n);
    bs.push_back(nbytes);
    const size_t K = cs.size() - 1;
    std::vector<cudaEvent_t> landed(K, nullptr), counted(K, nullptr);
    int rc = MDET_OK;
    for (size_t k = 0; k < K && rc == MDET_OK; ++k) {
        rc = ctx_cuda(ctx, cudaEventCreateWithFlags(&landed[k], cudaEventDisableTiming), "cudaEventCreate");
        if (rc == MDET_OK)
            rc = ctx_cuda(ctx, cudaEventCreateWithFlags(&counted[k], cudaEventDisableTiming), "cudaEventCreate");
    }
    for (size_t k = 0; k < K && rc == MDET_OK; ++k) {
        rc = ctx_cuda(ctx,
                      cudaMemcpyAsync(d_bytes + bs[k], bytes + bs[k], bs[k + 1] - bs[k], cudaMemcpyHostToDevice,
                                      ctx->io_in),
                      "cudaMemcpyAsync");
        if (rc == MDET_OK) rc = ctx_cuda(ctx, cudaEventRecord(landed[k], ctx->io_in), "cudaEventRecord");
    }
    for (size_t k = 0; k < K && rc == MDET_OK; ++k) {
        const uint64_t c0 = cs[k], nk = cs[k + 1] - cs[k];
        rc = ctx_cuda(ctx, cudaStreamWaitEvent(s, landed[k], 0), "cudaStreamWaitEvent");
        if (rc == MDET_OK && nk)
            rc = count_impl(ctx, d_bytes, nbytes, d_off + c0, d_len + c0, nk, d_counts + c0 * MDET_NTNF,
                            d_tnf + c0 * MDET_NTNF);
        if (rc == MDET_OK) rc = ctx_cuda(ctx, cudaEventRecord(counted[k], s), "cudaEventRecord");
        if (rc == MDET_OK) rc = ctx_cuda(ctx, cudaStreamWaitEvent(ctx->io_out, counted[k], 0), "cudaStreamWaitEvent");
        if (rc == MDET_OK && nk && counts)
            rc = ctx_cuda(ctx,
                          cudaMemcpyAsync(counts + c0 * MDET_NTNF, d_counts + c0 * MDET_NTNF, nk * MDET_NTNF * 4,
                                          cudaMemcpyDeviceToHost, ctx->io_out),
                          "cudaMemcpyAsync");
        if (rc == MDET_OK && nk)
            rc = ctx_cuda(ctx,
                          cudaMemcpyAsync(tnf + c0 * MDET_NTNF, d_tnf + c0 * MDET_NTNF, nk * MDET_NTNF * 4,
                                          cudaMemcpyDeviceToHost, ctx->io_out),
                          "cudaMemcpyAsync");
    }
    if (rc != MDET_OK) ctx->count_scratch_dirty = true;
    // no copy may still touch the caller's buffers when this returns
    cudaStreamSynchronize(ctx->io_in);
    cudaStreamSynchronize(ctx->io_out);
    for (auto e : landed)
        if (e) cudaEventDestroy(e);
    for (auto e : counted)
        if (e) cudaEventDestroy(e);
    if (rc != MDET_OK) return rc;
    return check_flag(ctx);
}

int mdet_tnf_count(mdet_ctx* ctx, const char* bytes, uint64_t nbytes, const uint64_t* off, const uint64_t* len,
                   uint64_t n, uint32_t* counts, float* tnf) {
    if (!ctx) return MDET_ERR_INVALID;
    if (n && (!bytes || !off || !len || !tnf)) return ctx_fail(ctx, MDET_ERR_INVALID, "null pointer");
    MDET_CUDA(ctx, cudaSetDevice(ctx->device));
    ctx->launches = 0;
    if (n == 0) return MDET_OK;
    for (uint64_t i = 0; i < n; ++i)
        if (off[i] > nbytes || len[i] > nbytes - off[i])
            return ctx_fail(ctx, MDET_ERR_INVALID, "contig %llu lies outside the byte buffer", (unsigned long long)i);
    cudaStream_t s = ctx->stream;
    uint64_t padded = (nbytes + 31) & ~(uint64_t)15;
    char* d_bytes = (char*)ctx_scratch(ctx, "io.bytes", padded);
    uint64_t* d_off = (uint64_t*)ctx_scratch(ctx, "io.off", n * 8);
    uint64_t* d_len = (uint64_t*)ctx_scratch(ctx, "io.len", n * 8);
    uint32_t* d_counts = (uint32_t*)ctx_scratch(ctx, "io.counts", n * MDET_NTNF * 4);
    float* d_tnf = (float*)ctx_scratch(ctx, "io.tnf", n * MDET_NTNF * 4);
    if (!d_bytes || !d_off || !d_len || !d_counts || !d_tnf) return MDET_ERR_NOMEM;
    MDET_CUDA(ctx, cudaMemcpyAsync(d_off, off, n * 8, cudaMemcpyHostToDevice, s));
    MDET_CUDA(ctx, cudaMemcpyAsync(d_len, len, n * 8, cudaMemcpyHostToDevice, s));
    // Views in file order (each contig after the previous one), as a FASTA
    // reader makes them: copy the bytes in ~1 GB chunks on a copy stream and
    // count each chunk once it has landed, returning its rows on a second copy
    // stream, so the count and the result copies hide behind the input copy.
    // The kernel reads nothing outside a contig's own bytes for its counts.
    bool ordered = n >= 2 && nbytes >= ((uint64_t)2 << 30);
    for (uint64_t i = 1; ordered && i < n; ++i) ordered = off[i] >= off[i - 1] + len[i - 1];
    if (ordered) return count_chunked(ctx, bytes, nbytes, off, len, n, counts, tnf, d_bytes, d_off, d_len, d_counts,
                                      d_tnf);
    MDET_CUDA(ctx, cudaMemcpyAsync(d_bytes, bytes, nbytes, cudaMemcpyHostToDevice, s));
    int rc = count_impl(ctx, d_bytes, nbytes, d_off, d_len, n, d_counts, d_tnf);
    if (rc != MDET_OK) {
        ctx->count_scratch_dirty = true;
        return rc;
    }
    if (counts) MDET_CUDA(ctx, cudaMemcpyAsync(counts, d_counts, n * MDET_NTNF * 4, cudaMemcpyDeviceToHost, s));
    MDET_CUDA(ctx, cudaMemcpyAsync(tnf, d_tnf, n * MDET_NTNF * 4, cudaMemcpyDeviceToHost, s));
    return check_flag(ctx);
}

// The reader's record split and the TNF loop in one call from host bytes:
// one copy of the file to the device, the split there (mdet_fasta_index_dev),
// the count on the views it produced, and the rows copied back.
int mdet_tnf_count_fasta(mdet_ctx* ctx, const char* bytes, uint64_t nbytes, uint64_t min_contig, uint64_t capacity,
                         uint64_t* seq_off, uint64_t* seq_len, uint64_t* size, double* log_size, uint64_t* name_off,
                         uint32_t* name_len, uint32_t* counts, float* tnf, mdet_fasta_stats* stats) {
    if (!ctx || !stats) return MDET_ERR_INVALID;
    MDET_CUDA(ctx, cudaSetDevice(ctx->device));
    memset(stats, 0, sizeof(*stats));
    if (nbytes == 0) return MDET_OK;
    if (!bytes) return ctx_fail(ctx, MDET_ERR_INVALID, "null pointer");
    if (capacity && !tnf) return ctx_fail(ctx, MDET_ERR_INVALID, "null output pointer");
    cudaStream_t s = ctx->stream;
    const uint64_t padded = (nbytes + 31) & ~(uint64_t)15, cap = capacity ? capacity : 1;
    char* d_bytes = (char*)ctx_scratch(ctx, "io.bytes", padded);
    uint64_t* d_off = (uint64_t*)ctx_scratch(ctx, "io.off", cap * 8);
    uint64_t* d_len = (uint64_t*)ctx_scratch(ctx, "io.len", cap * 8);
    double* d_ls = (double*)ctx_scratch(ctx, "io.fa_ls", cap * 8);
    uint64_t* d_size = (uint64_t*)ctx_scratch(ctx, "io.fa_size", cap * 8);
    uint64_t* d_noff = (uint64_t*)ctx_scratch(ctx, "io.fa_noff", cap * 8);
    uint32_t* d_nlen = (uint32_t*)ctx_scratch(ctx, "io.fa_nlen", cap * 4);
    if (!d_bytes || !d_off || !d_len || !d_ls || !d_size || !d_noff || !d_nlen) return MDET_ERR_NOMEM;
    MDET_CUDA(ctx, cudaMemcpyAsync(d_bytes, bytes, nbytes, cudaMemcpyHostToDevice, s));
    MDET_TRY(mdet_fasta_index_dev(ctx, d_bytes, nbytes, min_contig, capacity, d_off, d_len, d_size, d_ls, d_noff,
                                  d_nlen, stats));
    const uint64_t n = stats->n_large;
    if (n == 0) return MDET_OK;
    uint32_t* d_counts = (uint32_t*)ctx_scratch(ctx, "io.counts", n * MDET_NTNF * 4);
    float* d_tnf = (float*)ctx_scratch(ctx, "io.tnf", n * MDET_NTNF * 4);
    if (!d_counts || !d_tnf) return MDET_ERR_NOMEM;
    int rc = count_impl(ctx, d_bytes, nbytes, d_off, d_len, n, d_counts, d_tnf);
    if (rc != MDET_OK) {
        ctx->count_scratch_dirty = true;
        return rc;
    }
    if (seq_off) MDET_CUDA(ctx, cudaMemcpyAsync(seq_off, d_off, n * 8, cudaMemcpyDeviceToHost, s));
    if (seq_len) MDET_CUDA(ctx, cudaMemcpyAsync(seq_len, d_len, n * 8, cudaMemcpyDeviceToHost, s));
    if (size) MDET_CUDA(ctx, cudaMemcpyAsync(size, d_size, n * 8, cudaMemcpyDeviceToHost, s));
    if (log_size) MDET_CUDA(ctx, cudaMemcpyAsync(log_size, d_ls, n * 8, cudaMemcpyDeviceToHost, s));
    if (name_off) MDET_CUDA(ctx, cudaMemcpyAsync(name_off, d_noff, n * 8, cudaMemcpyDeviceToHost, s));
    if (name_len) MDET_CUDA(ctx, cudaMemcpyAsync(name_len, d_nlen, n * 4, cudaMemcpyDeviceToHost, s));
    if (counts) MDET_CUDA(ctx, cudaMemcpyAsync(counts, d_counts, n * MDET_NTNF * 4, cudaMemcpyDeviceToHost, s));
    MDET_CUDA(ctx, cudaMemcpyAsync(tnf, d_tnf, n * MDET_NTNF * 4, cudaMemcpyDeviceToHost, s));
    return check_flag(ctx);
}

}  // extern "C"

// ------------------------------------------------- allocation-free variant --
// Some callers cannot allocate device memory at all: a host application that
// hands this library fixed device buffers from its own arena, or a pipeline
// in which a cudaMalloc (which synchronises the device and can fail under
// memory pressure) is not allowed between its stages.  For them,
// mdet_tnf_count_noalloc runs the same counting kernels with their scratch in
// the file-scope array below instead of context-owned buffers.  The array is
// loaded with the library and held by every GPU that loads it until exit.

#define MDET_NOALLOC_MAX_CONTIGS 8192u
#define MDET_NOALLOC_MAX_PIECES 65536u  // 64-KB pieces: about 4 GB of sequence
#define MDET_NOALLOC_CUB_BYTES (64u * 1024u)

namespace {
// word offsets inside the static scratch
constexpr uint32_t kNaNp = 0;                                           // npieces[MAX_CONTIGS]
constexpr uint32_t kNaStart = kNaNp + MDET_NOALLOC_MAX_CONTIGS;         // piece starts
constexpr uint32_t kNaDone = kNaStart + MDET_NOALLOC_MAX_CONTIGS;       // finished pieces per contig
constexpr uint32_t kNaMap = kNaDone + MDET_NOALLOC_MAX_CONTIGS;         // piece -> contig
constexpr uint32_t kNaAcc = kNaMap + MDET_NOALLOC_MAX_PIECES;           // multi-piece accumulators
constexpr uint32_t kNaWork = kNaAcc + MDET_NOALLOC_MAX_CONTIGS * MDET_NTNF;  // counter, flag, status (64 words)
constexpr uint32_t kNaCub = kNaWork + 64;                               // CUB scan temp storage
constexpr uint32_t kNaWords = kNaCub + MDET_NOALLOC_CUB_BYTES / 4;      // ~4.9 MB in total
}  // namespace

static __device__ __align__(256) uint32_t g_noalloc_scratch[kNaWords];

namespace {
struct NoallocDevice {
    uint32_t* scratch = nullptr;  // device address of g_noalloc_scratch
    int grid = 0;                 // k_count grid on this device
};
NoallocDevice g_na_dev[64];
std::mutex g_na_mutex;
}  // namespace

extern "C" int mdet_tnf_count_noalloc(const char* d_bytes, uint64_t nbytes, const uint64_t* d_off,
                                      const uint64_t* d_len, uint64_t n, uint32_t* d_counts, float* d_tnf,
                                      void* stream) {
    if (n == 0) return MDET_OK;
    if (!d_bytes || !d_off || !d_len || !d_counts || !d_tnf) return MDET_ERR_INVALID;
    if (n > MDET_NOALLOC_MAX_CONTIGS) return MDET_ERR_CAPACITY;
    if (((uintptr_t)d_bytes & 15) != 0) return MDET_ERR_INVALID;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return MDET_ERR_CUDA;
    cudaStream_t s = (cudaStream_t)stream;
    {
        // once per device, with that device current: resolve the array's
        // device address (host code cannot use the symbol itself)
        std::lock_guard<std::mutex> lock(g_na_mutex);
        NoallocDevice& d = g_na_dev[dev];
        if (!d.scratch) {
            void* p = nullptr;
            if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) {
                cudaGetLastError();
                return MDET_ERR_CUDA;
            }
            int num_sms = 0;
            if (cudaDeviceGetAttribute(&num_sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) {
                cudaGetLastError();
                return MDET_ERR_CUDA;
            }
            d.grid = k_count_grid(num_sms);
            d.scratch = (uint32_t*)p;
        }
    }
    const NoallocDevice& d = g_na_dev[dev];
    uint32_t* sc = d.scratch;
    CountScratch S{};
    S.npieces = sc + kNaNp;
    S.start = sc + kNaStart;
    S.done = sc + kNaDone;
    S.pmap = sc + kNaMap;
    S.acc = sc + kNaAcc;
    S.work = sc + kNaWork;
    int* flag = (int*)(sc + kNaWork + 1);
    S.status = (unsigned long long*)(sc + kNaWork + 2);
    S.cub_tmp = sc + kNaCub;
    S.cub_bytes = count_cub_bytes(n, s);
    if (S.cub_bytes > MDET_NOALLOC_CUB_BYTES) return MDET_ERR_CAPACITY;
    // From the first enqueued operation on, every error return first waits
    // for the stream, so no work of a failed call still writes the shared
    // array (or the caller's buffers) after it returns.
    auto fail = [&](int code) {
        cudaGetLastError();
        cudaStreamSynchronize(s);
        cudaGetLastError();
        return code;
    };
    // the array keeps the previous call's contents: clear what must start at zero
    if (cudaMemsetAsync(S.done, 0, (size_t)n * 4, s) != cudaSuccess ||
        cudaMemsetAsync(S.acc, 0, (size_t)n * MDET_NTNF * 4, s) != cudaSuccess ||
        cudaMemsetAsync(S.work, 0, 64 * 4, s) != cudaSuccess)
        return fail(MDET_ERR_CUDA);
    if (count_phase1(S, d_off, d_len, n, nbytes, s) != cudaSuccess) return fail(MDET_ERR_CUDA);
    // the 64-bit piece total and the count of views outside [0, nbytes),
    // checked before k_piece_map writes piece entries into the array
    unsigned long long st[2] = {0, 0};
    if (cudaMemcpyAsync(st, S.status, 16, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess)
        return fail(MDET_ERR_CUDA);
    if (st[1]) return MDET_ERR_INVALID;
    if (st[0] > MDET_NOALLOC_MAX_PIECES) return MDET_ERR_CAPACITY;
    if (count_phase2(S, (const unsigned char*)d_bytes, d_off, d_len, n, (uint32_t)st[0], d_counts, d_tnf, flag,
                     d.grid, s) != cudaSuccess)
        return fail(MDET_ERR_CUDA);
    int h_flag = 0;
    if (cudaMemcpyAsync(&h_flag, flag, sizeof(int), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess)
        return fail(MDET_ERR_CUDA);
    return h_flag ? MDET_ERR_TIMEOUT : MDET_OK;
}
