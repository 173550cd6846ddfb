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
// left them (newlines included).  Work is cut into pieces of <= 16 KB of
// one contig; each warp takes pieces from a global counter and streams the
// piece through a private double buffer in shared memory with 1-D bulk
// copies (the TMA engine), histogramming raw 8-bit codes into a private
// 256-bin shared histogram.  The window that straddles two lanes' 16-byte
// chunks is carried by a warp scan over (last three bases, count) states.
// A contig cut into several pieces accumulates into a per-contig scratch row
// and the last piece to finish normalises it (and clears the scratch row).
#include <cub/cub.cuh>

#include <mutex>

#include "common.cuh"

namespace {

constexpr int kWarps = 8;
constexpr uint32_t kStage = 4096;   // bytes per warp stage
constexpr uint64_t kPiece = 16384;  // bytes per piece (multiple of kStage)
constexpr uint32_t kPoison = 0xFF00u;

struct FoldTables {
    uint8_t fw[MDET_NTNF];
    uint8_t rc[MDET_NTNF];
};

__global__ void k_piece_counts(const uint64_t* __restrict__ len, uint64_t n, uint32_t* __restrict__ npieces) {
    uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    uint64_t L = len[i];
    npieces[i] = L == 0 ? 1u : (uint32_t)((L + kPiece - 1) / kPiece);
}

__global__ void k_piece_map(const uint32_t* __restrict__ npieces, const uint32_t* __restrict__ start, uint64_t n,
                            uint32_t* __restrict__ piece_contig) {
    uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    uint32_t s = start[i], np = npieces[i];
    for (uint32_t k = 0; k < np; ++k) piece_contig[s + k] = (uint32_t)i;
}

// Shift character state `x` (codes in the low byte, poison in the high byte,
// two bits per slot) by one more character.
__device__ __forceinline__ uint32_t shift_in(uint32_t x, uint32_t ch) {
    uint32_t u = (ch | 0x20u) - 0x61u;  // 'a'..
    uint32_t valid = (u < 20u) ? ((0x80045u >> u) & 1u) : 0u;  // a, c, g, t
    return ((x << 2) & 0xFCFCu) | ((ch >> 1) & 3u) | (valid ? 0u : 0x300u);
}

// Compose the state of a prefix with the state of the following chunk that
// holds `cnt` (capped at 4) characters of its own.
__device__ __forceinline__ uint32_t compose(uint32_t pre, uint32_t chunk_x, uint32_t cnt) {
    uint32_t m8 = (0xFFu << (2 * cnt)) & 0xFFu;
    uint32_t m = m8 | (m8 << 8);
    return ((pre << (2 * cnt)) & m) | (chunk_x & ~m);
}

__device__ __forceinline__ uint32_t pack_state(uint32_t x, uint32_t cnt) { return x | (cnt << 16); }

struct Sums {
    uint64_t v;
};

__device__ __forceinline__ uint64_t warp_sum_u64(uint64_t v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Writes one finished contig row from per-lane canonical counts.
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
    double rsum = sqrt((double)s);
    double inv = 1.0 / rsum;
#pragma unroll
    for (int j = 0; j < 5; ++j) {
        uint32_t col = lane + 32 * j;
        if (col < MDET_NTNF) {
            counts[c * MDET_NTNF + col] = v[j];
            tnf[c * MDET_NTNF + col] = s ? (float)((double)v[j] * inv) : __int_as_float(0x7fffffff);
        }
    }
}

__global__ void __launch_bounds__(kWarps * 32) k_count(const unsigned char* __restrict__ bytes,
                                                      const uint64_t* __restrict__ off,
                                                      const uint64_t* __restrict__ len, uint64_t n,
                                                      const uint32_t* __restrict__ piece_start,
                                                      const uint32_t* __restrict__ npieces,
                                                      const uint32_t* __restrict__ piece_contig,
                                                      uint32_t* __restrict__ work, uint32_t* __restrict__ acc,
                                                      uint32_t* __restrict__ done, uint32_t* __restrict__ counts,
                                                      float* __restrict__ tnf, FoldTables tabs, int* flag) {
    extern __shared__ __align__(128) unsigned char smem[];
    __shared__ uint32_t hist_all[kWarps][257];  // 256 raw 4-mer codes + a bin for discarded windows
    __shared__ uint64_t bars[kWarps][2];
    // byte -> update word: 2-bit base code | 0x300 when not a base | 0x8000 for '\n'
    __shared__ uint16_t lut[256];
    const uint32_t w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    unsigned char* buf0 = smem + (size_t)w * 2 * kStage;
    uint32_t* hist = hist_all[w];
    for (uint32_t c = threadIdx.x; c < 256; c += blockDim.x) {
        const uint32_t u = (c | 0x20u) - 0x61u;
        const uint32_t valid = (u < 20u) ? ((0x80045u >> u) & 1u) : 0u;
        lut[c] = (uint16_t)(c == '\n' ? 0x8000u : (((c >> 1) & 3u) | (valid ? 0u : 0x300u)));
    }
    if (lane == 0) {
        mbar_init(&bars[w][0], 1);
        mbar_init(&bars[w][1], 1);
        mbar_fence_init();
    }
    __syncthreads();
    uint32_t phase[2] = {0, 0};
    const uint32_t total = piece_start[n - 1] + npieces[n - 1];

    while (true) {
        uint32_t p = 0;
        if (lane == 0) p = atomicAdd(work, 1u);
        p = __shfl_sync(0xffffffffu, p, 0);
        if (p >= total) break;
        if (*(volatile int*)flag) break;
        const uint64_t c = piece_contig[p];
        const uint32_t k = p - piece_start[c];
        const uint64_t s0 = off[c], L = len[c];
        const uint64_t p0 = s0 + (uint64_t)k * kPiece;
        const uint64_t p1 = min(s0 + L, p0 + kPiece);

        // carry-in: the last three non-newline characters before p0
        uint32_t carry = kPoison;
        {
            int need = 3;
            uint32_t got[3] = {0, 0, 0};  // newest first
            uint64_t pos = p0;
            while (need > 0 && pos > s0) {
                int64_t q = (int64_t)pos - 1 - (int64_t)lane;
                uint32_t ch = (q >= (int64_t)s0) ? bytes[q] : (uint32_t)'\n';
                bool inb = q >= (int64_t)s0;
                uint32_t good = __ballot_sync(0xffffffffu, inb && ch != '\n');
                while (good && need > 0) {
                    int src = __ffs(good) - 1;
                    got[3 - need] = __shfl_sync(0xffffffffu, ch, src);
                    good &= good - 1;
                    --need;
                }
                pos = pos > s0 + 32 ? pos - 32 : s0;
            }
            for (int t = 2; t >= 0; --t)
                if (t < 3 - need) carry = shift_in(carry, got[t]);
        }

        for (int i = lane; i < 257; i += 32) hist[i] = 0;
        __syncwarp();

        const uint64_t a0 = p0 & ~(uint64_t)15;
        const uint64_t a1 = (p1 + 15) & ~(uint64_t)15;
        const uint32_t nst = (uint32_t)((a1 - a0 + kStage - 1) / kStage);
        bool ok = true;
        if (lane == 0 && nst > 0) {
            fence_proxy_async_smem();
            uint32_t b0 = (uint32_t)min((uint64_t)kStage, a1 - a0);
            mbar_arrive_tx(&bars[w][0], b0);
            bulk_g2s(buf0, bytes + a0, b0, &bars[w][0]);
        }
        for (uint32_t st = 0; st < nst; ++st) {
            const uint32_t bi = st & 1;
            const uint64_t sabs = a0 + (uint64_t)st * kStage;
            const uint32_t sbytes = (uint32_t)min((uint64_t)kStage, a1 - sabs);
            if (st + 1 < nst) {
                __syncwarp();
                if (lane == 0) {
                    fence_proxy_async_smem();
                    uint64_t nabs = sabs + kStage;
                    uint32_t nb = (uint32_t)min((uint64_t)kStage, a1 - nabs);
                    mbar_arrive_tx(&bars[w][bi ^ 1], nb);
                    bulk_g2s(buf0 + (bi ^ 1) * kStage, bytes + nabs, nb, &bars[w][bi ^ 1]);
                }
            }
            if (!__all_sync(0xffffffffu, mbar_wait(&bars[w][bi], phase[bi], flag))) {  // bounded, warp-uniform
                ok = false;
                break;
            }
            phase[bi] ^= 1;
            const unsigned char* sb = buf0 + bi * kStage;
            for (uint32_t r = 0; r * 512 < sbytes; ++r) {
                const uint32_t cofs = r * 512 + lane * 16;
                const int64_t cb = (int64_t)(sabs + cofs);
                uint4 v = make_uint4(0, 0, 0, 0);
                if (cofs < sbytes) v = *reinterpret_cast<const uint4*>(sb + cofs);
                int64_t lo = (int64_t)p0 - cb, hi = (int64_t)p1 - cb;
                lo = lo < 0 ? 0 : (lo > 16 ? 16 : lo);
                hi = hi < 0 ? 0 : (hi > 16 ? 16 : hi);
                uint32_t act = ((hi >= 16 ? 0xFFFFu : ((1u << hi) - 1u)) & ~((1u << lo) - 1u));
                if (cofs >= sbytes) act = 0;
                uint32_t words[4] = {v.x, v.y, v.z, v.w};
                // pass over the chunk from a fully poisoned state
                uint32_t x = kPoison, nact = 0, x3 = 0, nlm = 0;
                const bool full = act == 0xFFFFu;
                bool packed = false;
                if (full) {
                    // SWAR per word: 2-bit codes, newline bytes, bytes that are no base letter
                    uint32_t xs[4], pzm = 0;
#pragma unroll
                    for (int q = 0; q < 4; ++q) {
                        const uint32_t w = words[q];
                        const uint32_t lc = w | 0x20202020u;
                        const uint32_t K = (lc >> 1) & 0x03030303u;
                        const uint32_t sel = __byte_perm(K | (K >> 4), 0u, 0x4420u);
                        const uint32_t bad = lc ^ __byte_perm(0x67746361u, 0u, sel);  // 'a' 'c' 't' 'g'
                        const uint32_t nz = (((bad & 0x7F7F7F7Fu) + 0x7F7F7F7Fu) | bad) & 0x80808080u;
                        const uint32_t z = w ^ 0x0A0A0A0Au;
                        const uint32_t nl = ~(((z & 0x7F7F7F7Fu) + 0x7F7F7F7Fu) | z) & 0x80808080u;
                        nlm |= ((((nl >> 7) * 0x01020408u) >> 24) & 0xFu) << (4 * q);
                        pzm |= (((((nz & ~nl) >> 7) * 0x01020408u) >> 24) & 0xFu) << (4 * q);
                        xs[q] = K * 0x40100401u;  // byte 3: the word's four codes, oldest highest
                    }
                    if (__popc(nlm) <= 2) {
                        packed = true;
                        // field f (2 bits at 2f) holds byte 15 - f; drop the newline fields
                        const uint32_t hi = __byte_perm(xs[0], xs[1], 0x3700u);
                        const uint32_t lo = __byte_perm(xs[2], xs[3], 0x0037u);
                        uint64_t P = __byte_perm(hi, lo, 0x3254u);
                        uint32_t pz = __brev(pzm) >> 16, nlr = __brev(nlm) >> 16;
                        while (nlr) {
                            const int f = 31 - __clz(nlr);
                            nlr &= ~(1u << f);
                            P = ((P >> (2 * f + 2)) << (2 * f)) | (P & ((1ull << (2 * f)) - 1));
                            pz = ((pz >> (f + 1)) << f) | (pz & ((1u << f) - 1));
                        }
                        nact = 16u - __popc(nlm);
                        // window k: fields k..k+3 (newest at k); poisoned when any of them is
                        const uint32_t wi = pz | (pz >> 1) | (pz >> 2) | (pz >> 3);
                        const uint32_t P32 = (uint32_t)P;
#pragma unroll
                        for (int k = 0; k < 13; ++k) {
                            const uint32_t code = (P32 >> (2 * k)) & 0xFFu;
                            const bool ok = (uint32_t)k + 4u <= nact && !((wi >> k) & 1u);
                            atomicAdd(&hist[ok ? code : 256u], 1u);
                        }
                        // states: the last four codes and the first three, poison in the high byte
                        auto spread = [](uint32_t b) {
                            return ((b & 1u) * 3u) | ((b & 2u) * 6u) | ((b & 4u) * 12u) | ((b & 8u) * 24u);
                        };
                        x = (P32 & 0xFFu) | (spread(pz & 0xFu) << 8);
                        x3 = ((P32 >> (2 * (nact - 3))) & 0x3Fu) | (spread((pz >> (nact - 3)) & 7u) << 8);
                    }
                }
                if (full && !packed) {
                    // every byte of the chunk is in the piece: table-driven
                    // update, newline bytes leave the state unchanged, and
                    // every window lands in a bin (bin 256 takes the invalid
                    // ones) so the loop has no branches
                    nlm = 0;
#pragma unroll
                    for (int b = 0; b < 16; ++b) {
                        const uint32_t ch = __byte_perm(words[b >> 2], 0u, 0x4440u | (uint32_t)(b & 3));
                        const uint32_t m = lut[ch];
                        const bool nl = m >= 0x8000u;
                        const uint32_t xn = ((x << 2) & 0xFCFCu) | m;
                        x = nl ? x : xn;
                        const uint32_t bin = (nl || x >= 256u) ? 256u : x;
                        atomicAdd(&hist[bin], 1u);
                        if (b == 2) x3 = x;
                    }
                    // newline bytes of the chunk (SWAR zero-byte test on w ^ '\n')
#pragma unroll
                    for (int q = 0; q < 4; ++q) {
                        const uint32_t z = words[q] ^ 0x0A0A0A0Au;
                        const uint32_t hit = ~(((z & 0x7F7F7F7Fu) + 0x7F7F7F7Fu) | z) & 0x80808080u;
                        nlm |= hit ? (((hit >> 7) * 0x01020408u) >> 24 & 0xFu) << (4 * q) : 0u;
                    }
                    nact = 16u - __popc(nlm);
                } else if (!full) {
#pragma unroll
                    for (int b = 0; b < 16; ++b) {
                        uint32_t ch = (words[b >> 2] >> (8 * (b & 3))) & 0xFFu;
                        bool on = ((act >> b) & 1u) && ch != '\n';
                        if (on) {
                            x = shift_in(x, ch);
                            ++nact;
                            if (x < 256u) atomicAdd(&hist[x], 1u);
                        }
                    }
                }
                uint32_t cnt = nact < 4 ? nact : 4;
                // carry-in for this lane: compose lanes 0..l-1 of this row onto `carry`
                uint32_t st_incl = pack_state(x & 0xFFFFu, cnt);
                uint32_t all_full = __all_sync(0xffffffffu, cnt >= 3);
                uint32_t cin;
                if (all_full) {
                    uint32_t prev = __shfl_up_sync(0xffffffffu, st_incl, 1);
                    cin = lane == 0 ? carry : (prev & 0xFFFFu);
                    uint32_t last = __shfl_sync(0xffffffffu, st_incl, 31);
                    carry = last & 0xFFFFu;
                } else {
#pragma unroll
                    for (int o = 1; o < 32; o <<= 1) {
                        uint32_t other = __shfl_up_sync(0xffffffffu, st_incl, o);
                        if (lane >= (uint32_t)o) {
                            uint32_t mc = st_incl >> 16;
                            uint32_t ox = other & 0xFFFFu, oc = other >> 16;
                            uint32_t nx = compose(ox, st_incl & 0xFFFFu, mc);
                            uint32_t nc = oc + mc;
                            st_incl = pack_state(nx, nc < 4 ? nc : 4);
                        }
                    }
                    uint32_t prev = __shfl_up_sync(0xffffffffu, st_incl, 1);
                    uint32_t excl = lane == 0 ? kPoison : (prev & 0xFFFFu);
                    uint32_t excl_cnt = lane == 0 ? 0u : (prev >> 16);
                    cin = excl_cnt >= 3 ? excl : compose(carry, excl, excl_cnt);
                    uint32_t last = __shfl_sync(0xffffffffu, st_incl, 31);
                    carry = (last >> 16) >= 3 ? (last & 0xFFFFu) : compose(carry, last & 0xFFFFu, last >> 16);
                }
                // the first (up to) three windows of the chunk depend on the carry-in
                if (packed || (full && (nlm & 7u) == 0)) {
                    // x3 holds the chunk's first three characters in slots 2, 1, 0
                    const uint32_t w1 = compose(cin, x3 >> 4, 1);
                    const uint32_t w2 = compose(cin, x3 >> 2, 2);
                    const uint32_t w3 = compose(cin, x3, 3);
                    atomicAdd(&hist[w1 < 256u ? w1 : 256u], 1u);
                    atomicAdd(&hist[w2 < 256u ? w2 : 256u], 1u);
                    atomicAdd(&hist[w3 < 256u ? w3 : 256u], 1u);
                } else if (nact > 0) {
                    uint32_t y = cin, seen = 0;
#pragma unroll
                    for (int b = 0; b < 16; ++b) {
                        uint32_t ch = (words[b >> 2] >> (8 * (b & 3))) & 0xFFu;
                        bool on = ((act >> b) & 1u) && ch != '\n' && seen < 3;
                        if (on) {
                            y = shift_in(y, ch);
                            ++seen;
                            if (y < 256u) atomicAdd(&hist[y], 1u);
                        }
                    }
                }
            }
        }
        if (!ok) break;
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

static int count_impl(mdet_ctx* ctx, const char* d_bytes, uint64_t nbytes, const uint64_t* d_off,
                      const uint64_t* d_len, uint64_t n, uint32_t* d_counts, float* d_tnf) {
    if (n == 0) return MDET_OK;
    if (n >= 0xFFFFFFFFull) return ctx_fail(ctx, MDET_ERR_INVALID, "too many contigs (%llu)", (unsigned long long)n);
    if (((uintptr_t)d_bytes & 15) != 0)
        return ctx_fail(ctx, MDET_ERR_INVALID, "sequence buffer must be 16-byte aligned");
    (void)nbytes;
    cudaStream_t s = ctx->stream;
    uint32_t* npieces = (uint32_t*)ctx_scratch(ctx, "cnt.np", n * 4);
    uint32_t* start = (uint32_t*)ctx_scratch(ctx, "cnt.start", n * 4);
    uint32_t* work = (uint32_t*)ctx_scratch(ctx, "cnt.work", 16);
    // per-contig accumulators for multi-piece contigs: zero when grown, and
    // every finishing warp clears its row again, so they stay zero between calls
    if (ctx->count_scratch_dirty) {
        ctx->bufs.erase("cnt.acc");
        ctx->bufs.erase("cnt.done");
        ctx->count_scratch_dirty = false;
    }
    uint32_t* acc = (uint32_t*)ctx_scratch(ctx, "cnt.acc", n * MDET_NTNF * 4, true);
    uint32_t* done = (uint32_t*)ctx_scratch(ctx, "cnt.done", n * 4, true);
    if (!npieces || !start || !work || !acc || !done) return MDET_ERR_NOMEM;
    unsigned blocks = (unsigned)((n + 255) / 256);
    k_piece_counts<<<blocks, 256, 0, s>>>(d_len, n, npieces);
    MDET_LAUNCHED(ctx, "k_piece_counts");
    size_t tmp_bytes = 0;
    cub::DeviceScan::ExclusiveSum(nullptr, tmp_bytes, npieces, start, (int)n, s);
    void* tmp = ctx_scratch(ctx, "cnt.cubtmp", tmp_bytes);
    if (!tmp) return MDET_ERR_NOMEM;
    MDET_CUDA(ctx, cub::DeviceScan::ExclusiveSum(tmp, tmp_bytes, npieces, start, (int)n, s));
    // exact piece total (contig views may overlap, so it is not bounded by nbytes)
    uint32_t tail[2] = {0, 0};
    MDET_CUDA(ctx, cudaMemcpyAsync(&tail[0], start + n - 1, 4, cudaMemcpyDeviceToHost, s));
    MDET_CUDA(ctx, cudaMemcpyAsync(&tail[1], npieces + n - 1, 4, cudaMemcpyDeviceToHost, s));
    MDET_CUDA(ctx, cudaStreamSynchronize(s));
    uint64_t max_pieces = (uint64_t)tail[0] + tail[1];
    uint32_t* pmap = (uint32_t*)ctx_scratch(ctx, "cnt.pmap", max_pieces * 4);
    if (!pmap) return MDET_ERR_NOMEM;
    k_piece_map<<<blocks, 256, 0, s>>>(npieces, start, n, pmap);
    MDET_LAUNCHED(ctx, "k_piece_map");
    MDET_CUDA(ctx, cudaMemsetAsync(work, 0, 4, s));
    FoldTables tabs;
    const TnTables& t = tn_tables();
    memcpy(tabs.fw, t.col_fw, MDET_NTNF);
    memcpy(tabs.rc, t.col_rc, MDET_NTNF);
    const size_t dyn = (size_t)kWarps * 2 * kStage;
    static bool attr_set[64] = {false};
    if (!attr_set[ctx->device & 63]) {
        MDET_CUDA(ctx, cudaFuncSetAttribute(k_count, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dyn));
        attr_set[ctx->device & 63] = true;
    }
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_count, kWarps * 32, dyn);
    if (per_sm < 1) per_sm = 1;
    ctx_timer_begin(ctx, "k_count");
    k_count<<<ctx->num_sms * per_sm, kWarps * 32, dyn, s>>>((const unsigned char*)d_bytes, d_off, d_len, n, start,
                                                            npieces, pmap, work, acc, done, d_counts, d_tnf, tabs,
                                                            ctx->d_flag);
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

int mdet_tnf_count(mdet_ctx* ctx, const char* bytes, uint64_t nbytes, const uint64_t* off, const uint64_t* len,
                   uint64_t n, uint32_t* counts, float* tnf) {
    if (!ctx) return MDET_ERR_INVALID;
    if (n && (!bytes || !off || !len || !counts || !tnf)) return ctx_fail(ctx, MDET_ERR_INVALID, "null pointer");
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
    MDET_CUDA(ctx, cudaMemcpyAsync(d_bytes, bytes, nbytes, cudaMemcpyHostToDevice, s));
    MDET_CUDA(ctx, cudaMemcpyAsync(d_off, off, n * 8, cudaMemcpyHostToDevice, s));
    MDET_CUDA(ctx, cudaMemcpyAsync(d_len, len, n * 8, cudaMemcpyHostToDevice, s));
    int rc = count_impl(ctx, d_bytes, nbytes, d_off, d_len, n, d_counts, d_tnf);
    if (rc != MDET_OK) {
        ctx->count_scratch_dirty = true;
        return rc;
    }
    MDET_CUDA(ctx, cudaMemcpyAsync(counts, d_counts, n * MDET_NTNF * 4, cudaMemcpyDeviceToHost, s));
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
#define MDET_NOALLOC_MAX_PIECES 65536u
#define MDET_NOALLOC_CUB_BYTES (64u * 1024u)

namespace {
// word offsets inside the static scratch
constexpr uint32_t kNaNp = 0;                                           // npieces[MAX_CONTIGS]
constexpr uint32_t kNaStart = kNaNp + MDET_NOALLOC_MAX_CONTIGS;         // piece starts
constexpr uint32_t kNaDone = kNaStart + MDET_NOALLOC_MAX_CONTIGS;       // finished pieces per contig
constexpr uint32_t kNaMap = kNaDone + MDET_NOALLOC_MAX_CONTIGS;         // piece -> contig
constexpr uint32_t kNaAcc = kNaMap + MDET_NOALLOC_MAX_PIECES;           // multi-piece accumulators
constexpr uint32_t kNaWork = kNaAcc + MDET_NOALLOC_MAX_CONTIGS * MDET_NTNF;  // work counter + flag (64 words)
constexpr uint32_t kNaCub = kNaWork + 64;                               // CUB scan temp storage
constexpr uint32_t kNaWords = kNaCub + MDET_NOALLOC_CUB_BYTES / 4;      // ~4.9 MB in total
}  // namespace

static __device__ __align__(256) uint32_t g_noalloc_scratch[kNaWords];

namespace {
struct NoallocDevice {
    uint32_t* scratch = nullptr;  // device address of g_noalloc_scratch
    int num_sms = 0;
    int per_sm = 0;
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
    const size_t dyn = (size_t)kWarps * 2 * kStage;
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
            if (cudaFuncSetAttribute(k_count, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dyn) != cudaSuccess ||
                cudaDeviceGetAttribute(&d.num_sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
                cudaOccupancyMaxActiveBlocksPerMultiprocessor(&d.per_sm, k_count, kWarps * 32, dyn) != cudaSuccess) {
                cudaGetLastError();
                return MDET_ERR_CUDA;
            }
            if (d.per_sm < 1) d.per_sm = 1;
            d.scratch = (uint32_t*)p;
        }
    }
    const NoallocDevice& d = g_na_dev[dev];
    uint32_t* sc = d.scratch;
    uint32_t* npieces = sc + kNaNp;
    uint32_t* start = sc + kNaStart;
    uint32_t* done = sc + kNaDone;
    uint32_t* pmap = sc + kNaMap;
    uint32_t* acc = sc + kNaAcc;
    uint32_t* work = sc + kNaWork;
    int* flag = (int*)(sc + kNaWork + 1);
    void* cub_tmp = sc + kNaCub;
    // the array keeps the previous call's contents: clear what must start at zero
    if (cudaMemsetAsync(done, 0, (size_t)n * 4, s) != cudaSuccess ||
        cudaMemsetAsync(acc, 0, (size_t)n * MDET_NTNF * 4, s) != cudaSuccess ||
        cudaMemsetAsync(work, 0, 64 * 4, s) != cudaSuccess) {
        cudaGetLastError();
        return MDET_ERR_CUDA;
    }
    const unsigned blocks = (unsigned)((n + 255) / 256);
    k_piece_counts<<<blocks, 256, 0, s>>>(d_len, n, npieces);
    size_t tmp_bytes = 0;
    if (cub::DeviceScan::ExclusiveSum(nullptr, tmp_bytes, npieces, start, (int)n, s) != cudaSuccess ||
        tmp_bytes > MDET_NOALLOC_CUB_BYTES)
        return MDET_ERR_CUDA;
    if (cub::DeviceScan::ExclusiveSum(cub_tmp, tmp_bytes, npieces, start, (int)n, s) != cudaSuccess) {
        cudaGetLastError();
        return MDET_ERR_CUDA;
    }
    uint32_t tail[2] = {0, 0};
    if (cudaMemcpyAsync(&tail[0], start + n - 1, 4, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaMemcpyAsync(&tail[1], npieces + n - 1, 4, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess) {
        cudaGetLastError();
        return MDET_ERR_CUDA;
    }
    if ((uint64_t)tail[0] + tail[1] > MDET_NOALLOC_MAX_PIECES) return MDET_ERR_CAPACITY;
    k_piece_map<<<blocks, 256, 0, s>>>(npieces, start, n, pmap);
    FoldTables tabs;
    const TnTables& t = tn_tables();
    memcpy(tabs.fw, t.col_fw, MDET_NTNF);
    memcpy(tabs.rc, t.col_rc, MDET_NTNF);
    k_count<<<d.num_sms * d.per_sm, kWarps * 32, dyn, s>>>((const unsigned char*)d_bytes, d_off, d_len, n, start,
                                                           npieces, pmap, work, acc, done, d_counts, d_tnf, tabs,
                                                           flag);
    if (cudaGetLastError() != cudaSuccess) return MDET_ERR_CUDA;
    int h_flag = 0;
    if (cudaMemcpyAsync(&h_flag, flag, sizeof(int), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess) {
        cudaGetLastError();
        return MDET_ERR_CUDA;
    }
    return h_flag ? MDET_ERR_TIMEOUT : MDET_OK;
}
