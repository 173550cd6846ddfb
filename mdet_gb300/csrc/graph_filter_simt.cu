// graph_filter_simt.cu -- the PLAIN distance filter: FP32 SIMT all-pairs
// squared distances sum_k (a_k - b_k)^2 in the reference's element order
// (cuda/Cuda2.cu:193-196, accumulated in FP32), compared per tile with the
// conservative d* bound of the tile's size range.  Pairs that pass go to the
// exact stage; nothing n x n is written.
//
// 128 x 128 tiles, 256 threads, 8 x 8 pairs per thread, K staged through
// shared memory in chunks of 8.  Triangular schedule (tile J >= I, pairs
// i < j) for the graph, rectangular for the max-probability sample.
#include "graph.cuh"

namespace {

constexpr int BM = 128, BN = 128, BK = 8, TH = 256;

struct SimtArgs {
    const float* a;          // [na][136] rows
    const float* b;          // [nb][136] columns
    uint32_t na, nb;
    uint32_t ta, tb;         // tiles along rows / columns
    int triangular;
    const BlockMeta* ameta;  // per 128-row block of a
    const BlockMeta* bmeta;  // per 128-row block of b
    DstarTable tbl;
    CandBuf out;
    unsigned long long ntiles;
    const uint32_t* tiles;   // optional list (I * tb + J); null: the full schedule
    const uint8_t* row_tbl;  // optional table index per row tile (tables tbl_stride floats apart)
    uint64_t tbl_stride;
};

__device__ __forceinline__ void tile_of(const SimtArgs& p, unsigned long long t, uint32_t& I, uint32_t& J) {
    if (p.tiles) {
        const uint32_t v = p.tiles[t];
        I = v / p.tb;
        J = v % p.tb;
        return;
    }
    if (!p.triangular) {
        I = (uint32_t)(t / p.tb);
        J = (uint32_t)(t % p.tb);
        return;
    }
    // row-major upper triangle: row I holds tiles J = I..T-1; start(I) = I*T - I(I-1)/2
    double T = (double)p.ta;
    double disc = (2 * T + 1) * (2 * T + 1) - 8.0 * (double)t;
    long long i = (long long)floor(((2 * T + 1) - sqrt(disc > 0 ? disc : 0)) / 2);
    if (i < 0) i = 0;
    auto start = [&](long long r) { return (unsigned long long)(r * (long long)p.ta - r * (r - 1) / 2); };
    while (i > 0 && start(i) > t) --i;
    while (i + 1 < (long long)p.ta && start(i + 1) <= t) ++i;
    I = (uint32_t)i;
    J = (uint32_t)(i + (long long)(t - start(i)));
}

__global__ void __launch_bounds__(TH, 2) k_filter_simt(SimtArgs p) {
    __shared__ __align__(16) float As[2][BK][BM + 4];
    __shared__ __align__(16) float Bs[2][BK][BN + 4];
    const int tid = threadIdx.x;
    const int tx = tid & 15, ty = tid >> 4;
    const int lane = tid & 31;
    for (unsigned long long t = blockIdx.x; t < p.ntiles; t += gridDim.x) {
        uint32_t I, J;
        tile_of(p, t, I, J);
        const uint32_t i0 = I * BM, j0 = J * BN;
        // tile threshold
        BlockMeta ma = p.ameta[I], mb = p.bmeta[J];
        DstarTable tb = p.tbl;
        if (tb.dyn) {
            tb.lmin = tb.dyn[0];
            tb.inv_h = tb.dyn[1];
        }
        if (p.row_tbl) tb.st += (uint64_t)p.row_tbl[I] * p.tbl_stride;
        float T = tile_dstar(tb, ma.lo, ma.hi, mb.lo, mb.hi);
        float R = T * (1.f + 2e-5f) + 1e-6f;
        float R2 = R * R;
        if (!(R2 < 1e30f)) R2 = __int_as_float(0x7f800000);

        float acc[8][8];
#pragma unroll
        for (int i = 0; i < 8; ++i)
#pragma unroll
            for (int j = 0; j < 8; ++j) acc[i][j] = 0.f;

        // loader mapping: 128 rows x 8 k per tile side -> 256 threads x float4
        const int lr = tid >> 1, lk = (tid & 1) * 4;
        const uint32_t ga = i0 + lr, gb = j0 + lr;
        auto load = [&](int buf, int k0) {
            float4 va = make_float4(0, 0, 0, 0), vb = make_float4(0, 0, 0, 0);
            int k = k0 + lk;
            if (ga < p.na && k < MDET_NTNF) va = *reinterpret_cast<const float4*>(p.a + (uint64_t)ga * MDET_NTNF + k);
            if (gb < p.nb && k < MDET_NTNF) vb = *reinterpret_cast<const float4*>(p.b + (uint64_t)gb * MDET_NTNF + k);
            As[buf][lk + 0][lr] = va.x;
            As[buf][lk + 1][lr] = va.y;
            As[buf][lk + 2][lr] = va.z;
            As[buf][lk + 3][lr] = va.w;
            Bs[buf][lk + 0][lr] = vb.x;
            Bs[buf][lk + 1][lr] = vb.y;
            Bs[buf][lk + 2][lr] = vb.z;
            Bs[buf][lk + 3][lr] = vb.w;
        };
        __syncthreads();
        load(0, 0);
        __syncthreads();
        constexpr int NK = (MDET_NTNF + BK - 1) / BK;  // 17
#pragma unroll 1
        for (int kc = 0; kc < NK; ++kc) {
            const int cur = kc & 1;
            if (kc + 1 < NK) load(cur ^ 1, (kc + 1) * BK);
#pragma unroll
            for (int kk = 0; kk < BK; ++kk) {
                float4 a0 = *reinterpret_cast<const float4*>(&As[cur][kk][ty * 8]);
                float4 a1 = *reinterpret_cast<const float4*>(&As[cur][kk][ty * 8 + 4]);
                float4 b0 = *reinterpret_cast<const float4*>(&Bs[cur][kk][tx * 8]);
                float4 b1 = *reinterpret_cast<const float4*>(&Bs[cur][kk][tx * 8 + 4]);
                float av[8] = {a0.x, a0.y, a0.z, a0.w, a1.x, a1.y, a1.z, a1.w};
                float bv[8] = {b0.x, b0.y, b0.z, b0.w, b1.x, b1.y, b1.z, b1.w};
#pragma unroll
                for (int i = 0; i < 8; ++i)
#pragma unroll
                    for (int j = 0; j < 8; ++j) {
                        float df = av[i] - bv[j];
                        acc[i][j] = fmaf(df, df, acc[i][j]);
                    }
            }
            __syncthreads();
        }
        // epilogue: 64-bit mask of passing pairs, then warp-aggregated append
        unsigned long long mask = 0;
#pragma unroll
        for (int i = 0; i < 8; ++i)
#pragma unroll
            for (int j = 0; j < 8; ++j) {
                uint32_t gi = i0 + ty * 8 + i, gj = j0 + tx * 8 + j;
                bool ok = acc[i][j] < R2 && gi < p.na && gj < p.nb && (!p.triangular || gi < gj);
                mask |= (unsigned long long)ok << (i * 8 + j);
            }
        while (__any_sync(0xffffffffu, mask != 0)) {
            bool has = mask != 0;
            int bit = has ? __ffsll((long long)mask) - 1 : 0;
            if (has) mask &= mask - 1;
            uint32_t bal = __ballot_sync(0xffffffffu, has);
            unsigned long long base = 0;
            int leader = __ffs(bal) - 1;
            if (lane == leader) base = atomicAdd(p.out.count, (unsigned long long)__popc(bal));
            base = __shfl_sync(0xffffffffu, base, leader);
            if (has) {
                unsigned long long pos = base + __popc(bal & ((1u << lane) - 1u));
                if (pos < p.out.cap)
                    p.out.cand[pos] = make_uint2(i0 + ty * 8 + (bit >> 3), j0 + tx * 8 + (bit & 7));
            }
        }
    }
}

}  // namespace

int filter_simt(mdet_ctx* ctx, const float* a, uint32_t na, const BlockMeta* ameta, const float* b, uint32_t nb,
                const BlockMeta* bmeta, bool triangular, const DstarTable& tbl, CandBuf out, const uint32_t* tiles,
                uint64_t nlist, const uint8_t* row_tbl, uint64_t tbl_stride) {
    SimtArgs p;
    p.a = a;
    p.b = b;
    p.na = na;
    p.nb = nb;
    p.ta = (na + BM - 1) / BM;
    p.tb = (nb + BN - 1) / BN;
    p.triangular = triangular ? 1 : 0;
    p.ameta = ameta;
    p.bmeta = bmeta;
    p.tbl = tbl;
    p.out = out;
    p.ntiles = triangular ? (unsigned long long)p.ta * (p.ta + 1) / 2 : (unsigned long long)p.ta * p.tb;
    p.tiles = tiles;
    p.row_tbl = row_tbl;
    p.tbl_stride = tbl_stride;
    if (tiles) p.ntiles = nlist;
    if (p.ntiles == 0) return MDET_OK;
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_filter_simt, TH, 0);
    if (per_sm < 1) per_sm = 1;
    unsigned long long grid = (unsigned long long)ctx->num_sms * per_sm * 8;
    if (grid > p.ntiles) grid = p.ntiles;
    ctx_timer_begin(ctx, "k_filter_simt");
    k_filter_simt<<<(unsigned)grid, TH, 0, ctx->stream>>>(p);
    ctx_timer_end(ctx, "k_filter_simt");
    MDET_LAUNCHED(ctx, "k_filter_simt");
    return MDET_OK;
}
