// graph_filter_tc.cu -- tensor-core distance filter (tcgen05, sm_103a).
//
// The pairwise stage restructured as ||a||^2 + ||b||^2 - 2 a.b over centred
// reduced-precision rows: a.b - ||b||^2/2 is a 128 x 256 x 144 tile GEMM per
// (row tile, column tile) -- the column term rides in two spare K columns --
// issued by one thread with tcgen05.mma (kind::f16, BF16 x BF16 -> FP32; or
// kind::tf32 on TF32 rows in FP32 containers, 128 x 128 tiles), operands
// staged in shared memory by TMA (cp.async.bulk.tensor, 128-byte swizzle for
// K 0..127, 32-byte (BF16) or 64-byte (TF32) swizzle for K 128..143),
// accumulators in TMEM (two buffers, so the epilogue of one tile overlaps
// the MMA of the next).  The epilogue reads TMEM with tcgen05.ld and keeps pairs with
//     a~.b~ - ||b~||^2/2 > (||a~||^2 - R^2)/2,
// R = d*_tile + e_a + e_b + slack, where d*_tile bounds the model's distance
// threshold over the tile's sizes and e_a, e_b bound the BF16 rounding of the
// rows (||a~ - a||).  By the triangle inequality no pair whose exact
// distance is below d* is dropped; the exact stage re-scores every kept pair,
// so the edge set equals the plain form's.  Nothing n x n leaves the SM.
//
// Warp roles: 0 = TMA producer, 1 = MMA issuer + TMEM owner, 2.. = epilogue
// (TMEM lane quarter = warp % 4; the groups of four split the tile's columns
// and M halves).
// CTAs take whole row tiles in waves (see the schedule below), so the A tile
// (128 rows) is loaded once per row tile and B tiles stream through a
// two-stage ring.  All waits are bounded.
#include <cudaTypedefs.h>

#include "graph.cuh"

namespace {

constexpr int kBM = 128;
constexpr int kMaxEpiWarps = 16;

// Row layout in shared memory for EB-byte elements (2: BF16, 4: TF32): EB
// chunks of 128 bytes per row (K 0..127, 128-byte swizzle) and a tail of
// 16 elements (K 128..143; 32-byte swizzle for BF16, 64-byte for TF32).
// Every MMA consumes 32 bytes of K per row: four per chunk, EB/2 in the tail.
template <int EB>
struct Elem {
    static constexpr int kChunks = EB;                    // 128-byte K chunks
    static constexpr uint32_t kChunkEl = 128 / EB;         // elements per chunk
    static constexpr uint32_t kTailBytes = 16 * EB;        // bytes per row of the tail
    static constexpr uint32_t kTailLayout = EB == 2 ? 6u : 4u;  // SW32 or SW64 descriptor layout
    static constexpr int kTailSteps = EB / 2;
    static constexpr int kSteps = 4 * kChunks + kTailSteps;      // 9 or 18 MMAs per tile
    static constexpr uint32_t kFormat = EB == 2 ? 1u : 2u;     // instruction-descriptor A/B format: BF16, TF32
};

// Tile shapes: BM rows (one or two M = 128 MMAs) x BN columns, with NST
// stages of B tiles in shared memory.  BF16: 128 x 256 x 2 and 256 x 128 x 4
// run one CTA per SM, 128 x 128 x 2 runs two; a 256-row tile reads each B
// tile for twice the rows, halving the B traffic per output.  TF32 rows are
// twice as wide: 128 x 128 x 2 (216 KB of operands) runs one CTA per SM.
template <int BM, int BN, int NST, int EB = 2>
struct Shape {
    using E = Elem<EB>;
    static constexpr int MH = BM / 128;                         // M halves
    static constexpr uint32_t kAChunk = kBM * 128;              // one 128-byte K chunk of an A half
    static constexpr uint32_t kABytes = E::kChunks * kAChunk + kBM * E::kTailBytes;
    static constexpr uint32_t kABytesAll = MH * kABytes;
    static constexpr uint32_t kBChunk = BN * 128;               // one 128-byte K chunk of B
    static constexpr uint32_t kBBytes = E::kChunks * kBChunk + BN * E::kTailBytes;
    static constexpr uint32_t kAccCols = MH * BN;               // one accumulator
    static constexpr uint32_t kTmemCols = 2 * kAccCols;         // double buffered
    static constexpr uint32_t kSmemBytes = kABytesAll + NST * kBBytes + 1024;  // + alignment slack
    static constexpr int kCtasPerSm = (BM == 128 && BN == 128 && EB == 2) ? 2 : 1;
    // epilogue warps: 4 TMEM lane quarters x one group per 64 columns of each
    // M half (16 for the 128 x 256 and 256 x 128 shapes, 8 for 128 x 128), so
    // each warp reads one 64-column chunk of its quarter per tile.
    static constexpr int kEpi = 4 * (BN / 64) * MH;
    static constexpr int kThreads = (2 + kEpi) * 32;
    static constexpr int kGroupsPerHalf = kEpi / 4 / MH;
    static constexpr uint32_t kWarpCols = BN / kGroupsPerHalf;
    // candidate queue per epilogue warp, within the shared memory left
    static constexpr int kQueue = kCtasPerSm == 2 ? 32 : (kSmemBytes + kEpi * 256 * 8 <= 227 * 1024 ? 256 : 64);
    static_assert(kWarpCols == 64, "each epilogue warp reads one 64-column chunk per tile");
    static_assert(kSmemBytes + kEpi * kQueue * 8 + 512 <= 227 * 1024, "shared memory of one CTA");
    // BF16 x BF16 or TF32 x TF32 -> FP32 (D format bits 4-5), A/B formats
    // (bits 7-9, 10-12), M = 128, N = BN, A and B K-major.
    static constexpr uint32_t kIdesc = (1u << 4) | (E::kFormat << 7) | (E::kFormat << 10) |
                                       ((uint32_t)(BN >> 3) << 17) | ((uint32_t)(128 >> 4) << 24);
    static_assert(kTmemCols <= 512, "TMEM holds 512 columns");
    static_assert(NST <= 4, "at most four B stages");
};

struct TcArgs {
    uint32_t na, nb, ta, tb, segs;
    uint32_t jnum, jden;  // the first column tile of row tile I is I * jnum / jden (BM / 128, BN / 128)
    const uint32_t* tiles;  // optional list of tiles (I * tb + J, row-major); null: full schedule
    uint64_t nlist;
    const unsigned long long* rowoff;  // optional: list entries of row tile I are [rowoff[I], rowoff[I+1])
    const uint8_t* row_tbl;  // optional table index per row tile (tables tbl_stride floats apart)
    uint64_t tbl_stride;
    int triangular;
    const float* a_nsq;
    const BlockMeta* ameta;
    const BlockMeta* bmeta;
    DstarTable tbl;
    CandBuf out;
    unsigned long long ntiles;
    int* flag;
};

struct __align__(8) Ctl {
    uint64_t a_full, a_empty;
    uint64_t b_full[4], b_empty[4];
    uint64_t acc_full[2], acc_empty[2];
    uint32_t tmem_base;
    uint32_t qcount[kMaxEpiWarps];
    float r2[2];  // one-half shapes: R^2 of the tile in each accumulator
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
constexpr uint32_t kLayoutSW128 = 2;

template <int EB>
__device__ __forceinline__ void mma_rows(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                         uint32_t accumulate) {
    if constexpr (EB == 2) {
        asm volatile(
            "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
            " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem_d),
            "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
            : "memory");
    } else {
        asm volatile(
            "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
            " tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem_d),
            "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
            : "memory");
    }
}

__device__ __forceinline__ void mma_commit(uint64_t* bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
                 : "memory");
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// max(a, b, c) in one instruction (three-source max.f32)
__device__ __forceinline__ float max3f(float a, float b, float c) {
    float r;
    asm("max.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
    return r;
}

// 64 consecutive FP32 columns of this thread's TMEM lane; the wait sits in
// the same asm statement, so no use of the registers can be scheduled early.
__device__ __forceinline__ void tmem_ld64(uint32_t taddr, float (&v)[64]) {
    uint32_t r[64];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x64.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
        "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31,"
        "%32,%33,%34,%35,%36,%37,%38,%39,%40,%41,%42,%43,%44,%45,%46,%47,"
        "%48,%49,%50,%51,%52,%53,%54,%55,%56,%57,%58,%59,%60,%61,%62,%63}, [%64];\n"
        "tcgen05.wait::ld.sync.aligned;\n"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
          "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
          "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31]),
          "=r"(r[32]), "=r"(r[33]), "=r"(r[34]), "=r"(r[35]), "=r"(r[36]), "=r"(r[37]), "=r"(r[38]), "=r"(r[39]),
          "=r"(r[40]), "=r"(r[41]), "=r"(r[42]), "=r"(r[43]), "=r"(r[44]), "=r"(r[45]), "=r"(r[46]), "=r"(r[47]),
          "=r"(r[48]), "=r"(r[49]), "=r"(r[50]), "=r"(r[51]), "=r"(r[52]), "=r"(r[53]), "=r"(r[54]), "=r"(r[55]),
          "=r"(r[56]), "=r"(r[57]), "=r"(r[58]), "=r"(r[59]), "=r"(r[60]), "=r"(r[61]), "=r"(r[62]), "=r"(r[63])
        : "r"(taddr)
        : "memory");
#pragma unroll
    for (int k = 0; k < 64; ++k) v[k] = __uint_as_float(r[k]);
}

// Squared pass radius of row block ib against column tile J:
// R = d*_tile + e_a + e_b + slack, where d*_tile bounds the model's distance
// threshold over the blocks' sizes, e_a and e_b bound the BF16 rounding of the
// rows, and the slack covers FP32 accumulation and the two-term split of
// ||b~||^2/2.
//
// It takes two dependent rounds of loads (block metadata, then the two d*
// table cells), split here so that a caller can run them ahead of use.
struct R2Meta {  // first loads: the blocks' metadata and the table selector
    BlockMeta ma, mb0, mb1;
    uint32_t tsel;
};
struct R2Cells {  // second loads: the table cells (in flight) and the other terms
    float t0, t1, E, N;
};
template <int BN>
__device__ __forceinline__ R2Meta r2_meta(const TcArgs& p, uint32_t ib, uint32_t J) {
    constexpr uint32_t kBlk = BN / MDET_BLK;  // metadata blocks per column tile
    R2Meta m;
    m.ma = p.ameta[ib];
    m.mb0 = p.bmeta[kBlk * J];
    m.mb1 = p.bmeta[kBlk * J + kBlk - 1];
    m.tsel = p.row_tbl ? p.row_tbl[ib] : 0u;
    return m;
}
// tbase: p.tbl with the dynamic grid (if any) already read
__device__ __forceinline__ R2Cells r2_cells(const TcArgs& p, const DstarTable& tbase, const R2Meta& m) {
    DstarTable tb = tbase;
    tb.st += (uint64_t)m.tsel * p.tbl_stride;
    const float *c0, *c1;
    tile_dstar_cells(tb, m.ma.lo, m.ma.hi, fminf(m.mb0.lo, m.mb1.lo), fmaxf(m.mb0.hi, m.mb1.hi), c0, c1);
    R2Cells c;
    c.t0 = __ldg(c0);
    c.t1 = __ldg(c1);
    c.E = m.ma.emax + fmaxf(m.mb0.emax, m.mb1.emax);
    const float nb = fmaxf(m.mb0.nmax, m.mb1.nmax);
    c.N = m.ma.nmax * nb + nb * nb;
    return c;
}
__device__ __forceinline__ float r2_finish(const R2Cells& c) {
    const float R = fmaxf(c.t0, c.t1) * (1.f + 2e-5f) + 1e-6f + c.E;
    float R2 = R * R + 4e-5f * c.N + 1e-7f;
    if (!(R2 < 1e30f)) R2 = __int_as_float(0x7f800000);
    return R2;
}
__device__ __forceinline__ DstarTable table_base(const TcArgs& p) {
    DstarTable tb = p.tbl;
    if (tb.dyn) {
        tb.lmin = tb.dyn[0];
        tb.inv_h = tb.dyn[1];
    }
    return tb;
}
template <int BN>
__device__ __forceinline__ float tile_r2(const TcArgs& p, uint32_t ib, uint32_t J) {
    return r2_finish(r2_cells(p, table_base(p), r2_meta<BN>(p, ib, J)));
}

// ------------------------------------------------------------ schedule --
// Waves of G row tiles (G = grid size): in wave w, CTA c takes row tile
// w*G + c (w even) or w*G + G-1-c (w odd), and walks its column tiles J from
// j_start(I) upward.  All CTAs of a wave sweep the same B tiles at about the
// same time, so each B tile comes from DRAM about once per wave and from L2
// for the other CTAs; the snake order evens out the triangular row lengths.

__device__ __forceinline__ uint32_t j_start(const TcArgs& p, uint32_t I) {
    return p.triangular ? (I * p.jnum) / p.jden : 0u;
}

// A work unit is one segment of one row tile's column range: p.segs segments
// per row tile (1 when row tiles outnumber the CTAs).
struct Cursor {
    uint32_t I, J, Jend, w;
    uint64_t li, lend;  // list mode: current and end index
    bool valid;
};

__device__ __forceinline__ uint32_t unit_of_wave(uint32_t w, uint32_t c, uint32_t G) {
    return w * G + ((w & 1) ? (G - 1 - c) : c);
}

__device__ __forceinline__ bool set_unit(const TcArgs& p, Cursor& k, uint32_t u) {
    const uint32_t I = u / p.segs, seg = u % p.segs;
    if (I >= p.ta) return false;
    const uint32_t j0 = j_start(p, I), len = p.tb - j0;
    k.I = I;
    k.J = j0 + (uint32_t)((uint64_t)len * seg / p.segs);
    k.Jend = j0 + (uint32_t)((uint64_t)len * (seg + 1) / p.segs);
    return true;
}

__device__ __forceinline__ void advance(const TcArgs& p, Cursor& k, uint32_t c, uint32_t G);

__device__ __forceinline__ void list_decode(const TcArgs& p, Cursor& k) {
    k.valid = k.li < k.lend;
    if (k.valid) {
        const uint32_t t = p.tiles[k.li];
        k.I = t / p.tb;
        k.J = t % p.tb;
    }
}

// Wave-ordered list: row tiles in the waves of the full schedule, each row
// tile's listed column tiles in order (so concurrent CTAs sweep the same B
// tiles, as in the full schedule).  Moves to the first non-empty row tile
// from wave k.w on.
__device__ __forceinline__ void list_next_row(const TcArgs& p, Cursor& k, uint32_t c, uint32_t G) {
    while (true) {
        const uint32_t I = unit_of_wave(k.w, c, G);
        if (I >= p.ta) {
            k.valid = false;
            return;
        }
        k.li = p.rowoff[I];
        k.lend = p.rowoff[I + 1];
        if (k.li < k.lend) {
            list_decode(p, k);
            return;
        }
        ++k.w;
    }
}

__device__ __forceinline__ Cursor cursor_first(const TcArgs& p, uint32_t c, uint32_t G) {
    Cursor k;
    if (p.tiles && p.rowoff) {
        k.w = 0;
        list_next_row(p, k, c, G);
        return k;
    }
    if (p.tiles) {
        // list mode: CTA c takes a contiguous range of the row-major list
        k.li = p.nlist * c / G;
        k.lend = p.nlist * (c + 1) / G;
        list_decode(p, k);
        return k;
    }
    k.w = 0;
    k.valid = set_unit(p, k, unit_of_wave(0, c, G));
    if (k.valid && k.J >= k.Jend) advance(p, k, c, G);  // empty segment
    return k;
}

__device__ __forceinline__ void advance(const TcArgs& p, Cursor& k, uint32_t c, uint32_t G) {
    if (p.tiles && p.rowoff) {
        if (++k.li < k.lend) {
            list_decode(p, k);
            return;
        }
        ++k.w;
        list_next_row(p, k, c, G);
        return;
    }
    if (p.tiles) {
        ++k.li;
        list_decode(p, k);
        return;
    }
    if (++k.J < k.Jend) return;
    while (true) {
        ++k.w;
        if (!set_unit(p, k, unit_of_wave(k.w, c, G))) {
            k.valid = false;
            return;
        }
        if (k.J < k.Jend) return;
    }
}

// -------------------------------------------------------------- kernel --

// tmA32/tmB32: the K 128..143 tail (32-byte swizzle for BF16, 64-byte for TF32)
template <int BM, int BN, int NST, int EB>
__global__ void __launch_bounds__(Shape<BM, BN, NST, EB>::kThreads, Shape<BM, BN, NST, EB>::kCtasPerSm)
    k_filter_tc(const __grid_constant__ CUtensorMap tmA128, const __grid_constant__ CUtensorMap tmA32,
                const __grid_constant__ CUtensorMap tmB128, const __grid_constant__ CUtensorMap tmB32, TcArgs p) {
    using S = Shape<BM, BN, NST, EB>;
    using E = typename S::E;
    extern __shared__ unsigned char smem_raw[];
    __shared__ Ctl ctl;
    constexpr int kQueue = S::kQueue;
    __shared__ uint2 queue[S::kEpi][kQueue];
    unsigned char* smem = (unsigned char*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    unsigned char* sA = smem;
    unsigned char* sB = smem + S::kABytesAll;
    const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

    const uint32_t G = gridDim.x, cta = blockIdx.x;

    if (threadIdx.x == 0) {
        mbar_init(&ctl.a_full, 1);
        mbar_init(&ctl.a_empty, 1);
        for (int s = 0; s < NST; ++s) {
            mbar_init(&ctl.b_full[s], 1);
            mbar_init(&ctl.b_empty[s], 1);
        }
        for (int s = 0; s < 2; ++s) {
            // one-half shapes: the MMA commit and the tile's R^2 written
            mbar_init(&ctl.acc_full[s], S::MH == 1 ? 2 : 1);
            mbar_init(&ctl.acc_empty[s], S::kEpi * 32);
        }
        for (int w = 0; w < S::kEpi; ++w) ctl.qcount[w] = 0;
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
                     "r"(S::kTmemCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = ctl.tmem_base;

    {
        if (warp == 0) {
            // ------------------------------------------------ TMA producer
            if (lane == 0) {
                Cursor c = cursor_first(p, cta, G);
                uint32_t a_e_ph = 0, b_e_ph[NST];
#pragma unroll
                for (int t = 0; t < NST; ++t) b_e_ph[t] = 0;
                uint32_t curI = 0xFFFFFFFFu;
                for (uint32_t lt = 0; c.valid; ++lt, advance(p, c, cta, G)) {
                    if (c.I != curI) {
                        if (!mbar_wait(&ctl.a_empty, a_e_ph ^ 1, p.flag)) break;
                        a_e_ph ^= 1;
                        mbar_arrive_tx(&ctl.a_full, S::kABytesAll);
#pragma unroll
                        for (int h = 0; h < S::MH; ++h) {
                            const int y = (int)(c.I * BM + h * 128);
                            unsigned char* dA = sA + h * S::kABytes;
#pragma unroll
                            for (int ch = 0; ch < E::kChunks; ++ch)
                                tma_load_2d(dA + ch * S::kAChunk, &tmA128, ch * (int)E::kChunkEl, y, &ctl.a_full);
                            tma_load_2d(dA + E::kChunks * S::kAChunk, &tmA32, 128, y, &ctl.a_full);
                        }
                        curI = c.I;
                    }
                    const uint32_t bs = lt % NST;
                    if (!mbar_wait(&ctl.b_empty[bs], b_e_ph[bs] ^ 1, p.flag)) break;
                    b_e_ph[bs] ^= 1;
                    unsigned char* dst = sB + bs * S::kBBytes;
                    mbar_arrive_tx(&ctl.b_full[bs], S::kBBytes);
                    const int y = (int)(c.J * BN);
#pragma unroll
                    for (int ch = 0; ch < E::kChunks; ++ch)
                        tma_load_2d(dst + ch * S::kBChunk, &tmB128, ch * (int)E::kChunkEl, y, &ctl.b_full[bs]);
                    tma_load_2d(dst + E::kChunks * S::kBChunk, &tmB32, 128, y, &ctl.b_full[bs]);
                }
            }
        } else if (warp == 1) {
            // -------------------------------------------------- MMA issuer
            if (lane == 0) {
                Cursor c = cursor_first(p, cta, G);
                // one-half shapes: the R^2 loads run ahead (metadata two tiles,
                // table cells one tile), so only arithmetic sits between MMA batches
                Cursor n1 = c;
                if (n1.valid) advance(p, n1, cta, G);
                const DstarTable tbase = table_base(p);
                R2Cells cc{};
                R2Meta mn{};
                if constexpr (S::MH == 1) {
                    if (c.valid) cc = r2_cells(p, tbase, r2_meta<BN>(p, c.I, c.J));
                    if (n1.valid) mn = r2_meta<BN>(p, n1.I, n1.J);
                }
                uint32_t a_ph = 0, b_ph[NST], e_ph[2] = {0, 0};
#pragma unroll
                for (int t = 0; t < NST; ++t) b_ph[t] = 0;
                uint32_t curI = 0xFFFFFFFFu;
                const uint32_t a_base = smem_u32(sA), b_base = smem_u32(sB);
                for (uint32_t lt = 0; c.valid; ++lt) {
                    if (c.I != curI) {
                        if (!mbar_wait(&ctl.a_full, a_ph, p.flag)) break;
                        a_ph ^= 1;
                        curI = c.I;
                    }
                    const uint32_t s = lt & 1, bs = lt % NST;
                    if (!mbar_wait(&ctl.acc_empty[s], e_ph[s] ^ 1, p.flag)) break;
                    e_ph[s] ^= 1;
                    if (!mbar_wait(&ctl.b_full[bs], b_ph[bs], p.flag)) break;
                    b_ph[bs] ^= 1;
                    tc_fence_after();
                    const uint32_t bb = b_base + bs * S::kBBytes;
#pragma unroll
                    for (int h = 0; h < S::MH; ++h) {
                        const uint32_t d = tmem + s * S::kAccCols + h * BN;
                        const uint32_t ab = a_base + h * S::kABytes;
#pragma unroll
                        for (int k = 0; k < E::kSteps; ++k) {
                            uint64_t ad, bd;
                            if (k < 4 * E::kChunks) {
                                const uint32_t ch = k >> 2, ko = (k & 3) * 32;
                                ad = smem_desc(ab + ch * S::kAChunk + ko, kLayoutSW128, 1024);
                                bd = smem_desc(bb + ch * S::kBChunk + ko, kLayoutSW128, 1024);
                            } else {
                                // tail: 8-row core groups E::kTailBytes * 8 apart, 32 bytes of K per step
                                const uint32_t ko = (k - 4 * E::kChunks) * 32;
                                ad = smem_desc(ab + E::kChunks * S::kAChunk + ko, E::kTailLayout, 8 * E::kTailBytes);
                                bd = smem_desc(bb + E::kChunks * S::kBChunk + ko, E::kTailLayout, 8 * E::kTailBytes);
                            }
                            mma_rows<EB>(d, ad, bd, S::kIdesc, k > 0 ? 1u : 0u);
                        }
                    }
                    mma_commit(&ctl.b_empty[bs]);
                    mma_commit(&ctl.acc_full[s]);
                    Cursor n2 = n1;
                    if (n2.valid) advance(p, n2, cta, G);
                    if constexpr (S::MH == 1) {
                        // the tile's R^2 for the epilogue (the epilogue of the
                        // tile that used this slot before is done: acc_empty)
                        ctl.r2[s] = r2_finish(cc);
                        mbar_arrive(&ctl.acc_full[s]);
                        if (n1.valid) cc = r2_cells(p, tbase, mn);
                        if (n2.valid) mn = r2_meta<BN>(p, n2.I, n2.J);
                    }
                    if (!n1.valid || n1.I != c.I) mma_commit(&ctl.a_empty);
                    c = n1;
                    n1 = n2;
                }
            }
        } else {
            // ---------------------------------------------------- epilogue
            const uint32_t ew = warp - 2;           // 0 .. kEpi - 1
            const uint32_t quarter = warp & 3;      // TMEM lanes 32*quarter ..
            const uint32_t grp = ew >> 2;
            const uint32_t mh = grp / S::kGroupsPerHalf;                      // M half of this warp
            const uint32_t cbase = (grp % S::kGroupsPerHalf) * S::kWarpCols;  // first column of this warp
            uint32_t* qc = &ctl.qcount[ew];
            uint2* q = queue[ew];
            Cursor c = cursor_first(p, cta, G);
            uint32_t f_ph[2] = {0, 0};
            uint32_t curI = 0xFFFFFFFFu;
            float ansq = 0.f;
            for (uint32_t lt = 0; c.valid; ++lt, advance(p, c, cta, G)) {
                const uint32_t s = lt & 1;
                const uint32_t row = c.I * BM + mh * 128 + quarter * 32 + lane;
                // TMEM holds a~.b~ - ||b~||^2/2 (the column term rides in K
                // columns 136/137); the pair passes when it exceeds
                // hr = (||a~||^2 - R^2)/2.  One-half shapes take R^2 from the
                // MMA thread; the two-half shape computes it here per M half.
                if (c.I != curI) {  // ||a~||^2 of this lane's row, once per row tile
                    ansq = __ldg(p.a_nsq + row);
                    curI = c.I;
                }
                float r2_own = 0.f;
                if constexpr (S::MH != 1) r2_own = tile_r2<BN>(p, c.I * S::MH + mh, c.J);
                const bool diag = p.triangular && (c.J * BN < c.I * BM + BM);
                const bool ok = mbar_wait(&ctl.acc_full[s], f_ph[s], p.flag);
                if (!__all_sync(0xffffffffu, ok)) break;  // warp-uniform, so tcgen05.ld stays converged
                f_ph[s] ^= 1;
                tc_fence_after();
                const float hr = 0.5f * (ansq - (S::MH == 1 ? ctl.r2[s] : r2_own));
                const uint32_t gc0 = c.J * BN + cbase;
                unsigned long long mask = 0;  // this lane's hits: bit k = column gc0 + k
                {
                    float v[64];
                    tmem_ld64(tmem + ((quarter * 32) << 16) + s * S::kAccCols + mh * BN + cbase, v);
                    float mx[8];
#pragma unroll
                    for (int t = 0; t < 8; ++t) {
                        float a = max3f(v[t], v[t + 8], v[t + 16]);
                        a = max3f(a, v[t + 24], v[t + 32]);
                        a = max3f(a, v[t + 40], v[t + 48]);
                        mx[t] = fmaxf(a, v[t + 56]);
                    }
                    const float m = max3f(max3f(mx[0], mx[1], mx[2]), max3f(mx[3], mx[4], mx[5]), fmaxf(mx[6], mx[7]));
                    if (m > hr) {
#pragma unroll
                        for (int t = 0; t < 8; ++t) {
                            if (mx[t] > hr) {
#pragma unroll
                                for (int j = 0; j < 8; ++j)
                                    mask |= (unsigned long long)(v[t + 8 * j] > hr ? 1u : 0u) << (t + 8 * j);
                            }
                        }
                    }
                }
                // the hits are in registers: release the accumulator before emitting
                tc_fence_before();
                mbar_arrive(&ctl.acc_empty[s]);
                while (mask) {
                    const int k = __ffsll((long long)mask) - 1;
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
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(S::kTmemCols)
                     : "memory");
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

// Tensor map over [rows][144] elements of eb bytes (2: BF16, 4: FP32 holding
// TF32 values), box {box_k elements, box_rows rows}.
int make_map(mdet_ctx* ctx, CUtensorMap* map, const void* base, uint64_t rows, uint32_t box_k, uint32_t box_rows,
             CUtensorMapSwizzle sw, int eb) {
    auto enc = get_encode(ctx);
    if (!enc) return ctx_fail(ctx, MDET_ERR_CUDA, "cuTensorMapEncodeTiled unavailable");
    cuuint64_t dims[2] = {MDET_KPAD, rows};
    cuuint64_t strides[1] = {(cuuint64_t)MDET_KPAD * eb};
    cuuint32_t box[2] = {box_k, box_rows};
    cuuint32_t es[2] = {1, 1};
    CUresult r = enc(map, eb == 4 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32 : CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2,
                     (void*)base, dims, strides, box, es,
                     CU_TENSOR_MAP_INTERLEAVE_NONE, sw, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                     CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return ctx_fail(ctx, MDET_ERR_CUDA, "cuTensorMapEncodeTiled failed (%d)", (int)r);
    return MDET_OK;
}

template <int BM, int BN, int NST, int EB>
int launch_tc(mdet_ctx* ctx, const void* a, const float* a_nsq, uint32_t na, const BlockMeta* ameta,
              const void* b, uint32_t nb, const BlockMeta* bmeta, bool triangular, const DstarTable& tbl,
              CandBuf out, const uint32_t* tiles, uint64_t nlist, const uint8_t* row_tbl, uint64_t tbl_stride,
              const unsigned long long* rowoff) {
    using S = Shape<BM, BN, NST, EB>;
    using E = typename S::E;
    const uint64_t na_pad = (na + 255) / 256 * 256, nb_pad = (nb + 255) / 256 * 256;
    const CUtensorMapSwizzle tail_sw = EB == 2 ? CU_TENSOR_MAP_SWIZZLE_32B : CU_TENSOR_MAP_SWIZZLE_64B;
    CUtensorMap mA128, mA32, mB128, mB32;
    MDET_TRY(make_map(ctx, &mA128, a, na_pad, E::kChunkEl, kBM, CU_TENSOR_MAP_SWIZZLE_128B, EB));
    MDET_TRY(make_map(ctx, &mA32, a, na_pad, 16, kBM, tail_sw, EB));
    MDET_TRY(make_map(ctx, &mB128, b, nb_pad, E::kChunkEl, BN, CU_TENSOR_MAP_SWIZZLE_128B, EB));
    MDET_TRY(make_map(ctx, &mB32, b, nb_pad, 16, BN, tail_sw, EB));
    TcArgs p;
    p.na = na;
    p.nb = nb;
    p.ta = (na + BM - 1) / BM;
    p.tb = (nb + BN - 1) / BN;
    p.jnum = BM / 128;
    p.jden = BN / 128;
    p.triangular = triangular ? 1 : 0;
    p.a_nsq = a_nsq;
    p.ameta = ameta;
    p.bmeta = bmeta;
    p.tbl = tbl;
    p.out = out;
    p.flag = ctx->d_flag;
    p.ntiles = 0;
    static bool attr[64] = {false};
    if (!attr[ctx->device & 63]) {
        MDET_CUDA(ctx, cudaFuncSetAttribute(k_filter_tc<BM, BN, NST, EB>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                            (int)S::kSmemBytes));
        attr[ctx->device & 63] = true;
    }
    const uint32_t ctas = (uint32_t)ctx->num_sms * S::kCtasPerSm;
    // enough work units for every CTA: split row tiles into column segments when they are few
    p.segs = 1;
    while ((uint64_t)p.ta * p.segs < 2ull * ctas && p.segs < p.tb) ++p.segs;
    p.tiles = tiles;
    p.nlist = nlist;
    p.rowoff = tiles ? rowoff : nullptr;
    p.row_tbl = row_tbl;
    p.tbl_stride = tbl_stride;
    unsigned grid =
        (unsigned)std::min<unsigned long long>(ctas, tiles ? nlist : (unsigned long long)p.ta * p.segs);
    if (p.rowoff) grid = (unsigned)std::min<unsigned long long>(grid, p.ta);  // one row tile per CTA and wave
    if (grid == 0) return MDET_OK;
    ctx_timer_begin(ctx, "k_filter_tc");
    k_filter_tc<BM, BN, NST, EB><<<grid, S::kThreads, S::kSmemBytes, ctx->stream>>>(mA128, mA32, mB128, mB32, p);
    ctx_timer_end(ctx, "k_filter_tc");
    MDET_LAUNCHED(ctx, "k_filter_tc");
    return MDET_OK;
}

}  // namespace

int filter_tc(mdet_ctx* ctx, const void* a, const float* a_nsq, uint32_t na, const BlockMeta* ameta,
              const void* b, uint32_t nb, const BlockMeta* bmeta, bool triangular, const DstarTable& tbl,
              CandBuf out, const uint32_t* tiles, uint64_t nlist, const uint8_t* row_tbl, uint64_t tbl_stride,
              int bn, const unsigned long long* rowoff) {
    if (na == 0 || nb == 0) return MDET_OK;
    if (bn == kShapeTf32)
        return launch_tc<128, 128, 2, 4>(ctx, a, a_nsq, na, ameta, b, nb, bmeta, triangular, tbl, out, tiles, nlist,
                                         row_tbl, tbl_stride, rowoff);
    if (bn == 128)
        return launch_tc<128, 128, 2, 2>(ctx, a, a_nsq, na, ameta, b, nb, bmeta, triangular, tbl, out, tiles, nlist,
                                         row_tbl, tbl_stride, rowoff);
    if (bn == kShapeTall) {
        if (tiles) return ctx_fail(ctx, MDET_ERR_INVALID, "tile lists use 128-row tiles");
        return launch_tc<256, 128, 4, 2>(ctx, a, a_nsq, na, ameta, b, nb, bmeta, triangular, tbl, out, tiles, nlist,
                                         row_tbl, tbl_stride, rowoff);
    }
    return launch_tc<128, 256, 2, 2>(ctx, a, a_nsq, na, ameta, b, nb, bmeta, triangular, tbl, out, tiles, nlist,
                                     row_tbl, tbl_stride, rowoff);
}
