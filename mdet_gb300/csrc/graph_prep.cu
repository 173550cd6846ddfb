// graph_prep.cu -- per-call preparation of the pairwise stage.
//
// Contigs are put in ascending log-size order (stable, by original index on
// ties) so that every tile of the pairwise schedule covers a narrow range of
// sizes; the size-dependent distance threshold d*(x, y) of the MetaBAT2
// model (cuda/Cuda2.cu:199-240 solved for d) is then nearly constant over a
// tile and one conservative bound per tile filters its pairs.  This file
// builds: the permutation, sorted FP32 rows and log sizes, the per-contig
// FP64 model parts used by the exact stage, the centred BF16 rows with their
// norms and rounding errors for the tensor-core filter, per-block metadata,
// and the d* table.
#include <cub/cub.cuh>

#include <string>

#include <cmath>
#include <cstring>

#include "graph.cuh"

namespace {

__device__ __forceinline__ unsigned long long dkey(double v) {
    unsigned long long b = (unsigned long long)__double_as_longlong(v);
    return (b & 0x8000000000000000ull) ? ~b : (b | 0x8000000000000000ull);
}

__global__ void k_keys(const double* __restrict__ ls, uint64_t n, unsigned long long* __restrict__ keys,
                       uint32_t* __restrict__ vals) {
    uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    keys[i] = dkey(ls[i]);
    vals[i] = (uint32_t)i;
}

__device__ __forceinline__ double poly(const double* c, int deg, double v) {
    double r = c[deg];
    for (int k = deg - 1; k >= 0; --k) r = fma(r, v, c[k]);
    return r;
}

// Warp per position s of [0, npad) of one contig set placed at row `base`
// of the prepared arrays (all pointers here already offset by base): perm
// arrives with local original indices and leaves with base + local; inv is
// the full array.  Padding positions map to themselves.  The row is copied
// by the whole warp; the nine FP64 polynomials of the model parts run on
// nine lanes side by side (FP64 is a narrow unit here, so one long serial
// chain per row would bound the kernel).
__global__ void k_gather(const float* __restrict__ tnf, const double* __restrict__ ls, uint32_t* __restrict__ perm,
                         uint64_t n, uint64_t npad, uint32_t base, uint32_t* __restrict__ inv,
                         float* __restrict__ x32, double* __restrict__ ls_s, PartsFF* __restrict__ parts,
                         ModelSplit ms) {
    const uint64_t s = blockIdx.x * (uint64_t)(blockDim.x / 32) + (threadIdx.x >> 5);
    const uint32_t lane = threadIdx.x & 31;
    if (s >= npad) return;
    if (s >= n) {
        if (lane == 0) {
            perm[s] = base + (uint32_t)s;
            inv[base + s] = base + (uint32_t)s;
        }
        return;
    }
    uint32_t o = 0;
    if (lane == 0) o = perm[s];
    o = __shfl_sync(0xffffffffu, o, 0);  // read by lane 0 before lane 0 rewrites it below
    const float* src = tnf + (uint64_t)o * MDET_NTNF;
    float* dst = x32 + s * MDET_NTNF;
    for (int k = lane; k < MDET_NTNF; k += 32) dst[k] = src[k];
    const double v = ls[o];
    if (lane == 0) {
        perm[s] = base + o;
        inv[base + o] = base + (uint32_t)s;
        ls_s[s] = v;
    }
    // lanes 0-3: f[m] = F_m(v) (degree 7); lanes 4-7: g[m] = G_m(v) without
    // its constant (degree 6); lane 8: the log size itself
    ff* out = reinterpret_cast<ff*>(parts + s);  // f[0..3], g[0..3], ls
    if (lane < 4) {
        out[lane] = ff_from_double(poly(ms.F[lane], 7, v));
    } else if (lane < 8) {
        const int m = lane - 4;
        double r = ms.G[m][6];
        for (int k = 5; k >= 1; --k) r = fma(r, v, ms.G[m][k]);
        out[lane] = ff_from_double(r * v);
    } else if (lane == 8) {
        out[8] = ff_from_double(v);
    } else if (lane == 9) {
        parts[s].pad[0] = 0.f;
        parts[s].pad[1] = 0.f;
    }
}

__global__ void k_colsum(const float* __restrict__ x32, uint64_t n, double* __restrict__ sums) {
    // block: 136 threads (one per column), rows strided over the grid
    int k = threadIdx.x;
    if (k >= MDET_NTNF) return;
    double acc = 0;
    for (uint64_t s = blockIdx.x; s < n; s += gridDim.x) acc += x32[s * MDET_NTNF + k];
    atomicAdd(&sums[k], acc);
}

__global__ void k_mean(const double* __restrict__ sums, uint64_t n, float* __restrict__ mu) {
    int k = threadIdx.x;
    if (k < MDET_NTNF) mu[k] = (float)(sums[k] / (double)n);
}

// Warp per sorted row: centred BF16 copies in both GEMM roles, the squared
// norm of the rounded row, and its exact distance to the unrounded centred
// row.  Columns 136/137 fold the column term of ||a||^2+||b||^2-2a.b into the
// GEMM: the A role carries 1, 1 and the B role -hi, -lo of ||b~||^2/2 (a
// two-term BF16 split), so a.b' = a.b - ||b~||^2/2 comes out of TMEM.
__global__ void k_bf16(const float* __restrict__ x32, const float* __restrict__ mu, uint64_t n, uint64_t npad,
                       uint16_t* __restrict__ xa, uint16_t* __restrict__ xb, float* __restrict__ nsq,
                       float* __restrict__ err, float* __restrict__ nrm) {
    uint64_t s = blockIdx.x * (uint64_t)(blockDim.x / 32) + (threadIdx.x >> 5);
    uint32_t lane = threadIdx.x & 31;
    if (s >= npad) return;
    uint16_t* rowa = xa + s * MDET_KPAD;
    uint16_t* rowb = xb + s * MDET_KPAD;
    const uint16_t one = 0x3F80;      // bf16 1.0
    const uint16_t neg_inf = 0xFF80;  // bf16 -inf
    if (s >= n) {
        for (int k = lane; k < MDET_KPAD; k += 32) {
            rowa[k] = (k == MDET_NTNF || k == MDET_NTNF + 1) ? one : 0;
            rowb[k] = (k == MDET_NTNF) ? neg_inf : 0;
        }
        if (lane == 0) {
            nsq[s] = __int_as_float(0x7f800000);
            err[s] = 0.f;
            nrm[s] = 0.f;
        }
        return;
    }
    // FP32 throughout (FP64 is a narrow unit here).  hv^2 is exact in FP32
    // (8-bit significands), so a float-float accumulator gives ||x~||^2
    // exactly to ~2^-44; the rounding error d = hv - (a - mu) is exact per
    // entry up to one FP32 rounding (TwoSum of a - mu; v - hv is exact by
    // Sterbenz), and its sum of squares is inflated before the square root
    // is rounded up, so err stays an upper bound of ||x~ - x||.
    float e2 = 0.f;
    ff q = ff_make(0.f, 0.f);
    for (int k = lane; k < MDET_NTNF; k += 32) {
        const float a = x32[s * MDET_NTNF + k];
        const ff v = two_sum(a, -mu[k]);  // v.hi + v.lo == a - mu exactly
        const __nv_bfloat16 h = __float2bfloat16_rn(v.hi);
        const uint16_t b = *reinterpret_cast<const uint16_t*>(&h);
        const float hv = __bfloat162float(h);
        const float d = __fadd_rn(__fsub_rn(v.hi, hv), v.lo);
        e2 = __fmaf_rn(d, d, e2);
        q = ff_add_f(q, __fmul_rn(hv, hv));
        rowa[k] = b;
        rowb[k] = b;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        e2 += __shfl_xor_sync(0xffffffffu, e2, o);
        ff t;
        t.hi = __shfl_xor_sync(0xffffffffu, q.hi, o);
        t.lo = __shfl_xor_sync(0xffffffffu, q.lo, o);
        q = ff_add(q, t);
    }
    const float half = 0.5f * q.hi;
    const __nv_bfloat16 hi = __float2bfloat16_rn(half);
    const __nv_bfloat16 lo = __float2bfloat16_rn(half - __bfloat162float(hi));
    const uint16_t nhi = *reinterpret_cast<const uint16_t*>(&hi) ^ 0x8000u;
    const uint16_t nlo = *reinterpret_cast<const uint16_t*>(&lo) ^ 0x8000u;
    for (int k = MDET_NTNF + lane; k < MDET_KPAD; k += 32) {
        rowa[k] = (k < MDET_NTNF + 2) ? one : 0;
        rowb[k] = k == MDET_NTNF ? nhi : (k == MDET_NTNF + 1 ? nlo : 0);
    }
    if (lane == 0) {
        nsq[s] = q.hi;
        err[s] = __fsqrt_ru(__fmul_ru(e2, 1.001f));
        nrm[s] = __fsqrt_ru(__fadd_ru(q.hi, q.lo));
    }
}

// TF32 form of k_bf16: the same rows rounded to TF32 (round to nearest,
// ties away; low 13 bits zero, so the tensor cores read them unchanged) in
// FP32 containers.  hv^2 is exact in FP32 (11-bit significands); the column
// term -||x~||^2/2 rides in columns 136/137 as a two-term TF32 split.
__device__ __forceinline__ float to_tf32(float x) {
    uint32_t r;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
    return __uint_as_float(r);
}

__global__ void k_tf32(const float* __restrict__ x32, const float* __restrict__ mu, uint64_t n, uint64_t npad,
                       float* __restrict__ ta, float* __restrict__ tb, float* __restrict__ nsq,
                       float* __restrict__ err, float* __restrict__ nrm) {
    uint64_t s = blockIdx.x * (uint64_t)(blockDim.x / 32) + (threadIdx.x >> 5);
    uint32_t lane = threadIdx.x & 31;
    if (s >= npad) return;
    float* rowa = ta + s * MDET_KPAD;
    float* rowb = tb + s * MDET_KPAD;
    if (s >= n) {
        for (int k = lane; k < MDET_KPAD; k += 32) {
            rowa[k] = (k == MDET_NTNF || k == MDET_NTNF + 1) ? 1.f : 0.f;
            rowb[k] = (k == MDET_NTNF) ? __int_as_float(0xff800000) : 0.f;
        }
        if (lane == 0) {
            nsq[s] = __int_as_float(0x7f800000);
            err[s] = 0.f;
            nrm[s] = 0.f;
        }
        return;
    }
    float e2 = 0.f;
    ff q = ff_make(0.f, 0.f);
    for (int k = lane; k < MDET_NTNF; k += 32) {
        const float a = x32[s * MDET_NTNF + k];
        const ff v = two_sum(a, -mu[k]);  // v.hi + v.lo == a - mu exactly
        const float hv = to_tf32(v.hi);
        const float d = __fadd_rn(__fsub_rn(v.hi, hv), v.lo);
        e2 = __fmaf_rn(d, d, e2);
        q = ff_add_f(q, __fmul_rn(hv, hv));
        rowa[k] = hv;
        rowb[k] = hv;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        e2 += __shfl_xor_sync(0xffffffffu, e2, o);
        ff t;
        t.hi = __shfl_xor_sync(0xffffffffu, q.hi, o);
        t.lo = __shfl_xor_sync(0xffffffffu, q.lo, o);
        q = ff_add(q, t);
    }
    const float half = 0.5f * q.hi;
    const float hi = to_tf32(half);
    const float lo = to_tf32(__fsub_rn(half, hi));
    for (int k = MDET_NTNF + lane; k < MDET_KPAD; k += 32) {
        rowa[k] = (k < MDET_NTNF + 2) ? 1.f : 0.f;
        rowb[k] = k == MDET_NTNF ? -hi : (k == MDET_NTNF + 1 ? -lo : 0.f);
    }
    if (lane == 0) {
        nsq[s] = q.hi;
        err[s] = __fsqrt_ru(__fmul_ru(e2, 1.001f));
        nrm[s] = __fsqrt_ru(__fadd_ru(q.hi, q.lo));
    }
}

__global__ void k_meta(const double* __restrict__ ls_s, const float* __restrict__ err, const float* __restrict__ nrm,
                       uint64_t n, uint64_t nblk, BlockMeta* __restrict__ meta, BlockMeta* __restrict__ meta32) {
    uint64_t b = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (b >= nblk) return;
    uint64_t s0 = b * MDET_BLK, s1 = min(n, s0 + MDET_BLK);
    BlockMeta m;
    if (s0 >= n) {
        m.lo = m.hi = (float)ls_s[n - 1];
        m.emax = m.nmax = 0.f;
    } else {
        // true range (the rows need not be in size order)
        double lo = ls_s[s0], hi = ls_s[s0];
        for (uint64_t s = s0 + 1; s < s1; ++s) {
            lo = fmin(lo, ls_s[s]);
            hi = fmax(hi, ls_s[s]);
        }
        m.lo = __double2float_rd(lo);
        m.hi = __double2float_ru(hi);
        float e = 0.f, nm = 0.f;
        if (err)
            for (uint64_t s = s0; s < s1; ++s) {
                e = fmaxf(e, err[s]);
                nm = fmaxf(nm, nrm[s]);
            }
        m.emax = e;
        m.nmax = nm;
    }
    if (meta) meta[b] = m;
    BlockMeta m32 = m;
    m32.emax = 0.f;
    m32.nmax = 0.f;
    meta32[b] = m32;
}

// ---- d* table ----

__device__ double dev_dstar(double x, double y, double L, const ModelSplit& ms) {
    const double ln9 = 2.1972245773362196;
    double t = x * y, c[4];
    for (int m = 0; m < 4; ++m) {
        double g[7] = {0, ms.G[m][1], ms.G[m][2], ms.G[m][3], ms.G[m][4], ms.G[m][5], ms.G[m][6]};
        double h[6] = {0, ms.H[m][1], ms.H[m][2], ms.H[m][3], ms.H[m][4], ms.H[m][5]};
        c[m] = poly(ms.F[m], 7, x) + poly(g, 6, y) + poly(h, 5, t);
    }
    const double inf = __longlong_as_double(0x7ff0000000000000ll);
    if (!(c[1] > 0)) return inf;
    if (L >= ln9) return (-L - c[0]) / c[1];
    if (!(c[3] > 0)) return inf;
    double d1 = (-ln9 - c[0]) / c[1];
    double d2 = (-L - c[2]) / c[3];
    return d1 > d2 ? d1 : d2;
}

constexpr int kPts = 4 * MDET_TBL + 1;

__global__ void k_dstar_points(double lmin, double h, double L, ModelSplit ms, float* __restrict__ pts) {
    int a = blockIdx.y, b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= kPts) return;
    int lo = min(a, b), hi = max(a, b);
    double x = lmin + lo * (h / 4), y = lmin + hi * (h / 4);
    double d = dev_dstar(x, y, L, ms);
    pts[a * kPts + b] = __double2float_ru(d);
}

// the same points on a grid held in device memory
__global__ void k_dstar_points_dev(const TableGrid* __restrict__ grid, double L, ModelSplit ms, float* __restrict__ pts) {
    int a = blockIdx.y, b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= kPts) return;
    int lo = min(a, b), hi = max(a, b);
    const double lmin = grid->lmin, h = grid->h;
    double x = lmin + lo * (h / 4), y = lmin + hi * (h / 4);
    double d = dev_dstar(x, y, L, ms);
    pts[a * kPts + b] = __double2float_ru(d);
}

// union of (lo, hi) ranges -> table grid (one thread)
__global__ void k_grid_from_ranges(const double* __restrict__ r, uint32_t count, TableGrid* __restrict__ g) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    double lo = INFINITY, hi = -INFINITY;
    for (uint32_t k = 0; k < count; ++k)
        if (r[2 * k] <= r[2 * k + 1]) {
            lo = fmin(lo, r[2 * k]);
            hi = fmax(hi, r[2 * k + 1]);
        }
    if (!(lo <= hi)) lo = hi = 0;
    double h = (hi - lo) / MDET_TBL;
    if (!(h > 1e-7)) h = 1e-7;
    lo -= 1e-9;
    g->lmin = lo;
    g->h = h;
    g->lminf = (float)lo;
    g->inv_hf = (float)(1.0 / h);
}

__global__ void k_dstar_cells(const float* __restrict__ pts, float* __restrict__ st0) {
    int a = blockIdx.x, b = threadIdx.x;
    float mx = -__int_as_float(0x7f800000), mn = __int_as_float(0x7f800000);
    for (int i = 0; i <= 4; ++i)
        for (int j = 0; j <= 4; ++j) {
            float v = pts[(4 * a + i) * kPts + (4 * b + j)];
            mx = fmaxf(mx, v);
            mn = fminf(mn, v);
        }
    float T = mx + 0.5f * (mx - mn) + 1e-6f + 1e-5f * fabsf(mx);
    if (isinf(mx) || isnan(mx)) T = __int_as_float(0x7f800000);
    st0[a * MDET_TBL + b] = T;
}

// Suffix maximum along x (the min-size axis): cell (a, b) then bounds every
// cell (a', b) with a' >= a, so a box [x0, x1] x [y0, y1] is bounded by row
// x0 alone.  d* falls as the smaller contig grows, so this costs little.
__global__ void k_suffix_x(float* __restrict__ st0) {
    const int b = threadIdx.x;
    float m = st0[(MDET_TBL - 1) * MDET_TBL + b];
    for (int a = MDET_TBL - 2; a >= 0; --a) {
        m = fmaxf(m, st0[a * MDET_TBL + b]);
        st0[a * MDET_TBL + b] = m;
    }
}

__global__ void k_sparse(float* __restrict__ st, int k) {
    int a = blockIdx.x, b = threadIdx.x;
    const float* prev = st + (size_t)(k - 1) * MDET_TBL * MDET_TBL;
    float* cur = st + (size_t)k * MDET_TBL * MDET_TBL;
    int b2 = min(b + (1 << (k - 1)), MDET_TBL - 1);
    cur[a * MDET_TBL + b] = fmaxf(prev[a * MDET_TBL + b], prev[a * MDET_TBL + b2]);
}

// Range of the log sizes: the end points when sorted, else a one-block scan.
__global__ void k_minmax(const double* __restrict__ ls_s, uint64_t n, int sorted, double* __restrict__ out) {
    if (sorted) {
        if (threadIdx.x == 0) {
            out[0] = ls_s[0];
            out[1] = ls_s[n - 1];
        }
        return;
    }
    __shared__ double smin[32], smax[32];
    double lo = INFINITY, hi = -INFINITY;
    for (uint64_t i = threadIdx.x; i < n; i += blockDim.x) {
        lo = fmin(lo, ls_s[i]);
        hi = fmax(hi, ls_s[i]);
    }
    for (int o = 16; o > 0; o >>= 1) {
        lo = fmin(lo, __shfl_xor_sync(0xffffffffu, lo, o));
        hi = fmax(hi, __shfl_xor_sync(0xffffffffu, hi, o));
    }
    if ((threadIdx.x & 31) == 0) {
        smin[threadIdx.x >> 5] = lo;
        smax[threadIdx.x >> 5] = hi;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 1; w < (int)(blockDim.x >> 5); ++w) {
            lo = fmin(lo, smin[w]);
            hi = fmax(hi, smax[w]);
        }
        out[0] = lo;
        out[1] = hi;
    }
}

}  // namespace

ModelHFF model_h_ff() {
    const ModelH h = model_h();
    ModelHFF r;
    for (int m = 0; m < 4; ++m)
        for (int k = 0; k < 6; ++k) {
            const float hi = (float)h.h[m][k];
            r.h[m][k].hi = hi;
            r.h[m][k].lo = (float)(h.h[m][k] - (double)hi);
        }
    return r;
}

ModelH model_h() {
    ModelH h;
    const ModelSplit& s = model_split();
    for (int m = 0; m < 4; ++m)
        for (int k = 0; k < 6; ++k) h.h[m][k] = s.H[m][k];
    return h;
}

int prep_alloc(mdet_ctx* ctx, const char* tag, uint64_t rows, int tck, GraphPrep* g) {
    const std::string t(tag);
    const uint64_t nblk = rows / MDET_BLK;
    g->perm = (uint32_t*)ctx_scratch(ctx, (t + ".perm").c_str(), rows * 4);
    g->inv = (uint32_t*)ctx_scratch(ctx, (t + ".inv").c_str(), rows * 4);
    g->x32 = (float*)ctx_scratch(ctx, (t + ".x32").c_str(), rows * MDET_NTNF * 4);
    g->ls = (double*)ctx_scratch(ctx, (t + ".ls").c_str(), rows * 8);
    g->parts = (PartsFF*)ctx_scratch(ctx, (t + ".parts").c_str(), rows * sizeof(PartsFF));
    g->meta32 = (BlockMeta*)ctx_scratch(ctx, (t + ".meta32").c_str(), nblk * sizeof(BlockMeta));
    g->mu = (float*)ctx_scratch(ctx, (t + ".mu").c_str(), MDET_NTNF * 4);
    g->xa = g->xb = nullptr;
    g->ta = g->tb = nullptr;
    g->tck = tck;
    g->nsq = nullptr;
    g->meta = nullptr;
    if (tck == kTcBf16) {
        g->xa = (uint16_t*)ctx_scratch(ctx, (t + ".xa").c_str(), rows * MDET_KPAD * 2);
        g->xb = (uint16_t*)ctx_scratch(ctx, (t + ".xb").c_str(), rows * MDET_KPAD * 2);
        if (!g->xa || !g->xb) return MDET_ERR_NOMEM;
    } else if (tck == kTcTf32) {
        g->ta = (float*)ctx_scratch(ctx, (t + ".ta").c_str(), rows * MDET_KPAD * 4);
        g->tb = (float*)ctx_scratch(ctx, (t + ".tb").c_str(), rows * MDET_KPAD * 4);
        if (!g->ta || !g->tb) return MDET_ERR_NOMEM;
    }
    if (tck != kTcNone) {
        g->nsq = (float*)ctx_scratch(ctx, (t + ".nsq").c_str(), rows * 4);
        g->meta = (BlockMeta*)ctx_scratch(ctx, (t + ".meta").c_str(), nblk * sizeof(BlockMeta));
        if (!g->nsq || !g->meta) return MDET_ERR_NOMEM;
    }
    if (!g->perm || !g->inv || !g->x32 || !g->ls || !g->parts || !g->meta32 || !g->mu) return MDET_ERR_NOMEM;
    return MDET_OK;
}

int prep_into(mdet_ctx* ctx, const float* d_tnf, const double* d_ls, uint64_t n, int tck, const GraphPrep& g,
              uint64_t base, const uint32_t* order) {
    cudaStream_t s = ctx->stream;
    const uint64_t npad = (n + 255) / 256 * 256;
    const uint64_t nblk = npad / MDET_BLK;
    unsigned long long* keys = (unsigned long long*)ctx_scratch(ctx, "pre.keys", n * 8);
    unsigned long long* keys2 = (unsigned long long*)ctx_scratch(ctx, "pre.keys2", n * 8);
    uint32_t* vals = (uint32_t*)ctx_scratch(ctx, "pre.vals", n * 4);
    double* sums = (double*)ctx_scratch(ctx, "pre.sums", MDET_NTNF * 8);
    if (!keys || !keys2 || !vals || !sums) return MDET_ERR_NOMEM;
    uint32_t* perm = g.perm + base;
    float* x32 = g.x32 + base * MDET_NTNF;
    double* ls = g.ls + base;
    PartsFF* parts = g.parts + base;
    const unsigned blocks = (unsigned)((n + 255) / 256);
    if (order) {
        // caller's order (original index per position)
        MDET_CUDA(ctx, cudaMemcpyAsync(perm, order, n * 4, cudaMemcpyDeviceToDevice, s));
    } else {
        k_keys<<<blocks, 256, 0, s>>>(d_ls, n, keys, vals);
        MDET_LAUNCHED(ctx, "k_keys");
        size_t tmpb = 0;
        cub::DeviceRadixSort::SortPairs(nullptr, tmpb, keys, keys2, vals, perm, (int)n, 0, 64, s);
        void* tmp = ctx_scratch(ctx, "pre.cubtmp", tmpb);
        if (!tmp) return MDET_ERR_NOMEM;
        MDET_CUDA(ctx, cub::DeviceRadixSort::SortPairs(tmp, tmpb, keys, keys2, vals, perm, (int)n, 0, 64, s));
    }
    k_gather<<<(unsigned)((npad + 7) / 8), 256, 0, s>>>(d_tnf, d_ls, perm, n, npad, (uint32_t)base, g.inv, x32, ls,
                                                       parts, model_split());
    MDET_LAUNCHED(ctx, "k_gather");
    float* err = nullptr;
    float* nrm = nullptr;
    if (tck != kTcNone) {
        err = (float*)ctx_scratch(ctx, "pre.err", npad * 4);
        nrm = (float*)ctx_scratch(ctx, "pre.nrm", npad * 4);
        if (!err || !nrm) return MDET_ERR_NOMEM;
        MDET_CUDA(ctx, cudaMemsetAsync(sums, 0, MDET_NTNF * 8, s));
        k_colsum<<<std::min<uint64_t>(1024, n), MDET_NTNF, 0, s>>>(x32, n, sums);
        MDET_LAUNCHED(ctx, "k_colsum");
        k_mean<<<1, MDET_NTNF, 0, s>>>(sums, n, g.mu);
        MDET_LAUNCHED(ctx, "k_mean");
        if (tck == kTcTf32) {
            k_tf32<<<(unsigned)((npad + 7) / 8), 256, 0, s>>>(x32, g.mu, n, npad, g.ta + base * MDET_KPAD,
                                                             g.tb + base * MDET_KPAD, g.nsq + base, err, nrm);
            MDET_LAUNCHED(ctx, "k_tf32");
        } else {
            k_bf16<<<(unsigned)((npad + 7) / 8), 256, 0, s>>>(x32, g.mu, n, npad, g.xa + base * MDET_KPAD,
                                                             g.xb + base * MDET_KPAD, g.nsq + base, err, nrm);
            MDET_LAUNCHED(ctx, "k_bf16");
        }
    }
    k_meta<<<(unsigned)((nblk + 127) / 128), 128, 0, s>>>(ls, err, nrm, n, nblk,
                                                         tck != kTcNone ? g.meta + base / MDET_BLK : nullptr,
                                                         g.meta32 + base / MDET_BLK);
    MDET_LAUNCHED(ctx, "k_meta");
    return MDET_OK;
}

// A 64-bit hash of the prepared inputs' contents (sum over the words of a
// splitmix64 finaliser of word and position), to recognise unchanged inputs.
__global__ void k_content_hash(const uint32_t* __restrict__ a, uint64_t na, const uint32_t* __restrict__ b,
                               uint64_t nb, unsigned long long* __restrict__ out) {
    unsigned long long h = 0;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < na + nb; i += stride) {
        unsigned long long z = (unsigned long long)(i < na ? a[i] : b[i - na]) + (i + 1) * 0x9E3779B97F4A7C15ull;
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        h += z ^ (z >> 31);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) h += __shfl_xor_sync(0xffffffffu, h, o);
    if ((threadIdx.x & 31) == 0) atomicAdd(out, h);
}

// Rows sorted by size (or in the caller's order).  A preparation of the very
// same inputs that is still in place (same pointers and contents, no count
// since) is used as it is: the search and the graph of one assembly share it.
int prep_sorted(mdet_ctx* ctx, const float* d_tnf, const double* d_ls, uint64_t n, int tck, GraphPrep* g,
                const uint32_t* order) {
    g->n = (uint32_t)n;
    g->npad = (uint32_t)((n + 255) / 256 * 256);
    MDET_TRY(prep_alloc(ctx, "pre", g->npad, tck, g));
    auto& c = ctx->prep_cache;
    if (order) {
        c.valid = false;
        return prep_into(ctx, d_tnf, d_ls, n, tck, *g, 0, order);
    }
    unsigned long long* dh = (unsigned long long*)ctx_scratch(ctx, "pre.hash", 8);
    if (!dh) return MDET_ERR_NOMEM;
    cudaStream_t s = ctx->stream;
    unsigned long long h = 0;
    MDET_CUDA(ctx, cudaMemsetAsync(dh, 0, 8, s));
    k_content_hash<<<ctx->num_sms * 8, 256, 0, s>>>((const uint32_t*)d_tnf, n * MDET_NTNF, (const uint32_t*)d_ls,
                                                    n * 2, dh);
    MDET_LAUNCHED(ctx, "k_content_hash");
    MDET_CUDA(ctx, cudaMemcpyAsync(&h, dh, 8, cudaMemcpyDeviceToHost, s));
    MDET_CUDA(ctx, cudaStreamSynchronize(s));
    // a preparation with other reduced-precision rows (or none) is remade:
    // nsq and the block metadata describe the rows last made
    if (c.valid && c.tnf == d_tnf && c.ls == d_ls && c.n == n && (c.tck == tck || tck == kTcNone) &&
        c.hash == h && c.x32 == g->x32 && (tck == kTcNone || (c.xa == g->xa && c.ta == g->ta)) &&
        c.gen == ctx->scratch_gen)
        return MDET_OK;
    c.valid = false;
    MDET_TRY(prep_into(ctx, d_tnf, d_ls, n, tck, *g, 0, nullptr));
    c.valid = true;
    c.tnf = d_tnf;
    c.ls = d_ls;
    c.n = n;
    c.tck = tck;
    c.hash = h;
    c.x32 = g->x32;
    c.xa = g->xa;
    c.ta = g->ta;
    c.gen = ctx->scratch_gen;
    return MDET_OK;
}

int build_dstar_table_at(mdet_ctx* ctx, double lmin, double lmax, double logit_cut, float* st, DstarTable* out) {
    cudaStream_t s = ctx->stream;
    out->dyn = nullptr;
    float* pts = (float*)ctx_scratch(ctx, "tbl.pts", (size_t)kPts * kPts * 4);
    if (!pts) return MDET_ERR_NOMEM;
    double h = (lmax - lmin) / MDET_TBL;
    if (!(h > 1e-7)) h = 1e-7;
    lmin -= 1e-9;
    dim3 grid((kPts + 127) / 128, kPts);
    k_dstar_points<<<grid, 128, 0, s>>>(lmin, h, logit_cut, model_split(), pts);
    MDET_LAUNCHED(ctx, "k_dstar_points");
    k_dstar_cells<<<MDET_TBL, MDET_TBL, 0, s>>>(pts, st);
    MDET_LAUNCHED(ctx, "k_dstar_cells");
    k_suffix_x<<<1, MDET_TBL, 0, s>>>(st);
    MDET_LAUNCHED(ctx, "k_suffix_x");
    for (int k = 1; k < MDET_TBL_LEVELS; ++k) {
        k_sparse<<<MDET_TBL, MDET_TBL, 0, s>>>(st, k);
        MDET_LAUNCHED(ctx, "k_sparse");
    }
    out->st = st;
    out->lmin = (float)lmin;
    out->inv_h = (float)(1.0 / h);
    return MDET_OK;
}

int grid_from_ranges(mdet_ctx* ctx, const double* ranges, uint32_t count, TableGrid* grid) {
    k_grid_from_ranges<<<1, 32, 0, ctx->stream>>>(ranges, count, grid);
    MDET_LAUNCHED(ctx, "k_grid_from_ranges");
    return MDET_OK;
}

int build_dstar_table_dev(mdet_ctx* ctx, const TableGrid* grid, double logit_cut, float* st, DstarTable* out) {
    cudaStream_t s = ctx->stream;
    float* pts = (float*)ctx_scratch(ctx, "tbl.pts", (size_t)kPts * kPts * 4);
    if (!pts) return MDET_ERR_NOMEM;
    dim3 g((kPts + 127) / 128, kPts);
    k_dstar_points_dev<<<g, 128, 0, s>>>(grid, logit_cut, model_split(), pts);
    MDET_LAUNCHED(ctx, "k_dstar_points");
    k_dstar_cells<<<MDET_TBL, MDET_TBL, 0, s>>>(pts, st);
    MDET_LAUNCHED(ctx, "k_dstar_cells");
    k_suffix_x<<<1, MDET_TBL, 0, s>>>(st);
    MDET_LAUNCHED(ctx, "k_suffix_x");
    for (int k = 1; k < MDET_TBL_LEVELS; ++k) {
        k_sparse<<<MDET_TBL, MDET_TBL, 0, s>>>(st, k);
        MDET_LAUNCHED(ctx, "k_sparse");
    }
    out->st = st;
    out->lmin = 0.f;
    out->inv_h = 0.f;
    out->dyn = &grid->lminf;
    return MDET_OK;
}

int build_dstar_table(mdet_ctx* ctx, const double* d_ls_sorted, uint64_t n, double logit_cut, DstarTable* out,
                      bool sorted, double* range) {
    out->dyn = nullptr;
    cudaStream_t s = ctx->stream;
    double lmin, lmax;
    if (range && !std::isnan(range[0])) {
        lmin = range[0];
        lmax = range[1];
    } else {
        // the range is needed on the host to place the grid
        double* mm = (double*)ctx_scratch(ctx, "tbl.mm", 16);
        if (!mm) return MDET_ERR_NOMEM;
        double r[2];
        k_minmax<<<1, sorted ? 32 : 1024, 0, s>>>(d_ls_sorted, n, sorted ? 1 : 0, mm);
        MDET_LAUNCHED(ctx, "k_minmax");
        MDET_CUDA(ctx, cudaMemcpyAsync(r, mm, 16, cudaMemcpyDeviceToHost, s));
        MDET_CUDA(ctx, cudaStreamSynchronize(s));
        lmin = r[0];
        lmax = r[1];
        if (range) {
            range[0] = lmin;
            range[1] = lmax;
        }
    }
    double h = (lmax - lmin) / MDET_TBL;
    if (!(h > 1e-7)) h = 1e-7;
    // a table already built for this cutoff and size range?
    int slot = -1, lru = 0;
    for (int k = 0; k < 4; ++k) {
        const auto& t = ctx->tbl[k];
        if (t.valid && t.L == logit_cut && t.lmin == lmin && t.lmax == lmax) slot = k;
        if (ctx->tbl[k].used < ctx->tbl[lru].used) lru = k;
    }
    const bool hit = slot >= 0;
    if (!hit) slot = lru;
    const std::string name = "tbl.st" + std::to_string(slot);
    float* st = (float*)ctx_scratch(ctx, name.c_str(), (size_t)MDET_TBL_LEVELS * MDET_TBL * MDET_TBL * 4);
    if (!st) return MDET_ERR_NOMEM;
    auto& t = ctx->tbl[slot];
    t.used = ++ctx->tbl_clock;
    out->st = st;
    out->lmin = (float)(lmin - 1e-9);
    out->inv_h = (float)(1.0 / h);
    if (hit) return MDET_OK;
    float* pts = (float*)ctx_scratch(ctx, "tbl.pts", (size_t)kPts * kPts * 4);
    if (!pts) return MDET_ERR_NOMEM;
    t.valid = false;
    dim3 grid((kPts + 127) / 128, kPts);
    k_dstar_points<<<grid, 128, 0, s>>>(lmin - 1e-9, h, logit_cut, model_split(), pts);
    MDET_LAUNCHED(ctx, "k_dstar_points");
    k_dstar_cells<<<MDET_TBL, MDET_TBL, 0, s>>>(pts, st);
    MDET_LAUNCHED(ctx, "k_dstar_cells");
    k_suffix_x<<<1, MDET_TBL, 0, s>>>(st);
    MDET_LAUNCHED(ctx, "k_suffix_x");
    for (int k = 1; k < MDET_TBL_LEVELS; ++k) {
        k_sparse<<<MDET_TBL, MDET_TBL, 0, s>>>(st, k);
        MDET_LAUNCHED(ctx, "k_sparse");
    }
    t.valid = true;
    t.L = logit_cut;
    t.lmin = lmin;
    t.lmax = lmax;
    return MDET_OK;
}
