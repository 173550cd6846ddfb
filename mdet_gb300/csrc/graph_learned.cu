// graph_learned.cu -- MDET_MODE_LEARNED: the TNF graph with the learned
// proposal.  The network embeds every contig (64 dims); contigs are ordered
// along a Morton curve over the leading principal axes of the embedding --
// either embedding-major (7 axes and the log size, then runs re-sorted by
// size) or size-major (size-sorted bands, 8 axes within a band) -- so that
// 128-row blocks gather similar contigs; each tile
// pair (128-row block I, 256-row block J) is kept when the triangle bound
// ||c_I - c_J|| - r_I - r_J on embedded distances is within the trained
// margin tau.  The kept tiles go through the same tensor-core filter and
// exact stage as the all-pairs form, so every emitted edge is exact; the only
// loss is recall, which is measured on a row sample against an all-columns
// pass before the graph is built, with the all-pairs form as the fallback.
// The reference has no learned component.
#include <cub/cub.cuh>
#include <thrust/iterator/counting_iterator.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "exact.cuh"
#include "mlp.cuh"

using namespace mdet_exact;

namespace {

constexpr int kPcs = 8;           // principal axes projected (the Morton key's dimensions)
constexpr int kFlagGroup = 8;     // row tiles per thread in the tile-flag kernel
constexpr uint32_t kBandRows = 16384;  // default band of the size-major order

// Morton key of one contig: 8 bits each of 8 coordinates, interleaved most
// significant bit first.  with_size: the 7 leading principal coordinates and
// the log size (which takes the lowest position of each bit level); else the
// 8 leading principal coordinates.
__global__ void k_morton(const float* __restrict__ proj, const double* __restrict__ ls, uint64_t n,
                         const float* __restrict__ off, const float* __restrict__ inv_span, float ls0, float ls_inv,
                         int with_size, unsigned long long* __restrict__ keys, uint32_t* __restrict__ vals) {
    const uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    uint32_t q[kPcs];
#pragma unroll
    for (int d = 0; d < kPcs; ++d) {
        const float u = (proj[i * kPcs + d] - off[d]) * inv_span[d];
        q[d] = (uint32_t)fminf(fmaxf(u * 256.f, 0.f), 255.f);
    }
    if (with_size) q[kPcs - 1] = (uint32_t)fminf(fmaxf(((float)ls[i] - ls0) * ls_inv * 256.f, 0.f), 255.f);
    unsigned long long key = 0;
#pragma unroll
    for (int b = 7; b >= 0; --b)
#pragma unroll
        for (int d = 0; d < kPcs; ++d) key = (key << 1) | ((q[d] >> b) & 1u);
    keys[i] = key;
    vals[i] = (uint32_t)i;
}

// size sort key: the log size's float bits (non-negative floats order as
// their bit patterns)
__global__ void k_size_keys(const double* __restrict__ ls, uint64_t n, unsigned long long* __restrict__ keys,
                            uint32_t* __restrict__ vals) {
    const uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    keys[i] = __float_as_uint(fmaxf((float)ls[i], 0.f));
    vals[i] = (uint32_t)i;
}

// size-major key: band of the size order (16 bits) above the top 48 bits of
// the embedding's Morton key
__global__ void k_band_keys(const uint32_t* __restrict__ by_size, const unsigned long long* __restrict__ morton,
                            uint64_t n, uint32_t band, unsigned long long* __restrict__ keys,
                            uint32_t* __restrict__ vals) {
    const uint64_t p = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (p >= n) return;
    const uint32_t o = by_size[p];
    keys[p] = ((unsigned long long)(p / band) << 48) | (morton[o] >> 16);
    vals[p] = o;
}

// Centroid and radius (in embedding space) of each block of `rows` prepared
// positions.  Centroids are written row-major [blk][64] or, for dim_major,
// [64][nblk] (the layout the tile-flag kernel reads coalesced).
__global__ void __launch_bounds__(256) k_block_stats(const float* __restrict__ z, const uint32_t* __restrict__ perm,
                                                     uint32_t n, uint32_t rows, uint32_t nblk, int dim_major,
                                                     float* __restrict__ cent, float* __restrict__ rad) {
    __shared__ float part[4][MLP_OUT];
    __shared__ float c[MLP_OUT];
    __shared__ float wmax[8];
    const uint32_t b = blockIdx.x;
    const uint32_t r0 = b * rows, r1 = min(n, r0 + rows);
    const uint32_t cnt = r1 > r0 ? r1 - r0 : 0;
    const uint32_t t = threadIdx.x, dim = t & 63, sub = t >> 6;
    float s = 0.f;
    for (uint32_t r = sub; r < cnt; r += 4) s += z[(uint64_t)perm[r0 + r] * MLP_OUT + dim];
    part[sub][dim] = s;
    __syncthreads();
    if (t < MLP_OUT) {
        const float v = cnt ? (part[0][t] + part[1][t] + part[2][t] + part[3][t]) / (float)cnt : 0.f;
        c[t] = v;
        if (dim_major)
            cent[(uint64_t)t * nblk + b] = v;
        else
            cent[(uint64_t)b * MLP_OUT + t] = v;
    }
    __syncthreads();
    float m = 0.f;
    for (uint32_t r = t; r < cnt; r += blockDim.x) {
        const float4* zr = reinterpret_cast<const float4*>(z + (uint64_t)perm[r0 + r] * MLP_OUT);
        float d2 = 0.f;
#pragma unroll
        for (int q = 0; q < MLP_OUT / 4; ++q) {
            const float4 v = zr[q];
            const float a = v.x - c[4 * q], bb = v.y - c[4 * q + 1], cc = v.z - c[4 * q + 2], dd = v.w - c[4 * q + 3];
            d2 += a * a + bb * bb + cc * cc + dd * dd;
        }
        m = fmaxf(m, d2);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((t & 31) == 0) wmax[t >> 5] = m;
    __syncthreads();
    if (t == 0) {
        float v = 0.f;
        for (int w = 0; w < 8; ++w) v = fmaxf(v, wmax[w]);
        // float rounding slack on the radius
        rad[b] = cnt ? sqrtf(v) * 1.0001f + 1e-5f : -INFINITY;
    }
}

// keep[I * tb + J] = tile pair (row tile I of 128, column tile J of 256) of
// the upper triangle has an embedded lower bound within tau.
__global__ void __launch_bounds__(256) k_tile_flags(const float* __restrict__ rc, const float* __restrict__ rr,
                                                    const float* __restrict__ cc_t, const float* __restrict__ cr,
                                                    uint32_t ta, uint32_t tb, float tau, uint8_t* __restrict__ keep) {
    __shared__ float ci[kFlagGroup][MLP_OUT];
    __shared__ float ri[kFlagGroup];
    const uint32_t I0 = blockIdx.y * kFlagGroup;
    for (uint32_t e = threadIdx.x; e < kFlagGroup * MLP_OUT; e += blockDim.x) {
        const uint32_t I = I0 + e / MLP_OUT;
        ci[e / MLP_OUT][e % MLP_OUT] = I < ta ? rc[(uint64_t)I * MLP_OUT + e % MLP_OUT] : 0.f;
    }
    if (threadIdx.x < kFlagGroup) ri[threadIdx.x] = I0 + threadIdx.x < ta ? rr[I0 + threadIdx.x] : -INFINITY;
    __syncthreads();
    const uint32_t J = blockIdx.x * blockDim.x + threadIdx.x;
    if (J >= tb) return;
    float cj[MLP_OUT];
#pragma unroll
    for (int d = 0; d < MLP_OUT; ++d) cj[d] = cc_t[(uint64_t)d * tb + J];
    const float rj = cr[J];
#pragma unroll 1
    for (int g = 0; g < kFlagGroup; ++g) {
        const uint32_t I = I0 + g;
        if (I >= ta) break;
        float d2 = 0.f;
#pragma unroll
        for (int d = 0; d < MLP_OUT; ++d) {
            const float a = ci[g][d] - cj[d];
            d2 = fmaf(a, a, d2);
        }
        const bool live = ri[g] > -INFINITY && rj > -INFINITY && J >= (I >> 1);
        keep[(uint64_t)I * tb + J] = (live && sqrtf(d2) - ri[g] - rj <= tau) ? 1 : 0;
    }
}

// Exact edges of the sampled rows (all-columns pass): edges of even sample
// slots give their embedded distance to the calibration set; edges of odd
// slots go to the validation set as (row, column) positions.
__global__ void __launch_bounds__(256) k_sample_edges(const uint2* __restrict__ cand, unsigned long long ncand,
                                                      const uint32_t* __restrict__ row_map,
                                                      const float* __restrict__ x32,
                                                      const PartsFF* __restrict__ parts, ModelHFF H, ff L, int model2,
                                                      const uint32_t* __restrict__ perm, const float* __restrict__ z,
                                                      float* __restrict__ cal, uint2* __restrict__ val,
                                                      unsigned long long* __restrict__ counts) {
    for (unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; i < ncand;
         i += (unsigned long long)gridDim.x * blockDim.x) {
        const uint2 c = cand[i];
        const uint32_t r = row_map[c.x], q = c.y;
        if (r == q) continue;
        const ff d = exact_dist(x32 + (uint64_t)r * MDET_NTNF, x32 + (uint64_t)q * MDET_NTNF);
        const ff pre = pre_prob(parts[r], parts[q], d, H, model2 != 0);
        if (!ff_gt(pre, L)) continue;
        if (c.x & 1) {
            val[atomicAdd(counts + 1, 1ull)] = make_uint2(min(r, q), max(r, q));
        } else {
            const float4* za = reinterpret_cast<const float4*>(z + (uint64_t)perm[r] * MLP_OUT);
            const float4* zb = reinterpret_cast<const float4*>(z + (uint64_t)perm[q] * MLP_OUT);
            float e2 = 0.f;
#pragma unroll
            for (int k = 0; k < MLP_OUT / 4; ++k) {
                const float4 u = za[k], v = zb[k];
                e2 += (u.x - v.x) * (u.x - v.x) + (u.y - v.y) * (u.y - v.y) + (u.z - v.z) * (u.z - v.z) +
                      (u.w - v.w) * (u.w - v.w);
            }
            cal[atomicAdd(counts, 1ull)] = sqrtf(e2);
        }
    }
}

// Validation edges whose tile pair is kept.
__global__ void k_recall(const uint2* __restrict__ val, unsigned long long nval, const uint8_t* __restrict__ keep,
                         uint32_t tb, unsigned long long* __restrict__ hit) {
    unsigned long long h = 0;
    for (unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; i < nval;
         i += (unsigned long long)gridDim.x * blockDim.x) {
        const uint2 e = val[i];
        h += keep[(uint64_t)(e.x / 128) * tb + e.y / 256];
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) h += __shfl_xor_sync(0xffffffffu, h, o);
    if ((threadIdx.x & 31) == 0 && h) atomicAdd(hit, h);
}

// Runs of `seg` positions of the embedding order, each re-sorted by log size
// (so that 128-row blocks have narrow size ranges).
__global__ void k_seg_keys(const uint32_t* __restrict__ order, const double* __restrict__ ls, uint64_t n, uint32_t seg,
                           unsigned long long* __restrict__ keys, uint32_t* __restrict__ vals) {
    const uint64_t p = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (p >= n) return;
    const uint32_t o = order[p];
    const float l = fmaxf((float)ls[o], 0.f);
    keys[p] = ((unsigned long long)(p / seg) << 32) | __float_as_uint(l);
    vals[p] = o;
}

// kept tiles per row tile (block per row tile), widened for the scan
__global__ void k_row_kept(const uint8_t* __restrict__ keep, uint32_t tb, unsigned long long* __restrict__ cnt) {
    __shared__ uint32_t part[8];
    const uint32_t I = blockIdx.x;
    uint32_t c = 0;
    for (uint32_t J = threadIdx.x; J < tb; J += blockDim.x) c += keep[(uint64_t)I * tb + J];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
    if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = c;
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t t = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += part[w];
        cnt[I] = t;
    }
}

__global__ void k_sample_rows(uint32_t n, uint32_t m, uint32_t* __restrict__ rows) {
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < m) rows[k] = (uint32_t)(((uint64_t)k * 2 + 1) * n / (2ull * m));
}

// Cyclic Jacobi eigen-decomposition of a symmetric k x k matrix (row-major,
// destroyed); eigenvalues in w, eigenvectors as columns of V.
void jacobi_eigen(std::vector<double>& A, int k, std::vector<double>& w, std::vector<double>& V) {
    V.assign((size_t)k * k, 0.0);
    for (int i = 0; i < k; ++i) V[(size_t)i * k + i] = 1.0;
    for (int sweep = 0; sweep < 64; ++sweep) {
        double off = 0;
        for (int p = 0; p < k; ++p)
            for (int q = p + 1; q < k; ++q) off += A[(size_t)p * k + q] * A[(size_t)p * k + q];
        if (off < 1e-22) break;
        for (int p = 0; p < k; ++p)
            for (int q = p + 1; q < k; ++q) {
                const double apq = A[(size_t)p * k + q];
                if (std::fabs(apq) < 1e-300) continue;
                const double theta = (A[(size_t)q * k + q] - A[(size_t)p * k + p]) / (2 * apq);
                const double t = (theta >= 0 ? 1.0 : -1.0) / (std::fabs(theta) + std::sqrt(theta * theta + 1));
                const double c = 1 / std::sqrt(t * t + 1), s = t * c;
                for (int r = 0; r < k; ++r) {  // A <- A J
                    const double arp = A[(size_t)r * k + p], arq = A[(size_t)r * k + q];
                    A[(size_t)r * k + p] = c * arp - s * arq;
                    A[(size_t)r * k + q] = s * arp + c * arq;
                }
                for (int r = 0; r < k; ++r) {  // A <- J^T A
                    const double apr = A[(size_t)p * k + r], aqr = A[(size_t)q * k + r];
                    A[(size_t)p * k + r] = c * apr - s * aqr;
                    A[(size_t)q * k + r] = s * apr + c * aqr;
                }
                for (int r = 0; r < k; ++r) {  // V <- V J
                    const double vrp = V[(size_t)r * k + p], vrq = V[(size_t)r * k + q];
                    V[(size_t)r * k + p] = c * vrp - s * vrq;
                    V[(size_t)r * k + q] = s * vrp + c * vrq;
                }
            }
    }
    w.resize(k);
    for (int i = 0; i < k; ++i) w[i] = A[(size_t)i * k + i];
}

struct PhaseClock {
    cudaEvent_t ev[8];
    int n = 0;
    cudaStream_t s;
    explicit PhaseClock(cudaStream_t st) : s(st) {
        for (auto& e : ev) cudaEventCreate(&e);
    }
    ~PhaseClock() {
        for (auto& e : ev) cudaEventDestroy(e);
    }
    void mark() {
        if (n < 8) cudaEventRecord(ev[n++], s);
    }
    double ms(int a, int b) {
        if (b >= n) return 0;
        float t = 0;
        cudaEventSynchronize(ev[b]);
        cudaEventElapsedTime(&t, ev[a], ev[b]);
        return t;
    }
};

// The order of the embedded contigs z (original index per position) in
// `order`: size_major 0 -- Morton over 7 principal axes and the log size,
// then runs of `seg` positions re-sorted by size (seg <= 1: none);
// size_major 1 -- size-sorted bands of `seg` contigs, Morton over 8 principal
// axes within each band.
int learned_order(mdet_ctx* ctx, const double* d_ls, uint64_t n, const float* z, int size_major, uint32_t seg,
                  const float* basis, uint32_t* order) {
    cudaStream_t s = ctx->stream;
    float* proj = (float*)ctx_scratch(ctx, "lrn.proj", n * kPcs * 4);
    unsigned long long* keys = (unsigned long long*)ctx_scratch(ctx, "lrn.keys", n * 8);
    unsigned long long* keys2 = (unsigned long long*)ctx_scratch(ctx, "lrn.keys2", n * 8);
    unsigned long long* keys3 = (unsigned long long*)ctx_scratch(ctx, "lrn.keys3", n * 8);
    uint32_t* vals = (uint32_t*)ctx_scratch(ctx, "lrn.vals", n * 4);
    if (!proj || !keys || !keys2 || !keys3 || !vals) return MDET_ERR_NOMEM;
    // the network's principal axes (kept from its training set), else this
    // assembly's
    if (!basis) {
        float* b = (float*)ctx_scratch(ctx, "lrn.basis", MLP_PCA_FLOATS * 4);
        if (!b) return MDET_ERR_NOMEM;
        MDET_TRY(mlp_pca_basis(ctx, z, n, b));
        basis = b;
    }
    const float* V = basis;
    const float* off = basis + MLP_OUT * kPcs;
    MDET_TRY(mlp_project(ctx, z, n, V, kPcs, proj));
    // log10 size over 3..7 (1 kb .. 10 Mb)
    const unsigned grid = (unsigned)((n + 255) / 256);
    k_morton<<<grid, 256, 0, s>>>(proj, d_ls, n, off, off + kPcs, 3.f, 0.25f, size_major ? 0 : 1, keys, vals);
    MDET_LAUNCHED(ctx, "k_morton");
    size_t tb = 0;
    cub::DeviceRadixSort::SortPairs(nullptr, tb, keys, keys2, vals, order, (int)n, 0, 64, s);
    void* tmp = ctx_scratch(ctx, "lrn.sorttmp", tb);
    if (!tmp) return MDET_ERR_NOMEM;
    if (size_major) {
        // the band index must fit 16 bits
        const uint32_t band = (uint32_t)std::max<uint64_t>(seg, n / 65535 + 1);
        k_size_keys<<<grid, 256, 0, s>>>(d_ls, n, keys3, vals);
        MDET_LAUNCHED(ctx, "k_size_keys");
        MDET_CUDA(ctx, cub::DeviceRadixSort::SortPairs(tmp, tb, keys3, keys2, vals, order, (int)n, 0, 32, s));
        k_band_keys<<<grid, 256, 0, s>>>(order, keys, n, band, keys3, vals);
        MDET_LAUNCHED(ctx, "k_band_keys");
        MDET_CUDA(ctx, cub::DeviceRadixSort::SortPairs(tmp, tb, keys3, keys2, vals, order, (int)n, 0, 64, s));
        return MDET_OK;
    }
    MDET_CUDA(ctx, cub::DeviceRadixSort::SortPairs(tmp, tb, keys, keys2, vals, order, (int)n, 0, 64, s));
    if (seg > 1) {
        k_seg_keys<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(order, d_ls, n, seg, keys, vals);
        MDET_LAUNCHED(ctx, "k_seg_keys");
        MDET_CUDA(ctx, cub::DeviceRadixSort::SortPairs(tmp, tb, keys, keys2, vals, order, (int)n, 0, 64, s));
    }
    return MDET_OK;
}

}  // namespace

// Principal axes of the embeddings z (n x 64) for the Morton key: basis =
// V (64 x 8, the eigenvectors of the 8 largest eigenvalues of the
// covariance), then the key's offsets (mean - 3 sd) and inverse spans
// (1 / 6 sd) along them.
int mlp_pca_basis(mdet_ctx* ctx, const float* z, uint64_t n, float* basis) {
    cudaStream_t s = ctx->stream;
    float* G = (float*)ctx_scratch(ctx, "lrn.gram", MLP_OUT * MLP_OUT * 4);
    float* colsum = (float*)ctx_scratch(ctx, "lrn.colsum", MLP_OUT * 4);
    if (!G || !colsum) return MDET_ERR_NOMEM;
    MDET_CUDA(ctx, cudaMemsetAsync(G, 0, MLP_OUT * MLP_OUT * 4, s));
    MDET_CUDA(ctx, cudaMemsetAsync(colsum, 0, MLP_OUT * 4, s));
    MDET_TRY(mlp_gram(ctx, z, n, G));
    MDET_TRY(mlp_colsum(ctx, z, n, colsum));
    std::vector<float> hg(MLP_OUT * MLP_OUT), hs(MLP_OUT);
    MDET_CUDA(ctx, cudaMemcpyAsync(hg.data(), G, hg.size() * 4, cudaMemcpyDeviceToHost, s));
    MDET_CUDA(ctx, cudaMemcpyAsync(hs.data(), colsum, hs.size() * 4, cudaMemcpyDeviceToHost, s));
    MDET_CUDA(ctx, cudaStreamSynchronize(s));
    std::vector<double> C((size_t)MLP_OUT * MLP_OUT), w, E;
    for (int i = 0; i < MLP_OUT; ++i)
        for (int j = 0; j < MLP_OUT; ++j)
            C[(size_t)i * MLP_OUT + j] = (double)hg[(size_t)i * MLP_OUT + j] / (double)n -
                                         ((double)hs[i] / (double)n) * ((double)hs[j] / (double)n);
    jacobi_eigen(C, MLP_OUT, w, E);
    std::vector<int> idx(MLP_OUT);
    for (int i = 0; i < MLP_OUT; ++i) idx[i] = i;
    std::sort(idx.begin(), idx.end(), [&](int a, int b) { return w[a] > w[b]; });
    std::vector<float> h(MLP_PCA_FLOATS);
    float* hv = h.data();
    float* hoff = h.data() + MLP_OUT * kPcs;
    for (int p = 0; p < kPcs; ++p) {
        const int e = idx[p];
        double mproj = 0;
        for (int r = 0; r < MLP_OUT; ++r) {
            hv[(size_t)r * kPcs + p] = (float)E[(size_t)r * MLP_OUT + e];
            mproj += E[(size_t)r * MLP_OUT + e] * (double)hs[r] / (double)n;
        }
        const double sd = std::sqrt(std::max(w[e], 1e-20));
        hoff[p] = (float)(mproj - 3.0 * sd);            // the key spans mean +- 3 sd
        hoff[kPcs + p] = (float)(1.0 / (6.0 * sd));
    }
    MDET_CUDA(ctx, cudaMemcpyAsync(basis, h.data(), h.size() * 4, cudaMemcpyHostToDevice, s));
    MDET_CUDA(ctx, cudaStreamSynchronize(s));  // h is a local
    return MDET_OK;
}

int graph_learned(mdet_ctx* ctx, const float* d_tnf, const double* d_ls, uint64_t n, double cutoff, uint32_t max_edges,
                  mdet_graph_stats* st, GraphPrep& g, uint64_t* total) {
    cudaStream_t s = ctx->stream;
    const mdet_mlp* net = ctx->mlp;
    mdet_learned_report* rep = ctx->learned_report;
    const double target = rep && rep->recall_target > 0 ? rep->recall_target : 0.999;
    const uint32_t want_rows = rep && rep->recall_rows ? rep->recall_rows : 2048;
    const int size_major = rep && rep->order == 1 ? 1 : 0;
    const uint32_t seg = rep && rep->segment ? rep->segment : (size_major ? kBandRows : 1024);
    if (rep) {
        rep->recall = 0;
        rep->fell_back = 0;
        rep->tiles_skipped = 0;
        rep->tau = 0;
        rep->ms_embed = rep->ms_order = rep->ms_sample = 0;
    }
    float tau_net = INFINITY;
    MDET_CUDA(ctx, cudaMemcpyAsync(&tau_net, net->params + MLP_TAU, 4, cudaMemcpyDeviceToHost, s));
    MDET_CUDA(ctx, cudaStreamSynchronize(s));
    const uint32_t ta = (uint32_t)((n + 127) / 128), tb = (uint32_t)((n + 255) / 256);
    const uint64_t full = [&] {
        uint64_t t = (uint64_t)ta * tb;
        const uint64_t m = ta >> 1;
        return t - ((ta & 1) ? m * m : (m ? m * (m - 1) : 0));
    }();
    auto fallback = [&](double recall, double tau) -> int {
        if (rep) {
            rep->recall = recall;
            rep->fell_back = 1;
            rep->tiles_skipped = 0;
            rep->tau = tau;
        }
        return graph_core(ctx, d_tnf, d_ls, n, cutoff, max_edges, MDET_MODE_BF16, st, g, total);
    };
    if (n < 2048 || (uint64_t)ta * tb >= (1ull << 31)) return fallback(0.0, 0.0);

    PhaseClock tm(s);
    tm.mark();
    float* z = (float*)ctx_scratch(ctx, "lrn.z", n * MLP_OUT * 4);
    uint32_t* order = (uint32_t*)ctx_scratch(ctx, "lrn.order", n * 4);
    if (!z || !order) return MDET_ERR_NOMEM;
    MDET_TRY(mlp_embed(ctx, net->params, d_tnf, n, z));
    tm.mark();
    MDET_TRY(learned_order(ctx, d_ls, n, z, size_major, seg, net->pca_valid ? net->pca : nullptr, order));
    MDET_TRY(prep_sorted(ctx, d_tnf, d_ls, n, true, &g, order));
    MDET_TRY(abd_gate(ctx, g));
    const double L = logit(cutoff);
    DstarTable tbl;
    MDET_TRY(build_dstar_table(ctx, g.ls, n, L, &tbl, false));
    tm.mark();

    // block statistics in embedding space
    float* rcent = (float*)ctx_scratch(ctx, "lrn.rcent", (uint64_t)ta * MLP_OUT * 4);
    float* rrad = (float*)ctx_scratch(ctx, "lrn.rrad", (uint64_t)ta * 4);
    float* ccent = (float*)ctx_scratch(ctx, "lrn.ccent", (uint64_t)tb * MLP_OUT * 4);
    float* crad = (float*)ctx_scratch(ctx, "lrn.crad", (uint64_t)tb * 4);
    uint8_t* keep = (uint8_t*)ctx_scratch(ctx, "lrn.keep", (uint64_t)ta * tb);
    uint32_t* list = (uint32_t*)ctx_scratch(ctx, "lrn.list", (uint64_t)ta * tb * 4);
    int* nsel = (int*)ctx_scratch(ctx, "lrn.nsel", 8);
    if (!rcent || !rrad || !ccent || !crad || !keep || !list || !nsel) return MDET_ERR_NOMEM;
    k_block_stats<<<ta, 256, 0, s>>>(z, g.perm, (uint32_t)n, 128, ta, 0, rcent, rrad);
    MDET_LAUNCHED(ctx, "k_block_stats");
    k_block_stats<<<tb, 256, 0, s>>>(z, g.perm, (uint32_t)n, 256, tb, 1, ccent, crad);
    MDET_LAUNCHED(ctx, "k_block_stats");

    // sampled rows against all columns, scored exactly: calibration and
    // validation edges
    const uint32_t m = (uint32_t)std::min<uint64_t>(n, want_rows);
    uint32_t* rows = (uint32_t*)ctx_scratch(ctx, "lrn.rows", (uint64_t)m * 4);
    unsigned long long* counts = (unsigned long long*)ctx_scratch(ctx, "lrn.counts", 32);
    if (!rows || !counts) return MDET_ERR_NOMEM;
    k_sample_rows<<<(m + 255) / 256, 256, 0, s>>>((uint32_t)n, m, rows);
    MDET_LAUNCHED(ctx, "k_sample_rows");
    RowSet rs;
    MDET_TRY(gather_rows_bf16(ctx, g, rows, m, "lrn.s", &rs));
    uint2* rc = nullptr;
    unsigned long long nrc = 0;
    MDET_TRY(run_filter(ctx, MDET_MODE_BF16, g, true, nullptr, rs.ab, rs.ansq, m, rs.meta, nullptr, tbl, "lrn.rc", &rc,
                        &nrc));
    float* cal = (float*)ctx_scratch(ctx, "lrn.cal", (nrc + 1) * 4);
    float* cal2 = (float*)ctx_scratch(ctx, "lrn.cal2", (nrc + 1) * 4);
    uint2* val = (uint2*)ctx_scratch(ctx, "lrn.val", (nrc + 1) * sizeof(uint2));
    if (!cal || !cal2 || !val) return MDET_ERR_NOMEM;
    MDET_CUDA(ctx, cudaMemsetAsync(counts, 0, 32, s));
    if (nrc) {
        const uint64_t blocks = std::min<uint64_t>((nrc + 255) / 256, (uint64_t)ctx->num_sms * 8);
        ff Lff;
        Lff.hi = (float)L;
        Lff.lo = (float)(L - (double)Lff.hi);
        k_sample_edges<<<(unsigned)blocks, 256, 0, s>>>(rc, nrc, rows, g.x32, g.parts, model_h_ff(), Lff,
                                                         L < kLn9 ? 1 : 0, g.perm, z, cal, val, counts);
        MDET_LAUNCHED(ctx, "k_sample_edges");
    }
    unsigned long long hc[2] = {0, 0};
    MDET_CUDA(ctx, cudaMemcpyAsync(hc, counts, 16, cudaMemcpyDeviceToHost, s));
    MDET_CUDA(ctx, cudaStreamSynchronize(s));
    MDET_TRY(check_flag(ctx));
    // tau: an upper quantile of the calibration edges' embedded distances
    // (the network's own margin when the sample holds too few edges)
    float tau = tau_net;
    const unsigned long long ncal = hc[0], nval = hc[1];
    if (ncal >= 256) {
        size_t tmpb = 0;
        cub::DeviceRadixSort::SortKeys(nullptr, tmpb, cal, cal2, (int)ncal, 0, 32, s);
        void* tmp = ctx_scratch(ctx, "lrn.caltmp", tmpb);
        if (!tmp) return MDET_ERR_NOMEM;
        MDET_CUDA(ctx, cub::DeviceRadixSort::SortKeys(tmp, tmpb, cal, cal2, (int)ncal, 0, 32, s));
        const double q = rep && rep->tau_quantile > 0 && rep->tau_quantile < 1 ? rep->tau_quantile
                                                                              : 1.0 - (1.0 - target) / 4.0;
        const uint64_t qi = std::min<uint64_t>(ncal - 1, (uint64_t)std::ceil(q * (double)(ncal - 1)));
        float hq = 0;
        MDET_CUDA(ctx, cudaMemcpyAsync(&hq, cal2 + qi, 4, cudaMemcpyDeviceToHost, s));
        MDET_CUDA(ctx, cudaStreamSynchronize(s));
        tau = hq * 1.02f + 1e-4f;
    }
    if (!(tau < INFINITY)) return fallback(0.0, 0.0);

    // kept tiles and their list
    k_tile_flags<<<dim3((tb + 255) / 256, (ta + kFlagGroup - 1) / kFlagGroup), 256, 0, s>>>(rcent, rrad, ccent, crad,
                                                                                           ta, tb, tau, keep);
    MDET_LAUNCHED(ctx, "k_tile_flags");
    {
        size_t tmpb = 0;
        thrust::counting_iterator<uint32_t> it(0);
        cub::DeviceSelect::Flagged(nullptr, tmpb, it, keep, list, nsel, (int)((uint64_t)ta * tb), s);
        void* tmp = ctx_scratch(ctx, "lrn.seltmp", tmpb);
        if (!tmp) return MDET_ERR_NOMEM;
        MDET_CUDA(ctx, cub::DeviceSelect::Flagged(tmp, tmpb, it, keep, list, nsel, (int)((uint64_t)ta * tb), s));
    }
    if (nval) {
        const uint64_t blocks = std::min<uint64_t>((nval + 255) / 256, (uint64_t)ctx->num_sms * 8);
        k_recall<<<(unsigned)blocks, 256, 0, s>>>(val, nval, keep, tb, counts + 2);
        MDET_LAUNCHED(ctx, "k_recall");
    }
    int hsel = 0;
    unsigned long long hhit = 0;
    MDET_CUDA(ctx, cudaMemcpyAsync(&hsel, nsel, 4, cudaMemcpyDeviceToHost, s));
    MDET_CUDA(ctx, cudaMemcpyAsync(&hhit, counts + 2, 8, cudaMemcpyDeviceToHost, s));
    MDET_CUDA(ctx, cudaStreamSynchronize(s));
    const double recall = nval ? (double)hhit / (double)nval : 1.0;
    if (recall < target) return fallback(recall, tau);
    tm.mark();

    // list entries per row tile, so the filter takes row tiles in waves
    unsigned long long* rowcnt = (unsigned long long*)ctx_scratch(ctx, "lrn.rowcnt", ((uint64_t)ta + 1) * 8);
    unsigned long long* rowoff = (unsigned long long*)ctx_scratch(ctx, "lrn.rowoff", ((uint64_t)ta + 1) * 8);
    if (!rowcnt || !rowoff) return MDET_ERR_NOMEM;
    MDET_CUDA(ctx, cudaMemsetAsync(rowcnt + ta, 0, 8, s));
    k_row_kept<<<ta, 256, 0, s>>>(keep, tb, rowcnt);
    MDET_LAUNCHED(ctx, "k_row_kept");
    {
        size_t tmpb = 0;
        cub::DeviceScan::ExclusiveSum(nullptr, tmpb, rowcnt, rowoff, (int)ta + 1, s);
        void* tmp = ctx_scratch(ctx, "lrn.scantmp", tmpb);
        if (!tmp) return MDET_ERR_NOMEM;
        MDET_CUDA(ctx, cub::DeviceScan::ExclusiveSum(tmp, tmpb, rowcnt, rowoff, (int)ta + 1, s));
    }
    uint2* cand = nullptr;
    unsigned long long ncand = 0;
    if (hsel > 0)
        MDET_TRY(run_filter(ctx, MDET_MODE_BF16, g, false, nullptr, nullptr, nullptr, 0, nullptr, nullptr, tbl, "g",
                            &cand, &ncand, list, (uint64_t)hsel, nullptr, 0, 256, 0, nullptr, rowoff));
    tm.mark();
    Edge* edges = nullptr;
    unsigned long long ne = 0;
    uint32_t* deg = nullptr;
    MDET_TRY(exact_graph(ctx, g, cand, ncand, L, &edges, &ne, &deg));
    tm.mark();
    MDET_TRY(select_topk(ctx, g, edges, ne, deg, max_edges, total));
    tm.mark();
    if (st) {
        st->n_candidates = ncand;
        st->n_above_cutoff = ne;
        st->tiles_total = full;
        st->tiles_computed = (uint64_t)hsel;
        st->ms_prep = tm.ms(0, 3);
        st->ms_filter = tm.ms(3, 4);
        st->ms_exact = tm.ms(4, 5);
        st->ms_select = tm.ms(5, 6);
    }
    if (rep) {
        rep->recall = recall;
        rep->fell_back = 0;
        rep->tiles_skipped = full - (uint64_t)hsel;
        rep->tau = tau;
        rep->ms_embed = tm.ms(0, 1);
        rep->ms_order = tm.ms(1, 2);
        rep->ms_sample = tm.ms(2, 3);
    }
    return MDET_OK;
}
