// learned.cu -- the learned proposal's network: the pair loss, Adam, pair
// labelling with the exact probability kernel, the training loop and the C
// ABI of the network (mdet_mlp_*).  The GEMMs of inference and training run
// on the tensor cores (mlp_tc.cu); the SIMT GEMMs below serve the principal
// axes of the embedding (Gram matrix, projection).  The
// reference has no learned component; everything here is this project's.
#include <cub/cub.cuh>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "exact.cuh"
#include "mlp.cuh"

using namespace mdet_exact;

namespace {

// C[M x N] = op(A) * op(B) with op(A)(m,k) = TA ? A[k*lda+m] : A[m*lda+k] and
// op(B)(k,n) = TB ? B[n*ldb+k] : B[k*ldb+n] (FP32, SIMT): the principal axes
// of the embedding.  MODE 0: C = acc; MODE 2: atomicAdd into C over a K
// slice (blockIdx.z).
template <bool TA, bool TB, int MODE>
__global__ void __launch_bounds__(256) k_gemm(int M, int N, int K, const float* __restrict__ A, int lda,
                                              const float* __restrict__ B, int ldb, float* __restrict__ C, int ldc,
                                              int kslice) {
    __shared__ float As[16][64 + 4];
    __shared__ float Bs[16][64 + 4];
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    const int m0 = blockIdx.y * 64, n0 = blockIdx.x * 64;
    int kbeg = 0, kend = K;
    if (MODE == 2) {
        kbeg = blockIdx.z * kslice;
        kend = min(K, kbeg + kslice);
    }
    float acc[4][4];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = 0.f;
    for (int k0 = kbeg; k0 < kend; k0 += 16) {
#pragma unroll
        for (int t = 0; t < 4; ++t) {
            const int e = threadIdx.x + t * 256;  // 0..1023
            // A tile: 64 (m) x 16 (k)
            const int am = TA ? (e & 63) : (e >> 4), ak = TA ? (e >> 6) : (e & 15);
            const int gm = m0 + am, gk = k0 + ak;
            float av = 0.f;
            if (gm < M && gk < kend) av = TA ? A[(size_t)gk * lda + gm] : A[(size_t)gm * lda + gk];
            As[ak][am] = av;
            // B tile: 16 (k) x 64 (n)
            const int bk = TB ? (e & 15) : (e >> 6), bn = TB ? (e >> 4) : (e & 63);
            const int gk2 = k0 + bk, gn = n0 + bn;
            float bv = 0.f;
            if (gn < N && gk2 < kend) bv = TB ? B[(size_t)gn * ldb + gk2] : B[(size_t)gk2 * ldb + gn];
            Bs[bk][bn] = bv;
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < 16; ++kk) {
            float a[4], b[4];
#pragma unroll
            for (int i = 0; i < 4; ++i) a[i] = As[kk][ty * 4 + i];
#pragma unroll
            for (int j = 0; j < 4; ++j) b[j] = Bs[kk][tx * 4 + j];
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j) acc[i][j] = fmaf(a[i], b[j], acc[i][j]);
        }
        __syncthreads();
    }
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const int gm = m0 + ty * 4 + i;
        if (gm >= M) continue;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const int gn = n0 + tx * 4 + j;
            if (gn >= N) continue;
            const float v = acc[i][j];
            if (MODE == 2)
                atomicAdd(&C[(size_t)gm * ldc + gn], v);
            else
                C[(size_t)gm * ldc + gn] = v;
        }
    }
}

template <bool TA, bool TB, int MODE>
int gemm(mdet_ctx* ctx, int M, int N, int K, const float* A, int lda, const float* B, int ldb, float* C, int ldc) {
    if (M <= 0 || N <= 0 || K <= 0) return MDET_OK;
    dim3 grid((N + 63) / 64, (M + 63) / 64, 1);
    int kslice = K;
    if (MODE == 2) {
        // split the reduction so that every SM has work
        int tiles = (int)(grid.x * grid.y);
        int slices = std::max(1, std::min((K + 255) / 256, (ctx->num_sms * 4 + tiles - 1) / tiles));
        kslice = ((K + slices - 1) / slices + 15) / 16 * 16;
        grid.z = (K + kslice - 1) / kslice;
    }
    k_gemm<TA, TB, MODE><<<grid, 256, 0, ctx->stream>>>(M, N, K, A, lda, B, ldb, C, ldc, kslice);
    MDET_LAUNCHED(ctx, "k_gemm");
    return MDET_OK;
}

// column sums of dZ [rows][cols] added into grad (bias gradients)
__global__ void k_colsum_add(const float* __restrict__ dz, uint64_t rows, int cols, float* __restrict__ g) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= cols) return;
    const uint64_t r0 = blockIdx.y * 256ull, r1 = min(rows, r0 + 256);
    float s = 0.f;
    for (uint64_t r = r0; r < r1; ++r) s += dz[r * cols + c];
    atomicAdd(&g[c], s);
}

// Contrastive loss on embedded distance e = ||z_a - z_b||: label 1 pulls
// below m_pos, label 0 pushes beyond m_neg; mean over pairs.
__global__ void k_pair_loss(const float* __restrict__ z, uint64_t np, const float* __restrict__ labels, float m_pos,
                            float m_neg, float* __restrict__ dz, double* __restrict__ loss) {
    const uint64_t p = blockIdx.x * (uint64_t)(blockDim.x / 32) + (threadIdx.x >> 5);
    const uint32_t lane = threadIdx.x & 31;
    if (p >= np) return;
    const float* za = z + p * MLP_OUT;
    const float* zb = z + (np + p) * MLP_OUT;
    const float d0 = za[lane] - zb[lane], d1 = za[lane + 32] - zb[lane + 32];
    float s = d0 * d0 + d1 * d1;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    const float e = sqrtf(s);
    const float y = labels[p];
    const float up = fmaxf(e - m_pos, 0.f), dn = fmaxf(m_neg - e, 0.f);
    const float l = y * up * up + (1.f - y) * dn * dn;
    const float dl = (2.f * y * up - 2.f * (1.f - y) * dn) / (float)np;
    const float f = e > 1e-12f ? dl / e : 0.f;
    dz[p * MLP_OUT + lane] = f * d0;
    dz[p * MLP_OUT + lane + 32] = f * d1;
    dz[(np + p) * MLP_OUT + lane] = -f * d0;
    dz[(np + p) * MLP_OUT + lane + 32] = -f * d1;
    if (lane == 0) atomicAdd(loss, (double)l);
}

__global__ void k_adam(float* __restrict__ w, float* __restrict__ m, float* __restrict__ v, const float* __restrict__ g,
                       uint32_t count, float lr, float b1, float b2, float eps, float c1, float c2) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    w[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
}

// exact label of sorted-position pairs: 1 when pre-probability beats L
__global__ void k_label_pairs(const uint2* __restrict__ pairs, uint64_t np, const float* __restrict__ x32,
                              const PartsFF* __restrict__ parts, ModelHFF H, ff L, float* __restrict__ labels) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < np; i += (uint64_t)gridDim.x * blockDim.x) {
        const uint2 c = pairs[i];
        const ff d = exact_dist(x32 + (uint64_t)c.x * MDET_NTNF, x32 + (uint64_t)c.y * MDET_NTNF);
        const ff pre = pre_prob(parts[c.x], parts[c.y], d, H, true);
        labels[i] = ff_gt(pre, L) ? 1.f : 0.f;
    }
}

__device__ __forceinline__ uint64_t mix64(uint64_t z) {
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

// Pair pool: each entry is, with probability frac, a candidate pair of the
// distance filter drawn at random, else a uniformly random pair (i != j).
__global__ void k_pair_pool(uint64_t seed, uint64_t count, uint32_t n, const uint2* __restrict__ cand, uint64_t ncand,
                            double frac, uint2* __restrict__ out) {
    const uint64_t thr = (uint64_t)(frac * 4294967296.0);
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < count; i += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t r = mix64(seed + 0x9E3779B97F4A7C15ull * (i + 1));
        const uint64_t r2 = mix64(r ^ 0x632BE59BD9B4E019ull);
        if (ncand && (r2 & 0xFFFFFFFFull) < thr) {
            out[i] = cand[(uint64_t)(((r2 >> 32) * ncand) >> 32)];
            continue;
        }
        uint32_t a = (uint32_t)(((r & 0xFFFFFFFFull) * n) >> 32);
        uint32_t b = (uint32_t)(((r >> 32) * (uint64_t)(n - 1)) >> 32);
        if (b >= a) ++b;
        out[i] = make_uint2(a, b);
    }
}

// batch gather: rows [0,B) first endpoints, [B,2B) second endpoints, labels
__global__ void k_batch(const uint2* __restrict__ pairs, const float* __restrict__ labels, uint64_t npairs,
                        uint64_t seed, uint32_t B, uint32_t* __restrict__ idx, float* __restrict__ blab) {
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= B) return;
    const uint64_t r = mix64(seed + 0xD1B54A32D192ED03ull * (t + 1));
    const uint64_t k = (uint64_t)(((r >> 16) * (npairs)) >> 48);
    const uint2 pr = pairs[k < npairs ? k : npairs - 1];
    idx[t] = pr.x;
    idx[B + t] = pr.y;
    blab[t] = labels[k < npairs ? k : npairs - 1];
}

__global__ void k_pair_dist(const float* __restrict__ z, uint64_t np, float* __restrict__ e) {
    const uint64_t p = blockIdx.x * (uint64_t)(blockDim.x / 32) + (threadIdx.x >> 5);
    const uint32_t lane = threadIdx.x & 31;
    if (p >= np) return;
    const float* za = z + p * MLP_OUT;
    const float* zb = z + (np + p) * MLP_OUT;
    const float d0 = za[lane] - zb[lane], d1 = za[lane + 32] - zb[lane + 32];
    float s = d0 * d0 + d1 * d1;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == 0) e[p] = sqrtf(s);
}

// deterministic host initialisation: He-normal weights, zero biases
void host_init(uint64_t seed, std::vector<float>& p) {
    p.assign(MLP_NPARAM, 0.f);
    uint64_t s = seed * 0x9E3779B97F4A7C15ull + 12345;
    auto next = [&]() {
        s += 0x9E3779B97F4A7C15ull;
        uint64_t z = s;
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        return z ^ (z >> 31);
    };
    auto normal = [&]() {
        double u1 = ((next() >> 11) + 1.0) / 9007199254740993.0, u2 = (next() >> 11) / 9007199254740992.0;
        return std::sqrt(-2.0 * std::log(u1)) * std::cos(6.283185307179586 * u2);
    };
    const int fan[3] = {MLP_IN, MLP_H1, MLP_H2}, outs[3] = {MLP_H1, MLP_H2, MLP_OUT};
    const int off[3] = {MLP_W1, MLP_W2, MLP_W3};
    for (int l = 0; l < 3; ++l) {
        const double sd = std::sqrt(2.0 / fan[l]);
        for (int i = 0; i < outs[l] * fan[l]; ++i) p[off[l] + i] = (float)(sd * normal());
    }
    p[MLP_SCALE] = 1.f;
    p[MLP_TAU] = INFINITY;
}

}  // namespace

// ------------------------------------------------------------ host side --

int mlp_embed(mdet_ctx* ctx, const float* P, const float* tnf, uint64_t n, float* z) {
    return mlp_embed_tc(ctx, P, tnf, n, z, nullptr);
}

int mlp_pair_loss(mdet_ctx* ctx, const float* z, uint64_t np, const float* labels, float m_pos, float m_neg,
                  float* dz, double* loss_sum) {
    if (np == 0) return MDET_OK;
    k_pair_loss<<<(unsigned)((np + 7) / 8), 256, 0, ctx->stream>>>(z, np, labels, m_pos, m_neg, dz, loss_sum);
    MDET_LAUNCHED(ctx, "k_pair_loss");
    return MDET_OK;
}

int mlp_gram(mdet_ctx* ctx, const float* z, uint64_t n, float* G) {
    return gemm<true, false, 2>(ctx, MLP_OUT, MLP_OUT, (int)n, z, MLP_OUT, z, MLP_OUT, G, MLP_OUT);
}

int mlp_colsum(mdet_ctx* ctx, const float* z, uint64_t n, float* sum) {
    if (n == 0) return MDET_OK;
    k_colsum_add<<<dim3(1, (unsigned)((n + 255) / 256)), MLP_OUT, 0, ctx->stream>>>(z, n, MLP_OUT, sum);
    MDET_LAUNCHED(ctx, "k_colsum_add");
    return MDET_OK;
}

int mlp_project(mdet_ctx* ctx, const float* z, uint64_t n, const float* V, int k, float* P) {
    const uint64_t chunk = 1u << 20;  // keeps the grid's y extent in range
    for (uint64_t r0 = 0; r0 < n; r0 += chunk) {
        const int rows = (int)std::min(chunk, n - r0);
        MDET_TRY((gemm<false, false, 0>(ctx, rows, k, MLP_OUT, z + r0 * MLP_OUT, MLP_OUT, V, k, P + r0 * k, k)));
    }
    return MDET_OK;
}

extern "C" {

int mdet_mlp_create(mdet_ctx* ctx, uint64_t seed, mdet_mlp** out) {
    if (!ctx || !out) return MDET_ERR_INVALID;
    MDET_CUDA(ctx, cudaSetDevice(ctx->device));
    mdet_mlp* m = new mdet_mlp();
    m->device = ctx->device;
    std::vector<float> p;
    host_init(seed, p);
    if (cudaMalloc(&m->params, MLP_NPARAM * 4) != cudaSuccess || cudaMalloc(&m->m, MLP_NTRAIN * 4) != cudaSuccess ||
        cudaMalloc(&m->v, MLP_NTRAIN * 4) != cudaSuccess) {
        cudaGetLastError();
        cudaFree(m->params);
        cudaFree(m->m);
        cudaFree(m->v);
        delete m;
        return ctx_fail(ctx, MDET_ERR_NOMEM, "network allocation failed");
    }
    cudaMemcpy(m->params, p.data(), MLP_NPARAM * 4, cudaMemcpyHostToDevice);
    cudaMemset(m->m, 0, MLP_NTRAIN * 4);
    cudaMemset(m->v, 0, MLP_NTRAIN * 4);
    *out = m;
    return MDET_OK;
}

int mdet_mlp_destroy(mdet_mlp* m) {
    if (!m) return MDET_OK;
    cudaSetDevice(m->device);
    cudaFree(m->params);
    cudaFree(m->m);
    cudaFree(m->v);
    cudaFree(m->pca);
    delete m;
    return MDET_OK;
}

uint64_t mdet_mlp_param_count(void) { return MLP_NPARAM; }

int mdet_mlp_get_params(mdet_ctx* ctx, const mdet_mlp* m, float* host, uint64_t count) {
    if (!ctx || !m || !host || count < MLP_NPARAM) return MDET_ERR_INVALID;
    MDET_CUDA(ctx, cudaMemcpy(host, m->params, MLP_NPARAM * 4, cudaMemcpyDeviceToHost));
    return MDET_OK;
}

int mdet_mlp_set_params(mdet_ctx* ctx, mdet_mlp* m, const float* host, uint64_t count) {
    if (!ctx || !m || !host || count < MLP_NPARAM) return MDET_ERR_INVALID;
    MDET_CUDA(ctx, cudaMemcpy(m->params, host, MLP_NPARAM * 4, cudaMemcpyHostToDevice));
    m->pca_valid = 0;  // the kept axes belong to the old parameters
    return MDET_OK;
}

// Embedding of n TNF rows (device pointers): d_out is n x 64.
int mdet_mlp_embed_dev(mdet_ctx* ctx, const mdet_mlp* m, const float* d_tnf, uint64_t n, float* d_out) {
    if (!ctx || !m || (n && (!d_tnf || !d_out))) return MDET_ERR_INVALID;
    MDET_CUDA(ctx, cudaSetDevice(ctx->device));
    MDET_TRY(mlp_embed(ctx, m->params, d_tnf, n, d_out));
    MDET_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return MDET_OK;
}

int mdet_ctx_set_learned(mdet_ctx* ctx, const mdet_mlp* mlp, mdet_learned_report* report) {
    if (!ctx) return MDET_ERR_INVALID;
    ctx->mlp = mlp;
    ctx->learned_report = report;
    return MDET_OK;
}

// Loss and gradient (host buffers) of the mean contrastive loss of `np`
// pairs over the rows of x (rows x 136 TNF rows): pairs[2p], pairs[2p+1]
// index rows of x.  For gradient checks against a CPU reference.
int mdet_mlp_grad(mdet_ctx* ctx, const mdet_mlp* m, const float* x, uint64_t rows, const uint32_t* pairs,
                  const float* labels, uint64_t np, float m_pos, float m_neg, float* grad_out, double* loss_out) {
    if (!ctx || !m || !x || !pairs || !labels || !grad_out || !loss_out || np == 0) return MDET_ERR_INVALID;
    MDET_CUDA(ctx, cudaSetDevice(ctx->device));
    cudaStream_t s = ctx->stream;
    for (uint64_t i = 0; i < 2 * np; ++i)
        if (pairs[i] >= rows) return ctx_fail(ctx, MDET_ERR_INVALID, "pair index out of range");
    float* dx = (float*)ctx_scratch(ctx, "mlpq.in", rows * MLP_IN * 4);
    uint32_t* didx = (uint32_t*)ctx_scratch(ctx, "mlpq.idx", 2 * np * 4);
    float* dl = (float*)ctx_scratch(ctx, "mlpq.lab", np * 4);
    float* g = (float*)ctx_scratch(ctx, "mlpq.g", MLP_NTRAIN * 4);
    double* loss = (double*)ctx_scratch(ctx, "mlpq.loss", 8);
    if (!dx || !didx || !dl || !g || !loss) return MDET_ERR_NOMEM;
    std::vector<uint32_t> idx(2 * np);
    for (uint64_t p = 0; p < np; ++p) {
        idx[p] = pairs[2 * p];
        idx[np + p] = pairs[2 * p + 1];
    }
    MDET_CUDA(ctx, cudaMemcpyAsync(dx, x, rows * MLP_IN * 4, cudaMemcpyHostToDevice, s));
    MDET_CUDA(ctx, cudaMemcpyAsync(didx, idx.data(), 2 * np * 4, cudaMemcpyHostToDevice, s));
    MDET_CUDA(ctx, cudaMemcpyAsync(dl, labels, np * 4, cudaMemcpyHostToDevice, s));
    MDET_CUDA(ctx, cudaMemsetAsync(loss, 0, 8, s));
    MlpTcActs a;
    MDET_TRY(mlp_tc_alloc(ctx, "mlpq", 2 * np, &a));
    MDET_TRY(mlp_forward_tc(ctx, m->params, dx, didx, 2 * np, a));
    MDET_TRY(mlp_backward_tc(ctx, m->params, a, np, dl, m_pos, m_neg, g, loss));
    MDET_CUDA(ctx, cudaMemcpyAsync(grad_out, g, MLP_NTRAIN * 4, cudaMemcpyDeviceToHost, s));
    double h = 0;
    MDET_CUDA(ctx, cudaMemcpyAsync(&h, loss, 8, cudaMemcpyDeviceToHost, s));
    MDET_CUDA(ctx, cudaStreamSynchronize(s));
    *loss_out = h / (double)np;
    return MDET_OK;
}

// Trains the network on pairs of a training assembly (device TNF rows and
// log sizes).  Pairs: the candidate pairs of the distance filter at the
// loosest cutoff the pTNF search can choose (0.7), plus uniformly random
// pairs; each labelled by the exact probability kernel (edge at 0.7 or not).
// The margin tau is then set to the given quantile of the embedded distance
// over held-out edge pairs.
int mdet_mlp_train(mdet_ctx* ctx, mdet_mlp* m, const float* d_tnf, const double* d_ls, uint64_t n,
                   const mdet_train_params* tp, mdet_train_report* rep) {
    if (!ctx || !m || !d_tnf || !d_ls || !tp || n < 2) return MDET_ERR_INVALID;
    MDET_CUDA(ctx, cudaSetDevice(ctx->device));
    cudaStream_t s = ctx->stream;
    mdet_train_report r;
    memset(&r, 0, sizeof(r));
    GraphPrep g;
    const int mode = (ctx->cc_major == 10 && ctx->cc_minor == 3) ? MDET_MODE_BF16 : MDET_MODE_PLAIN;
    MDET_TRY(prep_sorted(ctx, d_tnf, d_ls, n, mode != MDET_MODE_PLAIN, &g));
    uint2* cand = nullptr;
    uint64_t ncand = 0;
    MDET_TRY(graph_candidates(ctx, g, tp->label_cutoff, mode, &cand, &ncand));
    // pair pool: candidate pairs and random pairs, mixed at random so that
    // the held-out tail has both kinds
    const uint64_t pool = tp->pairs ? tp->pairs : 50000000ull;
    const double frac = std::min(1.0, std::max(0.0, tp->candidate_fraction));
    const uint64_t nc = ncand ? (uint64_t)(pool * frac) : 0;
    uint2* pairs = (uint2*)ctx_scratch(ctx, "mlpt.pairs", pool * sizeof(uint2));
    float* labels = (float*)ctx_scratch(ctx, "mlpt.labels", pool * 4);
    if (!pairs || !labels) return MDET_ERR_NOMEM;
    k_pair_pool<<<ctx->num_sms * 8, 256, 0, s>>>(tp->seed, pool, (uint32_t)n, cand, ncand, frac, pairs);
    MDET_LAUNCHED(ctx, "k_pair_pool");
    const double L = log((1.0 / (1. - tp->label_cutoff)) - 1.0);
    ff Lff;
    Lff.hi = (float)L;
    Lff.lo = (float)(L - (double)Lff.hi);
    k_label_pairs<<<ctx->num_sms * 16, 256, 0, s>>>(pairs, pool, g.x32, g.parts, model_h_ff(), Lff, labels);
    MDET_LAUNCHED(ctx, "k_label_pairs");
    // hold out the last 1% for calibration
    const uint64_t hold = std::max<uint64_t>(pool / 100, 1);
    const uint64_t train_pool = pool - hold;
    const uint32_t B = tp->batch_pairs ? tp->batch_pairs : 8192;
    MlpTcActs a;
    MDET_TRY(mlp_tc_alloc(ctx, "mlpt", 2ull * B, &a));
    uint32_t* bidx = (uint32_t*)ctx_scratch(ctx, "mlpt.bidx", 2ull * B * 4);
    float* blab = (float*)ctx_scratch(ctx, "mlpt.blab", (uint64_t)B * 4);
    float* grad = (float*)ctx_scratch(ctx, "mlpt.grad", MLP_NTRAIN * 4);
    double* loss = (double*)ctx_scratch(ctx, "mlpt.loss", 8);
    if (!bidx || !blab || !grad || !loss) return MDET_ERR_NOMEM;
    // input normalisation from the training rows: mean and a fixed scale
    {
        std::vector<float> mu(MLP_IN);
        MDET_CUDA(ctx, cudaMemcpyAsync(mu.data(), g.mu, MLP_IN * 4, cudaMemcpyDeviceToHost, s));
        MDET_CUDA(ctx, cudaStreamSynchronize(s));
        float scale = 10.f;
        MDET_CUDA(ctx, cudaMemcpy(m->params + MLP_MU, mu.data(), MLP_IN * 4, cudaMemcpyHostToDevice));
        MDET_CUDA(ctx, cudaMemcpy(m->params + MLP_SCALE, &scale, 4, cudaMemcpyHostToDevice));
    }
    const uint64_t steps = tp->steps;
    double loss_acc = 0;
    uint64_t loss_n = 0;
    for (uint64_t st = 0; st < steps; ++st) {
        k_batch<<<(B + 255) / 256, 256, 0, s>>>(pairs, labels, train_pool, tp->seed * 1315423911ull + st, B, bidx,
                                                blab);
        MDET_LAUNCHED(ctx, "k_batch");
        MDET_TRY(mlp_forward_tc(ctx, m->params, g.x32, bidx, 2ull * B, a));
        MDET_CUDA(ctx, cudaMemsetAsync(loss, 0, 8, s));
        MDET_TRY(mlp_backward_tc(ctx, m->params, a, B, blab, tp->m_pos, tp->m_neg, grad, loss));
        m->step++;
        const float c1 = 1.f - powf(0.9f, (float)m->step), c2 = 1.f - powf(0.999f, (float)m->step);
        const float lr = tp->lr * (st < steps / 10 ? 1.f : 0.5f * (1.f + cosf(3.14159265f * (float)(st - steps / 10) /
                                                                              (float)(steps - steps / 10 + 1))));
        // warm-up keeps the first Adam steps small
        const float lr_w = st < 100 ? lr * (float)(st + 1) / 100.f : lr;
        k_adam<<<(MLP_NTRAIN + 255) / 256, 256, 0, s>>>(m->params, m->m, m->v, grad, MLP_NTRAIN, lr_w, 0.9f, 0.999f,
                                                         1e-8f, c1, c2);
        MDET_LAUNCHED(ctx, "k_adam");
        if (st + 50 >= steps) {
            double h = 0;
            MDET_CUDA(ctx, cudaMemcpyAsync(&h, loss, 8, cudaMemcpyDeviceToHost, s));
            MDET_CUDA(ctx, cudaStreamSynchronize(s));
            loss_acc += h / B;
            loss_n++;
        }
    }
    // calibration on the held-out pairs
    {
        const uint64_t hc = std::min<uint64_t>(hold, 1u << 20);
        std::vector<float> lab(hc), e(hc);
        uint32_t* hidx = (uint32_t*)ctx_scratch(ctx, "mlpt.hidx", 2 * hc * 4);
        float* he = (float*)ctx_scratch(ctx, "mlpt.he", hc * 4);
        if (!hidx || !he) return MDET_ERR_NOMEM;
        std::vector<uint2> hp(hc);
        MDET_CUDA(ctx, cudaMemcpyAsync(hp.data(), pairs + train_pool, hc * sizeof(uint2), cudaMemcpyDeviceToHost, s));
        MDET_CUDA(ctx, cudaMemcpyAsync(lab.data(), labels + train_pool, hc * 4, cudaMemcpyDeviceToHost, s));
        MDET_CUDA(ctx, cudaStreamSynchronize(s));
        std::vector<uint32_t> idx(2 * hc);
        for (uint64_t p = 0; p < hc; ++p) {
            idx[p] = hp[p].x;
            idx[hc + p] = hp[p].y;
        }
        MDET_CUDA(ctx, cudaMemcpyAsync(hidx, idx.data(), 2 * hc * 4, cudaMemcpyHostToDevice, s));
        float* hz = (float*)ctx_scratch(ctx, "mlph.z", 2 * hc * MLP_OUT * 4);
        if (!hz) return MDET_ERR_NOMEM;
        MDET_TRY(mlp_embed_tc(ctx, m->params, g.x32, 2 * hc, hz, hidx));
        k_pair_dist<<<(unsigned)((hc + 7) / 8), 256, 0, s>>>(hz, hc, he);
        MDET_LAUNCHED(ctx, "k_pair_dist");
        MDET_CUDA(ctx, cudaMemcpyAsync(e.data(), he, hc * 4, cudaMemcpyDeviceToHost, s));
        MDET_CUDA(ctx, cudaStreamSynchronize(s));
        std::vector<float> pos, neg;
        for (uint64_t p = 0; p < hc; ++p) (lab[p] > 0.5f ? pos : neg).push_back(e[p]);
        std::sort(pos.begin(), pos.end());
        std::sort(neg.begin(), neg.end());
        float tau = INFINITY;
        if (!pos.empty()) {
            const double q = tp->tau_quantile > 0 ? tp->tau_quantile : 0.9995;
            tau = pos[std::min<size_t>(pos.size() - 1, (size_t)(q * (pos.size() - 1)))] * 1.05f;
        }
        MDET_CUDA(ctx, cudaMemcpy(m->params + MLP_TAU, &tau, 4, cudaMemcpyHostToDevice));
        r.tau = tau;
        r.held_pos = pos.size();
        r.held_neg = neg.size();
        r.pos_median = pos.empty() ? 0 : pos[pos.size() / 2];
        r.neg_median = neg.empty() ? 0 : neg[neg.size() / 2];
        size_t below = 0;
        for (float v : neg) below += v <= tau;
        r.neg_below_tau = neg.empty() ? 0 : (double)below / neg.size();
    }
    // the principal axes of the training set's embeddings, kept for the
    // contig order of the learned graph
    {
        float* zt = (float*)ctx_scratch(ctx, "mlpt.zall", n * MLP_OUT * 4);
        if (!zt) return MDET_ERR_NOMEM;
        if (!m->pca) MDET_CUDA(ctx, cudaMalloc(&m->pca, MLP_PCA_FLOATS * 4));
        MDET_TRY(mlp_embed(ctx, m->params, d_tnf, n, zt));
        MDET_TRY(mlp_pca_basis(ctx, zt, n, m->pca));
        m->pca_valid = 1;
    }
    r.steps = steps;
    r.pairs = pool;
    r.candidate_pairs = nc;
    r.final_loss = loss_n ? loss_acc / loss_n : 0;
    if (rep) *rep = r;
    return MDET_OK;
}

}  // extern "C"
