// mlp.cuh -- the embedding network of the learned proposal: 136 -> 256 ->
// 128 -> 64 with GELU, BF16 weights (the FP32 master copy is rounded to
// BF16 wherever a GEMM reads it), FP32 accumulation.  Kernels are this
// project's own: inference on the tensor cores (tcgen05, mlp_tc.cu, BF16
// activations); training with tiled SIMT GEMMs for forward and backward (FP32
// activations), GELU and its derivative, a contrastive pair loss and Adam.
#pragma once

#include "graph.cuh"

#define MLP_IN 136
#define MLP_H1 256
#define MLP_H2 128
#define MLP_OUT 64

// Offsets of the parameter blob (FP32, device and host alike).
#define MLP_W1 0
#define MLP_B1 (MLP_W1 + MLP_H1 * MLP_IN)
#define MLP_W2 (MLP_B1 + MLP_H1)
#define MLP_B2 (MLP_W2 + MLP_H2 * MLP_H1)
#define MLP_W3 (MLP_B2 + MLP_H2)
#define MLP_B3 (MLP_W3 + MLP_OUT * MLP_H2)
#define MLP_MU (MLP_B3 + MLP_OUT)   // input centring: x' = (tnf - mu) * scale
#define MLP_SCALE (MLP_MU + MLP_IN)
#define MLP_TAU (MLP_SCALE + 1)     // calibrated embedded-distance margin
#define MLP_NPARAM (MLP_TAU + 1)    // 76362 floats
#define MLP_NTRAIN MLP_MU           // parameters updated by the optimiser

struct mdet_mlp {
    float* params = nullptr;  // device, MLP_NPARAM floats
    float* m = nullptr;       // Adam moments (MLP_NTRAIN each)
    float* v = nullptr;
    uint64_t step = 0;
    int device = 0;
};

struct MlpActs {
    float* x;   // [rows][136] normalised input
    float* z1;  // [rows][256] pre-activation
    float* h1;  // [rows][256]
    float* z2;  // [rows][128]
    float* h2;  // [rows][128]
    float* z3;  // [rows][64]  embedding
};

// Embedding of `n` TNF rows (rows addressed through `idx` when non-null).
int mlp_forward(mdet_ctx* ctx, const float* params, const float* tnf, const uint32_t* idx, uint64_t n,
                const MlpActs& a);
// Gradient of the mean contrastive loss over `npairs` pairs whose endpoints
// are rows [0, npairs) and [npairs, 2*npairs) of the forward activations.
int mlp_backward(mdet_ctx* ctx, const float* params, const MlpActs& a, uint64_t npairs, const float* labels,
                 float m_pos, float m_neg, float* grad, double* loss_sum);
int mlp_alloc_acts(mdet_ctx* ctx, const char* tag, uint64_t rows, MlpActs* a);
// Embeddings of n rows (original order) into z (n x 64): the tensor-core
// inference kernel of mlp_tc.cu (BF16 activations, FP32 accumulation).
int mlp_embed(mdet_ctx* ctx, const float* params, const float* tnf, uint64_t n, float* z);
int mlp_embed_tc(mdet_ctx* ctx, const float* params, const float* tnf, uint64_t n, float* z);
// G = Z^T Z (64 x 64, accumulated into a zeroed G) and P = Z V (n x k, V 64 x k).
int mlp_gram(mdet_ctx* ctx, const float* z, uint64_t n, float* G);
// column sums of Z added into a zeroed s (64)
int mlp_colsum(mdet_ctx* ctx, const float* z, uint64_t n, float* s);
int mlp_project(mdet_ctx* ctx, const float* z, uint64_t n, const float* V, int k, float* P);
