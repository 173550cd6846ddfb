// mlp.cuh -- the embedding network of the learned proposal: 136 -> 256 ->
// 128 -> 64 with GELU, BF16 weights (the FP32 master copy is rounded to
// BF16 wherever a GEMM reads it), FP32 accumulation.  Kernels are this
// project's own: the forward and backward GEMMs on the tensor cores
// (tcgen05, mlp_tc.cu, BF16 operands, FP32 accumulation), GELU and its
// derivative, a contrastive pair loss and Adam; a tiled SIMT GEMM serves the
// embedding's principal axes (64 x 64 Gram matrix, projections).
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

// the Morton key's basis: 64 x 8 principal axes, 8 offsets, 8 inverse spans
#define MLP_PCA_FLOATS (MLP_OUT * 8 + 16)

struct mdet_mlp {
    float* params = nullptr;  // device, MLP_NPARAM floats
    float* m = nullptr;       // Adam moments (MLP_NTRAIN each)
    float* v = nullptr;
    float* pca = nullptr;     // device, MLP_PCA_FLOATS: principal axes of the training set's embeddings
    int pca_valid = 0;        // set by training, cleared when the parameters are replaced
    uint64_t step = 0;
    int device = 0;
};

// principal axes of embeddings z (n x 64) into basis (MLP_PCA_FLOATS, device)
int mlp_pca_basis(mdet_ctx* ctx, const float* z, uint64_t n, float* basis);

// Embeddings of n rows (original order) into z (n x 64): the tensor-core
// inference kernel of mlp_tc.cu (BF16 activations, FP32 accumulation).
int mlp_embed(mdet_ctx* ctx, const float* params, const float* tnf, uint64_t n, float* z);
// (rows idx[i] of tnf when idx is non-null)
int mlp_embed_tc(mdet_ctx* ctx, const float* params, const float* tnf, uint64_t n, float* z, const uint32_t* idx);

// Training on the tensor cores (mlp_tc.cu): rows padded to ld (a multiple of
// 128); FP32 pre-activations and output gradients row-major, BF16 GEMM
// operands of the weight gradients feature-major ([features][ld]).
#include <cuda_bf16.h>
struct MlpTcActs {
    uint64_t ld;
    float *z1, *z2, *z3;  // [ld][256], [ld][128], [ld][64] (z3: the embedding)
    float *d3, *d2, *d1;  // dL/dz3, dL/dz2, dL/dz1
    __nv_bfloat16 *xT, *h1T, *h2T;  // layer inputs: [192][ld], [256][ld], [128][ld]
    __nv_bfloat16 *d3T, *d2T, *d1T; // output gradients: [64][ld], [128][ld], [256][ld]
};
int mlp_tc_alloc(mdet_ctx* ctx, const char* tag, uint64_t rows, MlpTcActs* a);
// forward over rows tnf[idx[i]], keeping what the backward pass needs
int mlp_forward_tc(mdet_ctx* ctx, const float* params, const float* tnf, const uint32_t* idx, uint64_t rows,
                   const MlpTcActs& a);
// loss over npairs pairs (rows p and npairs + p) and its gradient
int mlp_backward_tc(mdet_ctx* ctx, const float* params, const MlpTcActs& a, uint64_t npairs, const float* labels,
                    float m_pos, float m_neg, float* grad, double* loss_sum);
int mlp_pair_loss(mdet_ctx* ctx, const float* z, uint64_t np, const float* labels, float m_pos, float m_neg,
                  float* dz, double* loss_sum);
// G = Z^T Z (64 x 64, accumulated into a zeroed G) and P = Z V (n x k, V 64 x k).
int mlp_gram(mdet_ctx* ctx, const float* z, uint64_t n, float* G);
// column sums of Z added into a zeroed s (64)
int mlp_colsum(mdet_ctx* ctx, const float* z, uint64_t n, float* s);
int mlp_project(mdet_ctx* ctx, const float* z, uint64_t n, const float* V, int k, float* P);
