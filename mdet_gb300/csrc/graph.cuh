// graph.cuh -- internals shared by the pairwise-stage kernels.
#pragma once

#include "common.cuh"
#include "ff.cuh"

#include <functional>

#define MDET_KPAD 144     // BF16 row length: 136 features + 8 zeros (9 x 16)
constexpr int kShapeTall = 1256;  // filter_tc shape code of 256 x 128 tiles
constexpr int kShapeTf32 = 2128;  // filter_tc shape code of 128 x 128 TF32 tiles
#define MDET_TBL 256      // threshold table cells per axis
#define MDET_TBL_LEVELS 9 // sparse-table levels (2^8 = 256)
#define MDET_BLK 128      // rows per metadata block

// Per 128-row block of the length-sorted order.
struct BlockMeta {
    float lo, hi;  // log10 size range
    float emax;    // max rounding error ||x~ - x|| of the block's reduced-precision rows
    float nmax;    // max norm of the block's centred reduced-precision rows
};

// Conservative upper bound of d*(x, y) over boxes of log sizes: a
// 256 x 256 cell table over [lmin, lmax], suffix-maximised along x, with a
// sparse table along y.
struct DstarTable {
    const float* st;  // [levels][TBL][TBL]
    float lmin, inv_h;
    const float* dyn;  // optional device copy of {lmin, inv_h}, read by the kernels instead
};

// Grid of a table built from a device-resident size range.
struct TableGrid {
    double lmin, h;  // first cell edge and cell width
    float lminf, inv_hf;
};

// Pairs handed from the distance filter to the exact stage.
struct CandBuf {
    uint2* cand;                 // (row, col) in the filter's index spaces
    unsigned long long* count;   // total found (may exceed cap: then rerun bigger)
    unsigned long long cap;
};

// Model parts of one contig: F_m(x) and G_m(y) for m in {b1, c1, b2, c2}.
struct ModelParts {
    double f[4];
    double g[4];
};

struct ModelH {
    double h[4][6];  // H_m(t) coefficients t^1..t^5 (index 0 unused)
};

// The exact stage's per-contig data in float-float: F_m, G_m and the log size.
struct PartsFF {
    ff f[4];
    ff g[4];
    ff ls;
    float pad[2];
};

struct ModelHFF {
    ff h[4][6];
};

__device__ __forceinline__ int tbl_cell_lo(float v, const DstarTable& t) {
    int c = (int)floorf((v - t.lmin) * t.inv_h - 1e-3f);
    return c < 0 ? 0 : (c >= MDET_TBL ? MDET_TBL - 1 : c);
}
__device__ __forceinline__ int tbl_cell_hi(float v, const DstarTable& t) {
    int c = (int)floorf((v - t.lmin) * t.inv_h + 1e-3f);
    return c < 0 ? 0 : (c >= MDET_TBL ? MDET_TBL - 1 : c);
}

// Largest d* over all pairs whose sizes come from blocks with log-size
// ranges [alo, ahi] and [blo, bhi]: the x range starts at min(alo, blo),
// whose suffix-maximised row covers the whole x range; two sparse-table
// reads cover the y range.
// The bound is the larger of two table entries; tile_dstar_cells gives their
// addresses so that a caller can issue the loads early.
__device__ __forceinline__ void tile_dstar_cells(const DstarTable& t, float alo, float ahi, float blo, float bhi,
                                                 const float*& c0, const float*& c1) {
    const float xlo = fminf(alo, blo);
    const float ylo = fmaxf(alo, blo), yhi = fmaxf(ahi, bhi);
    const int cx0 = tbl_cell_lo(xlo, t);
    const int cy0 = tbl_cell_lo(ylo, t), cy1 = tbl_cell_hi(yhi, t);
    const int span = cy1 - cy0 + 1;
    const int k = 31 - __clz(span);
    const float* lvl = t.st + (size_t)k * MDET_TBL * MDET_TBL + cx0 * MDET_TBL;
    c0 = lvl + cy0;
    c1 = lvl + (cy1 - (1 << k) + 1);
}
__device__ __forceinline__ float tile_dstar(const DstarTable& t, float alo, float ahi, float blo, float bhi) {
    const float *c0, *c1;
    tile_dstar_cells(t, alo, ahi, blo, bhi, c0, c1);
    return fmaxf(__ldg(c0), __ldg(c1));
}

// Host-side entry points of the stages (graph_*.cu).
struct GraphPrep {
    uint32_t n, npad;                // contigs, rows padded to 256
    uint32_t* perm;                  // sorted position -> original index
    uint32_t* inv;                   // original index -> sorted position
    float* x32;                      // sorted FP32 TNF rows [n][136]
    double* ls;                      // sorted log sizes
    PartsFF* parts;                  // sorted model parts and log sizes (float-float)
    uint16_t* xa;                    // A role: sorted centred BF16 rows [x~, 1, 1, 0..] [npad][144]
    uint16_t* xb;                    // B role: [x~, -hi(||x~||^2/2), -lo(||x~||^2/2), 0..]; padding -inf
    float* ta;                       // the same two roles with TF32-rounded rows (FP32 containers)
    float* tb;
    int tck;                         // reduced-precision rows held: kTcNone, kTcBf16 or kTcTf32
    float* nsq;                      // ||x~||^2 per sorted row (inf for padding rows)
    BlockMeta* meta;                 // per 128-row block (rounding of the rows held)
    BlockMeta* meta32;               // per 128-row block (no rounding term)
    float* mu;                       // column means [136]
    const uint8_t* low = nullptr;    // abundance gate: sorted position has no depth above 1 (null: no gate)
};

// Sets g.low from the abundance on the context (a pair of two low contigs is
// not an edge); no abundance: g.low = null.  Fails when the abundance covers a
// different number of contigs.
int abd_gate(mdet_ctx* ctx, GraphPrep& g);

// Reduced-precision rows a preparation holds for the tensor-core filter.
constexpr int kTcNone = 0, kTcBf16 = 1, kTcTf32 = 2;
inline int tc_kind(int mode) {
    return mode == MDET_MODE_PLAIN ? kTcNone : (mode == MDET_MODE_TF32 ? kTcTf32 : kTcBf16);
}

// Prepares the contigs in ascending log-size order, or in `order` (original
// index per position, device) when given.  tck: the reduced-precision rows
// to make (kTcNone, kTcBf16, kTcTf32; a bool true means kTcBf16).
int prep_sorted(mdet_ctx* ctx, const float* d_tnf, const double* d_ls, uint64_t n, int tck, GraphPrep* out,
                const uint32_t* order = nullptr);
// Arrays of a prepared set of `rows` positions (a multiple of 256) in
// scratch named after tag; prep_into fills positions [base, base + npad) of
// them with one contig set (perm/inv values are base + local indices).
int prep_alloc(mdet_ctx* ctx, const char* tag, uint64_t rows, int tck, GraphPrep* g);
int prep_into(mdet_ctx* ctx, const float* d_tnf, const double* d_ls, uint64_t n, int tck, const GraphPrep& g,
              uint64_t base, const uint32_t* order = nullptr);
// sorted: d_ls_sorted is ascending (else its range is found by a scan).
// range: optional host copy of the log-size range {min, max}; when given with
// range[0] not NaN it is used as is, else it is found (one device round trip)
// and stored there for the next call over the same sizes.
int build_dstar_table(mdet_ctx* ctx, const double* d_ls_sorted, uint64_t n, double logit_cut, DstarTable* out,
                      bool sorted = true, double* range = nullptr);
// A table over a given log-size range written to st (MDET_TBL_LEVELS x TBL x TBL floats).
int build_dstar_table_at(mdet_ctx* ctx, double lmin, double lmax, double logit_cut, float* st, DstarTable* out);
// The same over the union of `count` device ranges (lo, hi pairs; entries
// with lo > hi are empty): no host synchronisation, grid left in *grid.
int grid_from_ranges(mdet_ctx* ctx, const double* ranges, uint32_t count, TableGrid* grid);
int build_dstar_table_dev(mdet_ctx* ctx, const TableGrid* grid, double logit_cut, float* st, DstarTable* out);
#define MDET_TBL_FLOATS ((uint64_t)MDET_TBL_LEVELS * MDET_TBL * MDET_TBL)
ModelH model_h();
ModelHFF model_h_ff();

// Above-cutoff pair found by the exact stage (sorted positions).
struct Edge {
    uint32_t i, j;
    double sim;
};

// One entry of a contig's edge list.
struct Ent {
    double sim;
    uint32_t ocol;  // original column index
    uint32_t pad;
};

// tiles/nlist: optional list of 128 x 128 tiles (I * tiles_b + J); row_tbl:
// optional d* table index per row tile (tables tbl_stride floats apart from
// tbl.st).
int filter_simt(mdet_ctx* ctx, const float* a, uint32_t na, const BlockMeta* ameta, const float* b, uint32_t nb,
                const BlockMeta* bmeta, bool triangular, const DstarTable& tbl, CandBuf out,
                const uint32_t* tiles = nullptr, uint64_t nlist = 0, const uint8_t* row_tbl = nullptr,
                uint64_t tbl_stride = 0);
// Tensor-core filter over centred reduced-precision rows: a (A role, na
// rows) against b (B role, nb rows), both padded to 256 rows; a_nsq =
// ||a~||^2 (+inf on padding rows).  BF16 rows (uint16) by default; with
// bn == kShapeTf32 TF32 rows (FP32 containers, 128 x 128 tiles).
// tiles/nlist: optional row-major list (I * tiles_b + J) of the tile pairs
// to evaluate (column tiles of bn); null evaluates the whole schedule.
// rowoff (with a list): entries of row tile I are [rowoff[I], rowoff[I+1]),
// and row tiles are taken in the waves of the full schedule.
// bn: tile shape: 256 = 128 x 256 tiles (one CTA per SM), 128 = 128 x 128
// (two per SM), kShapeTall = 256 x 128 with four B stages (no tile lists).
int filter_tc(mdet_ctx* ctx, const void* a, const float* a_nsq, uint32_t na, const BlockMeta* ameta,
              const void* b, uint32_t nb, const BlockMeta* bmeta, bool triangular, const DstarTable& tbl,
              CandBuf out, const uint32_t* tiles = nullptr, uint64_t nlist = 0, const uint8_t* row_tbl = nullptr,
              uint64_t tbl_stride = 0, int bn = 256, const unsigned long long* rowoff = nullptr);
// Cutoff of one 256-row block of a batch: logit(cutoff) in float-float and
// whether the second model is needed (logit(cutoff) < ln 9, decided in FP64).
struct BlkCut {
    ff L;
    uint32_t model2;
    uint32_t pad;
};
// blk_L: optional per-256-row-block cutoff overriding L.
// ncand_dev: the candidate count on the device (ncand is then its cap); with
// nedges_dev the edge count stays on the device too and nothing is read back.
int exact_graph(mdet_ctx* ctx, const GraphPrep& g, const uint2* cand, unsigned long long ncand, double L,
                Edge** edges_out, unsigned long long* nedges_out, uint32_t** deg_out,
                const BlkCut* blk_L = nullptr, const unsigned long long* ncand_dev = nullptr,
                unsigned long long** nedges_dev = nullptr);
// swapped: the pairs are (other row, sample slot) instead of (sample slot, other row)
int exact_maxprob(mdet_ctx* ctx, const GraphPrep& g, const uint2* cand, unsigned long long ncand,
                  const uint32_t* row_map, uint64_t m, const uint32_t* slot_of, double* d_out, bool swapped = false);
// Exact-stage distance and probability of given pairs (original indices).
int pair_scores(mdet_ctx* ctx, const GraphPrep& g, const uint64_t* pairs, uint64_t m, double* dist, double* prob);
// blk_K: optional per-256-row-block max_edges (each <= max_edges <= 512).
// ne_dev: the edge count on the device (ne is then its cap); the total is
// then left in the device outptr[n] and *n_out is 0.
// keep0/keep1: only rows whose sorted position lies in [keep0, keep1) are
// emitted (row shards; needs max_edges <= 512).
int select_topk(mdet_ctx* ctx, const GraphPrep& g, const Edge* edges, unsigned long long ne, uint32_t* deg,
                uint32_t max_edges, uint64_t* n_out, const uint32_t* blk_K = nullptr,
                const unsigned long long* ne_dev = nullptr, uint32_t keep0 = 0, uint32_t keep1 = 0xFFFFFFFFu);
int emit_topk(mdet_ctx* ctx, const GraphPrep& g, uint32_t max_edges, uint64_t* d_from, uint64_t* d_to,
              double* d_stnf, uint64_t total);

// Orchestration shared by the graph entry points (graph.cu, graph_learned.cu,
// graph_batch.cu).
double logit(double cutoff);
int check_flag(mdet_ctx* ctx);
int check_mode(mdet_ctx* ctx, int mode);
// A subset of rows in the B role (BF16 B layout, per-128-row metadata), for a
// rectangular pass of all rows (A role) against the subset.
struct BSide {
    const uint16_t* xb;
    uint32_t nb;
    const BlockMeta* meta;
};
int run_filter(mdet_ctx* ctx, int mode, const GraphPrep& g, bool rect, const float* a32, const uint16_t* ab,
               const float* ansq, uint32_t na, const BlockMeta* ameta, const BlockMeta* ameta32,
               const DstarTable& tbl, const char* tag, uint2** cand_out, unsigned long long* ncand_out,
               const uint32_t* tiles = nullptr, uint64_t nlist = 0, const uint8_t* row_tbl = nullptr,
               uint64_t tbl_stride = 0, int bn = 0, unsigned long long fixed_cap = 0,
               unsigned long long** cnt_dev = nullptr, const unsigned long long* rowoff = nullptr,
               const BSide* bside = nullptr);
// Tile-shape autotuner: run(bn) performs one filter pass with column tiles
// of bn.  The first pass of a shape class times bn = 256 and bn = 128 and
// keeps the faster (the later pass's output stands); later passes use it.
int tc_autotune(mdet_ctx* ctx, uint64_t key, const std::function<int(int)>& run, bool list = false);
// Launch-shape autotuner: the first call of a shape class times run(v) for
// every candidate value (the last run's output stands) and keeps the fastest
// in `table`; later calls run the kept value.
int launch_autotune(mdet_ctx* ctx, std::map<uint64_t, int>& table, uint64_t key, const std::vector<int>& values,
                    const std::function<int(int)>& run);
uint64_t tc_shape_key(bool rect, bool list, uint64_t na, uint64_t nb);
int graph_core(mdet_ctx* ctx, const float* d_tnf, const double* d_ls, uint64_t n, double cutoff, uint32_t max_edges,
               int mode, mdet_graph_stats* st, GraphPrep& g, uint64_t* total);
int graph_learned(mdet_ctx* ctx, const float* d_tnf, const double* d_ls, uint64_t n, double cutoff, uint32_t max_edges,
                  mdet_graph_stats* st, GraphPrep& g, uint64_t* total);
// Candidate pairs (prepared positions) of the triangular pass at `cutoff`.
int graph_candidates(mdet_ctx* ctx, const GraphPrep& g, double cutoff, int mode, uint2** cand, uint64_t* ncand);
// A-role BF16 rows of a prepared set gathered for a rectangular pass
// (row_map: ascending prepared positions on the device, m entries), padded
// to 256 rows, with their norms and block metadata.
struct RowSet {
    uint16_t* ab;
    float* ansq;
    BlockMeta* meta;
};
int gather_rows_bf16(mdet_ctx* ctx, const GraphPrep& g, const uint32_t* row_map, uint64_t m, const char* tag,
                     RowSet* out);
