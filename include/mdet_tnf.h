/*
 * mdet_tnf.h -- C ABI of the GB300 (sm_103a) MetaBAT2 TNF path.
 *
 * Plain C types only: host or device pointers plus sizes, int status codes,
 * an opaque context that owns its device memory and CUDA stream.  One host
 * thread at a time per context.  Every call that takes HOST buffers copies
 * them in and out itself (pinned staging inside the context); the *_dev
 * variants take device pointers that stay resident.
 *
 * Each entry point names the reference interface it replaces (paths
 * relative to the MdeT project root).  The reference itself has no library
 * boundary: its stages are free functions over globals that exit(1) on any
 * CUDA error (getError, cuda/Cuda2.cu:341-354); here every failure is a
 * status code and mdet_last_error() says why.
 */
#ifndef MDET_TNF_H
#define MDET_TNF_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes */
#define MDET_OK 0
#define MDET_ERR_INVALID 1     /* bad argument (null pointer, size out of range) */
#define MDET_ERR_CUDA 2        /* CUDA runtime / driver error */
#define MDET_ERR_NOMEM 3       /* device or pinned allocation failed */
#define MDET_ERR_CAPACITY 4    /* caller's output buffer too small; *n_out holds the size needed */
#define MDET_ERR_TIMEOUT 5     /* a bounded device-side wait ran out; the context stays usable */
#define MDET_ERR_UNSUPPORTED 6 /* mode not available (e.g. tensor-core path on a non-sm_103 device) */
#define MDET_ERR_INTERNAL 7    /* an internal consistency check of the device work failed */

/* distance-filter forms of the pairwise stage */
#define MDET_MODE_PLAIN 0   /* FP32 SIMT all-pairs distance in the reference's element order */
#define MDET_MODE_BF16 1    /* tcgen05 BF16 tile GEMM, FP32 accumulation in TMEM */
#define MDET_MODE_TF32 2    /* tcgen05 TF32 tile GEMM (128 x 128 tiles), FP32 accumulation in TMEM; the
                             * max-probability sample passes use the BF16 filter (same maxima) */
#define MDET_MODE_LEARNED 3 /* learned embedding proposal + BF16 tiles (see mdet_tnf_learned_*) */

typedef struct mdet_ctx mdet_ctx;

typedef struct {
    uint64_t n_candidates;   /* pairs that passed the conservative distance filter */
    uint64_t n_above_cutoff; /* unordered pairs whose exact probability beats the cutoff */
    uint64_t n_edges;        /* emitted (from < to) edges */
    uint64_t tiles_total;    /* tile pairs in the pairwise schedule */
    uint64_t tiles_computed; /* tile pairs actually evaluated (< total with the learned proposal) */
    uint32_t gpu_launches;   /* kernels this call launched */
    uint32_t tile_m_n;       /* filter tile of the last launch: 1000 * rows + columns (128256, 256128, 128128) */
    double ms_prep, ms_filter, ms_exact, ms_select, ms_total; /* device time per phase */
} mdet_graph_stats;

/* ---- context ---------------------------------------------------------- */
int mdet_ctx_create(int device, mdet_ctx** out);
int mdet_ctx_destroy(mdet_ctx* ctx);
/* Last error message of this context ("" if none). */
const char* mdet_last_error(const mdet_ctx* ctx);
/* Use `stream` (a cudaStream_t) for all later work instead of the context's own. */
int mdet_ctx_set_stream(mdet_ctx* ctx, void* stream);
/* Build identification: "sm_103a ..." */
const char* mdet_version(void);
/* Tile-shape autotuner (on by default): the first call of each shape class
 * times the tensor-core filter's tile shapes -- 128 x 256 (one CTA per SM),
 * 128 x 128 (two per SM), 256 x 128 with four B stages (one per SM) -- and
 * the exact stage's blocks per SM, and keeps the fastest for the context.
 * mode 1: tune; 0: fixed 128 x 256 tiles and 8 blocks per SM; 128256,
 * 128128 or 256128: force that filter tile (tile lists fall back to 128 x 256
 * for 256128). */
int mdet_ctx_set_autotune(mdet_ctx* ctx, int mode);

/* Kernel timing: when enabled, the main kernels (k_count, k_filter_tc,
 * k_filter_simt, k_exact_graph, k_exact_maxprob) are bracketed by CUDA events
 * on the context's stream; mdet_ctx_kernel_ms returns the summed device time
 * of the named kernel's launches since timing was last enabled, and *launches
 * their number. */
int mdet_ctx_set_timing(mdet_ctx* ctx, int enable);
int mdet_ctx_kernel_ms(mdet_ctx* ctx, const char* kernel, double* ms, uint32_t* launches);
/* Kernels this context has launched since it was created. */
uint64_t mdet_ctx_launch_count(const mdet_ctx* ctx);
/* Failure detection check (no counterpart in the reference, which has no
 * device-side waits): one thread of a one-block kernel waits, through the
 * same bounded mbarrier wait the tensor-core filter uses, on a barrier that
 * nothing arrives on, with a budget of budget_cycles SM cycles (at most the
 * library's own ~2 s budget).  The wait runs out, the kernel raises the
 * context's error flag and returns, and the call returns MDET_ERR_TIMEOUT
 * with the context still usable -- what every other entry point does when
 * one of its waits runs out. */
int mdet_ctx_check_wait(mdet_ctx* ctx, uint64_t budget_cycles);

/* Page-locked host memory, as the reference allocates its file buffer and
 * TNF rows (cudaMallocHost, cuda/Cuda2.cu:1462, 1826): copies between it and
 * the device run at the link's full rate, copies from ordinary memory are
 * staged.  mdet_host_free(null) does nothing. */
int mdet_host_alloc(uint64_t bytes, void** out);
int mdet_host_free(void* p);

/* ---- TNF counting ------------------------------------------------------
 * Replaces the TNF loop of main (cuda/Cuda2.cu:1825-1863) and the copy of
 * TNF/logSizes to the devices (cuda/Cuda2.cu:1866-1874).  bytes[off[i] ..
 * off[i]+len[i]) is contig i's sequence view exactly as the reference's
 * reader builds it (newlines included, cuda/Cuda2.cu:1521-1530).  Outputs
 * counts (n*136 uint32, canonical tetranucleotide columns in TNF.bin order)
 * and tnf (n*136 float, c / sqrt(sum float(c*c))).  A contig with no valid
 * tetranucleotide gets zero counts and NaN TNF (0/0), as in the reference.
 * mdet_tnf_count takes counts == null when the caller needs only the TNF
 * rows (the reference pipeline reads TNF alone); the integer counts are then
 * not copied back. */
int mdet_tnf_count(mdet_ctx* ctx, const char* bytes, uint64_t nbytes, const uint64_t* off,
                   const uint64_t* len, uint64_t n, uint32_t* counts, float* tnf);
int mdet_tnf_count_dev(mdet_ctx* ctx, const char* d_bytes, uint64_t nbytes, const uint64_t* d_off,
                       const uint64_t* d_len, uint64_t n, uint32_t* d_counts, float* d_tnf);

/* Allocation-free TNF counting.  No counterpart in the reference: it exists
 * for callers that cannot allocate device memory -- a host application that
 * owns a fixed device arena and passes this library only its own buffers, or
 * a pipeline where a cudaMalloc (which synchronises the device and can fail
 * under memory pressure) is not allowed between stages.  Same inputs, outputs
 * and results as mdet_tnf_count_dev, but no context: the work runs on
 * `stream` (a cudaStream_t, 0 for the default stream) with its scratch in a
 * static device array of about 4.9 MB that every GPU loading the library
 * holds until exit.  Limits: n <= 8192 contigs and at most 65536 64-KB pieces
 * of sequence (about 4 GB); larger inputs return MDET_ERR_CAPACITY, and a
 * contig view outside [0, nbytes) returns MDET_ERR_INVALID, both checked
 * on the device before any sequence byte is read.  The first call on a
 * device resolves the array's device address there.  All calls share the
 * one array, so calls
 * whose work overlaps on the GPU race; serialise them.  Every call,
 * successful or not, synchronises `stream` before it returns.  Errors are
 * status codes only (there is no context for mdet_last_error). */
int mdet_tnf_count_noalloc(const char* d_bytes, uint64_t nbytes, const uint64_t* d_off, const uint64_t* d_len,
                           uint64_t n, uint32_t* d_counts, float* d_tnf, void* stream);

/* ---- FASTA ingest ------------------------------------------------------
 * Replaces the reader of main (cuda/Cuda2.cu:1486-1553) for the file's bytes
 * already in memory: the record split, the size classes and the log sizes,
 * run on the GPU.  Record rules (the reference's loop, read sequentially): a
 * '>' starts a record wherever it stands, except inside the name line of the
 * record before it; the name is the rest of that line cut at its first space;
 * the sequence view runs from after that line's newline to the next record's
 * '>' (or the end of the buffer), inner newlines kept, one trailing newline
 * dropped; size = the view's bytes before that drop minus its newlines.  A
 * name line that reaches the end of the buffer without a newline is not a
 * record (the reference would read past its buffer there).  Records with
 * size >= min_contig are written in file order: sequence view (offset and
 * length into the buffer, as mdet_tnf_count takes them), size, log size
 * log10(min(size, 500000)) (cuda/Cuda2.cu:1535) and name (offset, length).
 * n_small counts the records with 1000 <= size < min_contig (the reference's
 * small contigs).  MDET_ERR_CAPACITY when more than `capacity` records
 * qualify (n_large then holds the count).  size, log_size, name_off and
 * name_len may be null.  The device form needs a 16-byte aligned buffer. */
typedef struct {
    uint64_t n_records;  /* records found */
    uint64_t n_large;    /* records with size >= min_contig */
    uint64_t n_small;    /* records with 1000 <= size < min_contig */
    double ms_total;     /* device time of the call */
} mdet_fasta_stats;

int mdet_fasta_index(mdet_ctx* ctx, const char* bytes, uint64_t nbytes, uint64_t min_contig,
                     uint64_t capacity, uint64_t* seq_off, uint64_t* seq_len, uint64_t* size,
                     double* log_size, uint64_t* name_off, uint32_t* name_len, mdet_fasta_stats* stats);
int mdet_fasta_index_dev(mdet_ctx* ctx, const char* d_bytes, uint64_t nbytes, uint64_t min_contig,
                         uint64_t capacity, uint64_t* d_seq_off, uint64_t* d_seq_len, uint64_t* d_size,
                         double* d_log_size, uint64_t* d_name_off, uint32_t* d_name_len,
                         mdet_fasta_stats* stats);

/* The reader's record split and the TNF loop of main (cuda/Cuda2.cu:
 * 1486-1553, 1825-1863) in one call from the file's bytes in host memory: one
 * copy to the device, the split there, the count on the views it produced.
 * Outputs for the contigs with size >= min_contig, in file order, up to
 * `capacity` of them: views (seq_off, seq_len), sizes, log sizes and names
 * (name_off, name_len) as mdet_fasta_index writes them (each may be null),
 * counts and TNF (n x 136 each).  stats as mdet_fasta_index. */
int mdet_tnf_count_fasta(mdet_ctx* ctx, const char* bytes, uint64_t nbytes, uint64_t min_contig,
                         uint64_t capacity, uint64_t* seq_off, uint64_t* seq_len, uint64_t* size,
                         double* log_size, uint64_t* name_off, uint32_t* name_len, uint32_t* counts,
                         float* tnf, mdet_fasta_stats* stats);

/* ---- max-probability sample --------------------------------------------
 * Replaces launch_tnf_max_prob_sample_kernel_multi (cuda/Cuda2.cu:356-379)
 * with get_tnf_max_prob_sample (cuda/Cuda2.cu:281-314): for each sampled
 * position b < m of the permutation `contigs` (length n), the similarity
 * sigmoid(max pre-probability) against every other contig.
 * floor_prob: values at or above it are exact; a sampled contig whose true
 * maximum is below floor_prob reports some value below floor_prob (the
 * reference's pTNF search never looks below 0.701).  floor_prob <= 0 makes
 * every value exact (all pairs scored). */
int mdet_tnf_max_prob(mdet_ctx* ctx, const float* tnf, const double* log_size, uint64_t n,
                      const uint64_t* contigs, uint64_t m, int mode, double floor_prob, double* out);
int mdet_tnf_max_prob_dev(mdet_ctx* ctx, const float* d_tnf, const double* d_log_size, uint64_t n,
                          const uint64_t* d_contigs, uint64_t m, int mode, double floor_prob,
                          double* d_out);

/* ---- pTNF search -------------------------------------------------------
 * Replaces gen_tnf_graph_sample and its driver (cuda/Cuda2.cu:972-1025,
 * 1883-1904): samples with glibc rand() in the reference's order (the caller
 * seeds it with srand, as the reference's main does) and returns pTNF in
 * permille in *ptnf_out. coverage = maxP/100. */
int mdet_tnf_ptnf_search(mdet_ctx* ctx, const float* tnf, const double* log_size, uint64_t n,
                         double coverage, int mode, double* ptnf_out);
int mdet_tnf_ptnf_search_dev(mdet_ctx* ctx, const float* d_tnf, const double* d_log_size, uint64_t n,
                             double coverage, int mode, double* ptnf_out);

/* ---- TNF graph ---------------------------------------------------------
 * Replaces gen_tnf_graph (cuda/Cuda2.cu:861-970) with kernel get_tnf_graph2
 * (cuda/Cuda2.cu:243-262): every pair with pre-probability above
 * logit(cutoff) is scored sigmoid(pre); each contig keeps its max_edges best
 * (ties by lower column), and edge (i, j, sTNF) is emitted when i < j and j
 * is among i's kept.  Output rows ascending, inside a row by similarity
 * descending then j ascending (the reference's order across tiles is
 * unspecified).  Host arrays of `capacity` entries; *n_edges receives the
 * count (on MDET_ERR_CAPACITY, the count needed). */
int mdet_tnf_graph(mdet_ctx* ctx, const float* tnf, const double* log_size, uint64_t n, double cutoff,
                   uint32_t max_edges, int mode, uint64_t* from, uint64_t* to, double* stnf,
                   uint64_t capacity, uint64_t* n_edges, mdet_graph_stats* stats);
/* Device-resident form: d_tnf/d_log_size and the three outputs on the device. */
int mdet_tnf_graph_dev(mdet_ctx* ctx, const float* d_tnf, const double* d_log_size, uint64_t n,
                       double cutoff, uint32_t max_edges, int mode, uint64_t* d_from, uint64_t* d_to,
                       double* d_stnf, uint64_t capacity, uint64_t* n_edges, mdet_graph_stats* stats);
/* Row shard `shard` of `nshards` (0 <= shard < nshards) of the same graph,
 * for one GPU each: the contigs in ascending log size are cut into nshards
 * contiguous blocks on 256-row boundaries, and a shard emits the edges (i, j),
 * i < j, of the rows i in its block, scored against all n contigs.  The
 * shards' edge lists together are exactly the mdet_tnf_graph edge list (as
 * when cuda/Cuda2.cu:888-891 deals row tiles to devices), so the only exchange
 * is their concatenation.  TNF and log sizes are passed whole to every shard.
 * PLAIN or BF16 form; max_edges <= 512. */
int mdet_tnf_graph_shard(mdet_ctx* ctx, const float* tnf, const double* log_size, uint64_t n, double cutoff,
                         uint32_t max_edges, int mode, uint32_t shard, uint32_t nshards, uint64_t* from,
                         uint64_t* to, double* stnf, uint64_t capacity, uint64_t* n_edges, mdet_graph_stats* stats);
int mdet_tnf_graph_shard_dev(mdet_ctx* ctx, const float* d_tnf, const double* d_log_size, uint64_t n, double cutoff,
                             uint32_t max_edges, int mode, uint32_t shard, uint32_t nshards, uint64_t* d_from,
                             uint64_t* d_to, double* d_stnf, uint64_t capacity, uint64_t* n_edges,
                             mdet_graph_stats* stats);

/* Exact-stage distance and probability of m given pairs (no counterpart in
 * the reference as an entry point): the arithmetic of cal_tnf_pre_dist_d
 * (cuda/Cuda2.cu:192-241) and the sigmoid of get_tnf_graph2 (255) for
 * d_pairs[2p], d_pairs[2p+1] (contig indices < n), with no cutoff.  Device
 * buffers; d_dist or d_prob may be null.  For rescoring chosen pairs and for
 * stating the error against an FP64 evaluation. */
int mdet_tnf_pair_scores_dev(mdet_ctx* ctx, const float* d_tnf, const double* d_log_size, uint64_t n,
                             const uint64_t* d_pairs, uint64_t m, double* d_dist, double* d_prob);

/* ---- many assemblies in one pass -----------------------------------------
 * Replaces running gen_tnf_graph (cuda/Cuda2.cu:861-970) once per assembly:
 * every assembly's graph is computed with the same rules as
 * mdet_tnf_graph_dev (its own cutoff and max_edges, indices local to the
 * assembly), but the whole batch shares one tile list, one filter launch,
 * one exact-stage launch and one selection launch.  Device inputs and
 * outputs; max_edges <= 512; mode PLAIN or BF16.  Returns MDET_ERR_CAPACITY
 * when some assembly's capacity is short (that assembly's status says so and
 * its n_edges holds the count needed; the others are written). */
typedef struct {
    const float* d_tnf;        /* n x 136 TNF rows */
    const double* d_log_size;  /* n log10 sizes */
    uint64_t n;
    double cutoff;             /* in (0, 1) */
    uint32_t max_edges;        /* 1 .. 512 */
    int32_t status;            /* out */
    uint64_t* d_from;          /* outputs of `capacity` entries, from < to */
    uint64_t* d_to;
    double* d_stnf;
    uint64_t capacity;
    uint64_t n_edges;          /* out */
} mdet_assembly;

int mdet_tnf_graph_batched(mdet_ctx* ctx, mdet_assembly* assemblies, uint32_t count, int mode,
                           mdet_graph_stats* stats);
/* CUDA-graph recording of batched calls (on by default): after a batch has
 * run once, its whole device work -- preparation, d* tables, filter, exact
 * stage, selection, output -- is recorded as one CUDA graph with every count
 * kept on the device; a later call with the same sizes, cutoffs, max_edges,
 * buffers and capacities (the data may differ) replays it with one launch.
 * A replay whose candidates outgrow the recording falls back to the sized
 * path.  The recording is dropped when any scratch buffer of the context is
 * reallocated.  mdet_ctx_graph_replays counts replays. */
int mdet_ctx_set_graph_capture(mdet_ctx* ctx, int enable);
uint64_t mdet_ctx_graph_replays(mdet_ctx* ctx);

/* ---- abundance (coverage) side --------------------------------------------
 * The coverage matrices the reference reads from its abundance file into the
 * globals ABD (mean depth) and ABD_VAR (depth variance) (cuda/Cuda2.cu:
 * 1593-1700; float matrices there, cuda/Cuda2.cu:124-125): n x nabd,
 * row-major, widened to FP64, rows in the contig order of the TNF rows.  mdet_ctx_set_abundance copies them (host buffers) into the context;
 * abd == null or nabd == 0 clears them.  While they are set, mdet_tnf_graph
 * and mdet_tnf_graph_dev skip every pair of two contigs none of whose depths
 * exceeds 1 before the per-contig top-k (is_nz, cuda/Cuda2.cu:845-856, as
 * applied at 925), and fail with MDET_ERR_INVALID when called for a
 * different number of contigs.  The batched graph, the max-probability sample
 * and the pTNF search do not apply it (neither does the reference). */
int mdet_ctx_set_abundance(mdet_ctx* ctx, const double* abd, const double* abd_var, uint64_t n,
                           uint32_t nabd);

/* sTNF -> sSCR of a graph's edges (cuda/Cuda2.cu:1921-1971) with the
 * abundance set on the context: per edge, the mean of 1 - cal_abd_dist
 * (cuda/Cuda2.cu:667-719) over the nnz samples where either depth exceeds
 * min_cv; sTNF ranked ("min" ties) and, when nabd >= min_sample, the depth
 * correlation cal_abd_corr (cuda/Cuda2.cu:1219-1245) ranked ("max" ties,
 * cuda/ranker.h:56-80) are replaced by those quantiles of the sorted mean
 * similarities; sSCR = (s^(1-w) t^w c)^(1/2), or s^(1-w) t^w without the
 * correlation, with w = 1 / (1 + nnz).  Edge e joins to[e] and from[e]
 * (contig indices < n), taken in that order as the reference does.  Without
 * abundance on the context, sscr = stnf.  MDET_ERR_INVALID when an index is
 * out of range or an edge has no sample above min_cv (the reference would
 * divide 0 by 0).  min_cv, min_sample: the reference's minCV (default 1)
 * and minSample (default 3).  As in the reference, a contig whose depths are
 * the same in every sample makes its correlations undefined.  Accuracy: the
 * depth correlations, and so their ranks, are the reference's FP64 values
 * bit for bit; the similarities and the final sSCR are within 1e-12
 * (absolute or relative) of an FP64 evaluation (float-float normal CDFs,
 * crossing points and powers). */
int mdet_edges_sscr(mdet_ctx* ctx, const uint64_t* from, const uint64_t* to, const double* stnf,
                    uint64_t n_edges, double min_cv, uint32_t min_sample, double* sscr);
int mdet_edges_sscr_dev(mdet_ctx* ctx, const uint64_t* d_from, const uint64_t* d_to,
                        const double* d_stnf, uint64_t n_edges, double min_cv, uint32_t min_sample,
                        double* d_sscr);

/* ---- learned proposal (no counterpart in the reference) ----------------
 * A 136 -> 256 -> 128 -> 64 GELU network (BF16 weights, FP32 accumulation)
 * embeds each TNF row.  In MDET_MODE_LEARNED the graph orders contigs by
 * their embedding, scores a sample of rows against all columns exactly, sets
 * the margin tau from half of the sample's edges (embedded distances), skips
 * tile pairs whose embedded distance bound exceeds tau, measures the recall
 * of the kept tiles on the other half and falls back to the all-pairs form
 * below target; kept tiles are scored exactly (tensor-core filter + exact
 * stage), so every emitted edge is exact. */
typedef struct mdet_mlp mdet_mlp;

typedef struct {
    uint64_t pairs;            /* training pair pool (0: 50,000,000) */
    double candidate_fraction; /* share of the pool drawn from the distance filter's candidates */
    double label_cutoff;       /* edge labels: exact probability above this cutoff (0.7) */
    uint64_t steps;            /* optimiser steps (0: none -- only the input scaling and tau are set) */
    uint32_t batch_pairs;      /* pairs per step (0: 8192) */
    float lr, m_pos, m_neg;    /* Adam learning rate; contrastive margins of edges / non-edges */
    double tau_quantile;       /* quantile of held-out edge distances that sets tau (0: 0.9995) */
    uint64_t seed;
} mdet_train_params;

typedef struct {
    uint64_t steps, pairs, candidate_pairs, held_pos, held_neg;
    double final_loss, tau, pos_median, neg_median, neg_below_tau;
} mdet_train_report;

typedef struct {
    double recall_target;      /* fall back to all pairs below this estimated recall (0: 0.999) */
    uint32_t recall_rows;      /* rows sampled to calibrate tau and estimate recall (0: 2048) */
    uint32_t segment;          /* order 0: contigs per size-sorted run of the embedding order (0: 1024;
                                  1: none); order 1: contigs per size band (0: 16384) */
    double recall;             /* out: estimated edge recall of the learned graph */
    uint32_t fell_back;        /* out: 1 when the all-pairs graph was returned */
    uint32_t order;            /* 0: embedding-major Morton order (7 principal axes + log size);
                                  1: size-major (size bands, 8 principal axes within a band) */
    uint64_t tiles_skipped;    /* out: 128 x 256 tiles skipped */
    double tau;                /* out: embedded-distance margin used */
    double ms_embed, ms_order, ms_sample; /* out: network pass; order + row preparation; sampled-row
                                  calibration, tile flags and recall estimate (device time) */
    double tau_quantile;       /* quantile of the calibration edges' embedded distances that sets tau
                                  (0: 1 - (1 - recall_target) / 4); lower skips more tiles and may lose
                                  edges, down to the recall target */
} mdet_learned_report;

int mdet_mlp_create(mdet_ctx* ctx, uint64_t seed, mdet_mlp** out);
int mdet_mlp_destroy(mdet_mlp* mlp);
uint64_t mdet_mlp_param_count(void);
int mdet_mlp_get_params(mdet_ctx* ctx, const mdet_mlp* mlp, float* host, uint64_t count);
int mdet_mlp_set_params(mdet_ctx* ctx, mdet_mlp* mlp, const float* host, uint64_t count);
int mdet_mlp_embed_dev(mdet_ctx* ctx, const mdet_mlp* mlp, const float* d_tnf, uint64_t n, float* d_out);
/* Mean contrastive loss and its gradient over host rows x (rows x 136 TNF),
 * pairs[2p], pairs[2p+1] indexing x -- for checking the backward kernels. */
int mdet_mlp_grad(mdet_ctx* ctx, const mdet_mlp* mlp, const float* x, uint64_t rows, const uint32_t* pairs,
                  const float* labels, uint64_t n_pairs, float m_pos, float m_neg, float* grad_out,
                  double* loss_out);
int mdet_mlp_train(mdet_ctx* ctx, mdet_mlp* mlp, const float* d_tnf, const double* d_log_size, uint64_t n,
                   const mdet_train_params* params, mdet_train_report* report);
/* Network (and options) used by MDET_MODE_LEARNED calls of this context;
 * report may be null; the context keeps both pointers. */
int mdet_ctx_set_learned(mdet_ctx* ctx, const mdet_mlp* mlp, mdet_learned_report* report);

/* ---- dissolving small bins, recruiting leftover and small contigs -------
 * Replaces the block of main after label propagation (cuda/Cuda2.cu:
 * 2064-2283): the large contigs are grouped into bins by label[i] (members in
 * ascending index); a bin whose sizes sum below min_cls_size is dissolved and
 * its members become leftovers.  Depth rows are replaced by their average
 * ranks (Spearman), every bin with at least 10 members gets the mean pairwise
 * depth correlation of its members, and a leftover (a small contig, against
 * the small contigs' own depths) joins a bin when its mean correlation with
 * the bin's first 10 members, and then with all of them, reaches the bin's
 * mean -- and only when exactly one bin accepts it.  Leftover recruits are
 * kept when their bases are under 10 % of the binned bases, small-contig
 * recruits when theirs are under 15 % of small_total (pass the reference's
 * totalSize1: it sums the small contigs' sizes only with --verbose, and 0
 * rejects every small recruit).  abd (n x nabd) and small_abd (n_small x
 * nabd) are the reference's ABD and small_ABD (float, row-major; 1 <= nabd
 * <= 256); they are not modified.  out[i]: the bin label of large contig i
 * afterwards, -1 if it has none; small_out[s] likewise.  n + n_small must
 * be below 2^32 - 1.  The reference dissolves small bins in every run but
 * recruits only when !noAdd and nABD >= minSample; this call does both, so
 * in the other runs a caller keeps the reference's dissolving loop
 * (cuda/Cuda2.cu:2081-2101) and does not call it. */
typedef struct {
    uint64_t n_bins;              /* bins kept (sizes sum to >= min_cls_size) */
    uint64_t n_bins_scored;       /* kept bins with >= 10 members: the ones that recruit */
    uint64_t n_leftovers;         /* large contigs of dissolved bins */
    uint64_t n_leftovers_matched; /* leftovers exactly one bin accepts */
    uint64_t n_small_matched;     /* small contigs exactly one bin accepts */
    uint64_t binned_bases, leftover_bases, small_bases;
    int leftovers_accepted, small_accepted; /* the 10 % and 15 % gates */
    uint64_t pairs_tested;        /* (contig, scored bin) pairs */
    uint64_t pairs_exact;         /* of those, the ones the FP32 prefilter left to the exact FP64 test */
    uint64_t pairs_undecided;     /* of those, tests within the error bound of a bin's estimated mean */
    uint64_t bins_exact;          /* bins whose exact mean was computed (degenerate rows, undecided tests) */
} mdet_recruit_stats;
int mdet_recruit(mdet_ctx* ctx, const float* abd, const float* small_abd, uint64_t n, uint64_t n_small,
                 uint32_t nabd, const int64_t* label, const uint64_t* sizes, const uint64_t* small_sizes,
                 uint64_t min_cls_size, uint64_t small_total, int64_t* out, int64_t* small_out,
                 mdet_recruit_stats* stats);

/* ---- binning by label propagation --------------------------------------
 * Replaces the traversal of the scored edges in main (cuda/Cuda2.cu:
 * 1980-2061) and label_propagation (cuda/Cuda2.cu:569-656).  Edge e joins
 * to[e] and from[e] (contigs < n) with score sscr[e] in [0, 1] (the
 * reference's g.to, g.from, g.sSCR).  Edges are taken in decreasing score --
 * equal scores in edge order, where the reference's std::sort leaves their
 * order open.  An edge whose contigs are in different bins connects them and,
 * when its score is above min_s, joins the traversal graph; the first such
 * edge at or below min_s ends the traversal.  Label propagation runs each
 * time the connected share of the contigs reaches max_p/10 * (1..10) and at
 * the last edge (at most 10 runs): Gauss-Seidel sweeps in first-seen order,
 * each contig taking the neighbour label with the largest chi-squared CDF of
 * -2 * sum log(1 - score) (2 x count degrees of freedom), exact ties going to
 * the label first in the reference's std::unordered_map iteration order
 * (GNU libstdc++); a contig that returns to a label it held in the same run
 * is frozen; a run stops when no contig moved to a new label, or after 10
 * sweeps without a new low.  max_p and min_s are fractions (the reference's
 * --maxP and --minS divided by 100).  The CDF and log(1 - score) are this
 * project's (bit-identical host and device functions; the reference calls
 * Boost's CDF and the C library's log).  mem[i] receives contig i's bin (a
 * contig index).  n < 2^31, n_edges < 2^30. */
typedef struct {
    uint64_t calls;       /* label propagation runs */
    uint64_t sweeps;      /* Gauss-Seidel sweeps, summed over runs */
    uint64_t graph_edges; /* edges in the traversal graph */
    uint64_t connected;   /* contigs in the first-seen order */
    uint64_t frozen;      /* contigs frozen, summed over runs */
    uint64_t ties;        /* evaluations decided among exactly tied labels (a contig none of whose
                             neighbours changed label since its last evaluation is not evaluated
                             again: the same label would win) */
    uint64_t levels_max;  /* most dependency levels of a sweep */
    uint64_t degree_max;  /* most traversal-graph edges of a contig */
    double ms_total;      /* device time of the call */
} mdet_lp_stats;
int mdet_label_propagation(mdet_ctx* ctx, const uint64_t* from, const uint64_t* to, const double* sscr,
                           uint64_t n_edges, uint64_t n, double max_p, double min_s, uint64_t* mem,
                           mdet_lp_stats* stats);
int mdet_label_propagation_dev(mdet_ctx* ctx, const uint64_t* d_from, const uint64_t* d_to, const double* d_sscr,
                               uint64_t n_edges, uint64_t n, double max_p, double min_s, uint64_t* d_mem,
                               mdet_lp_stats* stats);

#ifdef __cplusplus
}
#endif
#endif
