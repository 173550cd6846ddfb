/*
 * tnf_oracle.h -- CPU oracle for the MetaBAT2 TNF path of MdeT.
 *
 * TEST INFRASTRUCTURE ONLY.  This library restates, in plain C++, the
 * reference's own CPU/GPU arithmetic for the TNF hot path so that the CUDA
 * product can be checked against it.  Only tests/, __graft_entry__.smoke() and
 * bench.py's CPU-baseline leg may load it; the product never calls it.
 *
 * Every function cites the reference file:line it follows (paths relative to
 * the MdeT project root).
 */
#ifndef MDET_TNF_ORACLE_H
#define MDET_TNF_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* 136-entry canonical tetranucleotide order (the TNF.bin column order,
 * openmp/TNF.cpp:14-24) as a 136*4 character block. */
const char* orc_tn_order(void);

/* Raw 8-bit 4-mer code -> canonical column (cuda/Cuda2.cu:149-159), derived
 * from the column order and reverse complements. */
void orc_tnmap(uint8_t map[256]);

/* ASCII -> 2-bit base code, 4 = not a base (cuda/Cuda2.cu:162-168). */
void orc_base_code(uint8_t bn[256]);

/* Per-contig TNF counting + normalisation with the reference host loop's
 * semantics (cuda/Cuda2.cu:1825-1853, get_tn/next_contig 317-339).
 * bytes[off[i] .. off[i]+len[i]) is the contig's sequence view, newlines
 * included.  counts: n*136 uint32, tnf: n*136 float (float(c / rsum) with
 * rsum = sqrt(sum(float(c*c))) accumulated in double).  threads<=0: all. */
void orc_tnf_count(const char* bytes, const uint64_t* off, const uint64_t* len, uint64_t n,
                   uint32_t* counts, float* tnf, int threads);

/* TNF.cpp normalisation (openmp/TNF.cpp:207-218): c / sqrt(sum c^2), FP64. */
void orc_tnf_normalize_f64(const uint32_t* counts, uint64_t n, double* out);

/* cal_tnf_pre_dist_d (cuda/Cuda2.cu:192-241), FP64, GPU evaluation order. */
double orc_pre_prob(double r1, double r2, const float* a, const float* b);

/* Distance part only: sqrt(sum_k double(float((a_k-b_k)^2))) (cuda/Cuda2.cu:193-197). */
double orc_tnf_distance(const float* a, const float* b);

/* The logistic model given a distance (cuda/Cuda2.cu:199-240). */
double orc_pre_prob_from_d(double r1, double r2, double d);

/* cal_tnf_dist (cuda/Cuda2.cu:721-779): host-order probability that the two
 * contigs differ; similarity = 1 - result. */
double orc_tnf_dist_cpu(double r1, double r2, const float* a, const float* b);

/* logit(cutoff) as gen_tnf_graph computes it (cuda/Cuda2.cu:884). */
double orc_logit_cutoff(double cutoff);

/* Distance and probability of m given pairs (index pairs, 2m entries). */
void orc_pair_scores(const float* tnf, const double* logsize, const uint64_t* pairs, uint64_t m, double* dist,
                     double* prob, int threads);

/* gen_tnf_graph for rows [row0,row1) against all n columns
 * (cuda/Cuda2.cu:861-946, kernel get_tnf_graph2 243-262).  Per row a
 * std::priority_queue min-heap of size max_edges with the reference's strict
 * replacement rule; emits (i, j, sTNF) for i < j only.  Rows are emitted in
 * ascending i; inside a row in heap-pop order (ascending similarity).
 * Returns the edge count; writes at most cap edges. */
uint64_t orc_tnf_graph(const float* tnf, const double* logsize, uint64_t n, double cutoff,
                       uint32_t max_edges, uint64_t row0, uint64_t row1, uint64_t* from,
                       uint64_t* to, double* stnf, uint64_t cap, int threads);

/* Like orc_tnf_graph but returns each row's full top-k (both j<i and j>i),
 * CSR style: row_ptr[row1-row0+1], cols, sims.  Used to judge tolerance
 * bands around the per-row top-k cutoff. Returns total entries. */
uint64_t orc_tnf_topk_rows(const float* tnf, const double* logsize, uint64_t n, double cutoff,
                           uint32_t max_edges, uint64_t row0, uint64_t row1, uint64_t* row_ptr,
                           uint64_t* cols, double* sims, uint64_t cap, int threads);

/* orc_tnf_graph / orc_tnf_topk_rows with the abundance pair gate: low
 * (optional, n entries) marks contigs none of whose depths exceeds 1, and a
 * pair of two such contigs is skipped (is_nz, cuda/Cuda2.cu:845-856, 925). */
uint64_t orc_tnf_graph_nz(const float* tnf, const double* logsize, uint64_t n, double cutoff,
                          uint32_t max_edges, uint64_t row0, uint64_t row1, uint64_t* from,
                          uint64_t* to, double* stnf, uint64_t cap, int threads, const uint8_t* low);
uint64_t orc_tnf_topk_rows_nz(const float* tnf, const double* logsize, uint64_t n, double cutoff,
                              uint32_t max_edges, uint64_t row0, uint64_t row1, uint64_t* row_ptr,
                              uint64_t* cols, double* sims, uint64_t cap, int threads,
                              const uint8_t* low);

/* get_tnf_max_prob_sample (cuda/Cuda2.cu:281-314) for sampled positions
 * [0, m) of the permutation `contigs` (length n): for each sampled contig,
 * sigmoid of the max pre-probability over all other contigs, local max
 * seeded with DBL_MIN. */
void orc_max_prob(const float* tnf, const double* logsize, uint64_t n, const uint64_t* contigs,
                  uint64_t m, double* out, int threads);

/* glibc srand/rand wrappers so tests drive the same generator the
 * reference's host uses (cuda/Cuda2.cu:1311-1312). */
void orc_srand(uint32_t seed);
int orc_rand(void);

/* gen_tnf_graph_sample + driver (cuda/Cuda2.cu:972-1025, 1883-1904) with
 * orc_max_prob as the kernel; consumes rand() in the reference's order.
 * coverage = maxP/100.  Returns pTNF in permille (as a double, like the
 * reference's `pTNF` variable after the driver). */
double orc_ptnf_search(const float* tnf, const double* logsize, uint64_t n, double coverage,
                       int threads);

/* Abundance: abd, var are n x nabd row-major (mean depth and variance of
 * contig r in sample i, the reference's ABD / ABD_VAR).
 * orc_abd_low: low[r] = 1 when no depth of contig r exceeds 1 (is_nz,
 * cuda/Cuda2.cu:845-856). */
void orc_abd_low(const double* abd, uint64_t n, uint32_t nabd, uint8_t* low);

/* sTNF -> sSCR of the edges (cuda/Cuda2.cu:1921-1971, with cal_abd_dist
 * 667-719, cal_abd_corr 1219-1245 and rank, cuda/ranker.h:56-80).  Edge e
 * joins to[e] and from[e]; min_cv is the reference's minCV, min_sample its
 * minSample (the correlation term is used when nabd >= min_sample).
 * nabd == 0 copies sTNF. */
void orc_sscr(const uint64_t* from, const uint64_t* to, const double* stnf, uint64_t ne, const double* abd,
              const double* var, uint32_t nabd, double min_cv, uint32_t min_sample, double* sscr,
              int threads);

/* The reference reader's record split (cuda/Cuda2.cu:1507-1544), taken
 * sequentially: every record (no size classes) with its sequence view
 * (offset, length: inner newlines kept, one trailing newline dropped), its
 * size (bases: view bytes before the drop minus newlines) and its name (after
 * '>', cut at the first space).  Returns the record count; writes <= cap. */
uint64_t orc_fasta_index(const char* b, uint64_t nbytes, uint64_t cap, uint64_t* seq_off, uint64_t* seq_len,
                         uint64_t* size, uint64_t* name_off, uint32_t* name_len);

/* Label propagation: the binning traversal of the scored edges and its
 * propagation calls (cuda/Cuda2.cu:569-656, 1980-2061); see tnf_oracle.cpp. */
void orc_label_prop(const uint64_t* from, const uint64_t* to, const double* sscr, uint64_t ne, uint64_t n,
                    double max_p, double min_s, uint64_t* mem_out, uint64_t* stats);
void orc_umap_order(const uint64_t* keys, uint64_t k, uint64_t* out);
double orc_lp_log(double x);
double orc_lp_exp(double x);
double orc_lp_chi2_cdf(uint64_t count, double x);

#ifdef __cplusplus
}
#endif
#endif
