/*
 * tnf_oracle.cpp -- CPU oracle for MdeT's MetaBAT2 TNF path.
 *
 * TEST INFRASTRUCTURE ONLY: loaded by tests/, __graft_entry__.smoke() and the
 * CPU-baseline leg of bench.py, never by the product.  It restates the
 * reference's arithmetic so the CUDA kernels can be checked; each function
 * names the reference lines it follows.  Built with -ffp-contract=off so the
 * FP64 expressions are evaluated term by term as written in the reference.
 *
 * Pinning: the counting half is pinned against TNF.bin files written by the
 * unmodified openmp/TNF.cpp (tests/golden/), the canonical-index table against
 * the reference's TNmap_d/BN tables (tests/golden/ref_tables.json).  The
 * probability half is a line-by-line restatement of cuda/Cuda2.cu:192-241 and
 * 721-779; it is pinned bit for bit to those two reference functions, cut out
 * of the reference sources and compiled on the host by oracle/build_ref.py,
 * on the fixture tests/golden/prob_golden.npz (tests/test_oracle.py).  The
 * selection rules (per-row heap, strict '>', i<j emission) are a restatement
 * only: the reference's gen_tnf_graph needs Boost and a GPU.
 */
#include "tnf_oracle.h"

#include <algorithm>
#include <map>
#include <cfloat>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <numeric>
#include <queue>
#include <utility>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

/* Column order of the 136 canonical tetranucleotides: the TNF.bin format
 * (openmp/TNF.cpp:14-24).  The order is the file format, so it is kept. */
const char kTnOrder[] =
    "GGTAAGCCAAAAACATAGTCACGACATACGAAAAGTCAAACCAGGGACATTAGATCCCTCCTAAACTAAGGCGCAACCGCCGCCAAAC"
    "ACTCATCCGACCGAGAATAGATCACAGAAGTAATGAAAATTTAATATAAGTGAGCTCCACGGCCACCCGGGAGCGCATACCTGATAGA"
    "ATATGTCACTCCACAAACCTTAAAAACGCGAGAGGGATCGACGCTCAACTACCTCAGACAGGAACTTCGCCCCTGCTGCAGGCACACG"
    "GAGCAACTCATGAATTACAGAGATATAACATCGCCATCGACACACAACAAGGAGCAATGGATTCGTGAACCGGATAGCTACGTCCCCG"
    "AAGCCGTAGTACAGGAAATGCACCCAGCCGGCACACCCGGCCGACCCCTGAAAACAAGAGCCCACGGATACAACCAACGTGAACGTAA"
    "ATGCGTTATCCACAGGACTGAAAGAAGACAAGGCGAAACCACGGCCAACTTAAGACAGCGGAAAAATCATTGGCACCCTACGACCTAG"
    "AGAACGCACGCGAATA";

/* ASCII -> 2-bit code used by the reference's get_tn (cuda/Cuda2.cu:162-168):
 * A/a=0, C/c=1, T/t=2, G/g=3, anything else 4. */
inline uint8_t base_code(unsigned char c) {
    switch (c) {
        case 'A': case 'a': return 0;
        case 'C': case 'c': return 1;
        case 'T': case 't': return 2;
        case 'G': case 'g': return 3;
        default: return 4;
    }
}

const char kCodeBase[4] = {'A', 'C', 'T', 'G'};

char complement(char b) {
    switch (b) {
        case 'A': return 'T';
        case 'T': return 'A';
        case 'C': return 'G';
        default: return 'C';
    }
}

struct TnTables {
    uint8_t map[256];
    TnTables() {
        for (int code = 0; code < 256; ++code) {
            char s[4], rc[4];
            for (int p = 0; p < 4; ++p) s[p] = kCodeBase[(code >> (2 * (3 - p))) & 3];
            for (int p = 0; p < 4; ++p) rc[p] = complement(s[3 - p]);
            int idx = -1;
            for (int t = 0; t < 136 && idx < 0; ++t) {
                if (memcmp(kTnOrder + 4 * t, s, 4) == 0 || memcmp(kTnOrder + 4 * t, rc, 4) == 0) idx = t;
            }
            map[code] = (uint8_t)(idx < 0 ? 255 : idx);
        }
    }
};

const TnTables& tables() {
    static TnTables t;
    return t;
}

/* Logistic-model coefficients of MetaBAT2 (cuda/Cuda2.cu:170-188); these are
 * the model's parameters and must be identical. */
const double B1[18] = {46349.1624324381,  -76092.3748553155, -639.918334183,  53873.3933743949, -156.6547554844,
                       -21263.6010657275, 64.7719132839,     5003.2646455284, -8.5014386744,    -700.5825500292,
                       0.3968284526,      54.037542743,      -1.7713972342,   474.0850141891,   -23.966597785,
                       0.7800219061,      -0.0138723693,     0.0001027543};
const double C1[18] = {-443565.465710869, 718862.10804858, 5114.1630934534,   -501588.206183097, 784.4442123743,
                       194712.394138513,  -377.9645994741, -45088.7863182741, 50.5960513287,     6220.3310639927,
                       -2.3670776453,     -473.269785487,  15.3213264134,     -3282.8510348085,  164.0438603974,
                       -5.2778800755,     0.0929379305,    -0.0006826817};
const double B2[17] = {6770.9351457442, -5933.7589419767, -2976.2879986855, 3279.7524685865, 1602.7544794819,
                       -967.2906583423, -462.0149190219,  159.8317289682,   74.4884405822,   -14.0267151808,
                       -6.3644917671,   0.5108811613,     0.2252455343,     0.965040193,     -0.0546309127,
                       0.0012917084,    -1.14383e-05};
const double C2[19] = {39406.5712626297,  -77863.1741143294, 9586.8761567725, 55360.1701572325, -5825.2491611377,
                       -21887.8400068324, 1751.6803621934,   5158.3764225203, -290.1765894829,  -724.0348081819,
                       25.364646181,      56.0522105105,     -0.9172073892,   -1.8470088417,    449.4660736502,
                       -24.4141920625,    0.8465834103,      -0.0158943762,   0.0001235384};
const double kFloorPreProb = 2.1972245773362196; /* log(9), cuda/Cuda2.cu:190 */

int resolve_threads(int threads) {
#ifdef _OPENMP
    return threads > 0 ? threads : omp_get_max_threads();
#else
    (void)threads;
    return 1;
#endif
}

/* One row of gen_tnf_graph: visit columns in ascending order and keep the
 * reference's per-row min-heap (cuda/Cuda2.cu:921-934, CompareEdge 660-664). */
struct CompareEdge {
    bool operator()(const std::pair<uint64_t, double>& a, const std::pair<uint64_t, double>& b) const {
        return a.second > b.second;
    }
};
typedef std::priority_queue<std::pair<uint64_t, double>, std::vector<std::pair<uint64_t, double>>, CompareEdge> EdgeHeap;

/* low (optional): per contig 1 when none of its depths exceeds 1; a pair of
 * two such contigs is skipped before the heap (is_nz, cuda/Cuda2.cu:845-856,
 * applied at 925). */
void row_heap(const float* tnf, const double* logsize, uint64_t n, double floor_cut, uint32_t max_edges, uint64_t i,
              EdgeHeap& heap, const uint8_t* low) {
    const float* ti = tnf + i * 136;
    for (uint64_t j = 0; j < n; ++j) {
        if (i == j) continue;
        if (low && low[i] && low[j]) continue;
        double pre = orc_pre_prob(logsize[i], logsize[j], ti, tnf + j * 136);
        double s = pre > floor_cut ? 1. - 1. / (1. + exp(pre)) : 0.;
        if (s != 0. && (heap.size() < max_edges || (heap.size() == max_edges && s > heap.top().second))) {
            if (heap.size() == max_edges) heap.pop();
            heap.push(std::make_pair(j, s));
        }
    }
}

}  // namespace

extern "C" {

const char* orc_tn_order(void) { return kTnOrder; }

void orc_tnmap(uint8_t map[256]) { memcpy(map, tables().map, 256); }

void orc_base_code(uint8_t bn[256]) {
    for (int c = 0; c < 256; ++c) bn[c] = base_code((unsigned char)c);
}

/* cuda/Cuda2.cu:1830-1853 with next_contig (330-339) and get_tn (317-327):
 * a rolling 4-char window; '\n' overwrites the window's oldest char with a
 * non-base marker instead of shifting, so the k-mer that spans a line break
 * is still counted; any non-ACGT char skips the windows containing it. */
void orc_tnf_count(const char* bytes, const uint64_t* off, const uint64_t* len, uint64_t n, uint32_t* counts,
                   float* tnf, int threads) {
    const uint8_t* map = tables().map;
    int nt = resolve_threads(threads);
    (void)nt;
#pragma omp parallel for schedule(dynamic, 64) num_threads(nt)
    for (int64_t r = 0; r < (int64_t)n; ++r) {
        const unsigned char* seq = (const unsigned char*)bytes + off[r];
        uint64_t L = len[r];
        unsigned char win[4] = {0, 0, 0, 0};
        float cnt[136];
        for (int c = 0; c < 136; ++c) cnt[c] = 0.f;
        if (L >= 4) {
            for (uint64_t j = 0; j < L; ++j) {
                unsigned char ch = seq[j];
                if (ch == '\n') {
                    win[0] = 'X';
                } else {
                    win[0] = win[1];
                    win[1] = win[2];
                    win[2] = win[3];
                    win[3] = ch;
                }
                if (j < 3) continue;
                int tn = 0, bad = 0;
                for (int p = 0; p < 4; ++p) {
                    uint8_t b = base_code(win[p]);
                    if (b & 4) { bad = 1; break; }
                    tn = (tn << 2) | b;
                }
                if (bad) continue;
                cnt[map[tn]] += 1.f;
            }
        }
        double rsum = 0;
        for (int c = 0; c < 136; ++c) {
            float sq = cnt[c] * cnt[c];
            rsum += sq;
        }
        rsum = sqrt(rsum);
        for (int c = 0; c < 136; ++c) {
            counts[r * 136 + c] = (uint32_t)cnt[c];
            tnf[r * 136 + c] = (float)(cnt[c] / rsum);
        }
    }
}

void orc_tnf_normalize_f64(const uint32_t* counts, uint64_t n, double* out) {
    for (uint64_t r = 0; r < n; ++r) {
        double rsum = 0;
        for (int c = 0; c < 136; ++c) rsum += (double)counts[r * 136 + c] * (double)counts[r * 136 + c];
        rsum = sqrt(rsum);
        for (int c = 0; c < 136; ++c) out[r * 136 + c] = (double)counts[r * 136 + c] / rsum;
    }
}

double orc_tnf_distance(const float* a, const float* b) {
    double d = 0;
    for (int k = 0; k < 136; ++k) {
        float df = a[k] - b[k];
        float sq = df * df;
        d += sq;
    }
    return sqrt(d);
}

/* cuda/Cuda2.cu:199-240: powers of x = min(log sizes), y = max(log sizes),
 * model 1; if its pre-probability is at or below log(9) model 2, capped at
 * log(9). */
double orc_pre_prob_from_d(double r1, double r2, double d) {
    double lw[19];
    lw[0] = std::min(r1, r2);
    lw[1] = std::max(r1, r2);
    lw[2] = lw[0] * lw[0];
    lw[4] = lw[2] * lw[0];
    lw[6] = lw[4] * lw[0];
    lw[8] = lw[6] * lw[0];
    lw[10] = lw[8] * lw[0];
    lw[11] = lw[10] * lw[0];
    lw[3] = lw[1] * lw[1];
    lw[5] = lw[3] * lw[1];
    lw[7] = lw[5] * lw[1];
    lw[9] = lw[7] * lw[1];
    lw[12] = lw[0] * lw[1];
    lw[14] = lw[4] * lw[5];
    lw[15] = lw[6] * lw[7];
    lw[16] = lw[8] * lw[9];
    lw[13] = lw[2] * lw[3];
    lw[18] = lw[9] * lw[1];
    double b = B1[0] + B1[1] * lw[0] + B1[2] * lw[1] + B1[3] * lw[2] + B1[4] * lw[3] + B1[5] * lw[4] + B1[6] * lw[5] +
               B1[7] * lw[6] + B1[8] * lw[7] + B1[9] * lw[8] + B1[10] * lw[9] + B1[11] * lw[10] + B1[12] * lw[11] +
               B1[13] * lw[12] + B1[14] * lw[13] + B1[15] * lw[14] + B1[16] * lw[15] + B1[17] * lw[16];
    double c = C1[0] + C1[1] * lw[0] + C1[2] * lw[1] + C1[3] * lw[2] + C1[4] * lw[3] + C1[5] * lw[4] + C1[6] * lw[5] +
               C1[7] * lw[6] + C1[8] * lw[7] + C1[9] * lw[8] + C1[10] * lw[9] + C1[11] * lw[10] + C1[12] * lw[11] +
               C1[13] * lw[12] + C1[14] * lw[13] + C1[15] * lw[14] + C1[16] * lw[15] + C1[17] * lw[16];
    double pre = -(b + c * d);
    if (pre <= kFloorPreProb) {
        b = B2[0] + B2[1] * lw[0] + B2[2] * lw[1] + B2[3] * lw[2] + B2[4] * lw[3] + B2[5] * lw[4] + B2[6] * lw[5] +
            B2[7] * lw[6] + B2[8] * lw[7] + B2[9] * lw[8] + B2[10] * lw[9] + B2[11] * lw[10] + B2[12] * lw[18] +
            B2[13] * lw[13] + B2[14] * lw[14] + B2[15] * lw[15] + B2[16] * lw[16];
        c = C2[0] + C2[1] * lw[0] + C2[2] * lw[1] + C2[3] * lw[2] + C2[4] * lw[3] + C2[5] * lw[4] + C2[6] * lw[5] +
            C2[7] * lw[6] + C2[8] * lw[7] + C2[9] * lw[8] + C2[10] * lw[9] + C2[11] * lw[10] + C2[12] * lw[18] +
            C2[13] * lw[11] + C2[14] * lw[12] + C2[15] * lw[13] + C2[16] * lw[14] + C2[17] * lw[15] + C2[18] * lw[16];
        pre = -(b + c * d);
        if (pre > kFloorPreProb) pre = kFloorPreProb;
    }
    return pre;
}

double orc_pre_prob(double r1, double r2, const float* a, const float* b) {
    return orc_pre_prob_from_d(r1, r2, orc_tnf_distance(a, b));
}

/* cuda/Cuda2.cu:721-779, the host form with its own grouping. */
double orc_tnf_dist_cpu(double r1, double r2, const float* a, const float* bb) {
    const double floor_prob = 0.1;
    const double floor_pre = log((1.0 / floor_prob) - 1.0);
    double d = 0;
    for (int i = 0; i < 136; ++i) {
        float df = a[i] - bb[i];
        float sq = df * df;
        d += sq;
    }
    d = sqrt(d);
    double lw11 = std::min(r1, r2), lw21 = std::max(r1, r2);
    double lw12 = lw11 * lw11, lw13 = lw12 * lw11, lw14 = lw13 * lw11, lw15 = lw14 * lw11, lw16 = lw15 * lw11,
           lw17 = lw16 * lw11;
    double lw22 = lw21 * lw21, lw23 = lw22 * lw21, lw24 = lw23 * lw21, lw25 = lw24 * lw21, lw26 = lw25 * lw21;
    double b = 46349.1624324381 + -76092.3748553155 * lw11 + -639.918334183 * lw21 + 53873.3933743949 * lw12 +
               -156.6547554844 * lw22 + -21263.6010657275 * lw13 + 64.7719132839 * lw23 + 5003.2646455284 * lw14 +
               -8.5014386744 * lw24 + -700.5825500292 * lw15 + 0.3968284526 * lw25 + 54.037542743 * lw16 +
               -1.7713972342 * lw17 + 474.0850141891 * lw11 * lw21 + -23.966597785 * lw12 * lw22 +
               0.7800219061 * lw13 * lw23 + -0.0138723693 * lw14 * lw24 + 0.0001027543 * lw15 * lw25;
    double c = -443565.465710869 + 718862.10804858 * lw11 + 5114.1630934534 * lw21 + -501588.206183097 * lw12 +
               784.4442123743 * lw22 + 194712.394138513 * lw13 + -377.9645994741 * lw23 + -45088.7863182741 * lw14 +
               50.5960513287 * lw24 + 6220.3310639927 * lw15 + -2.3670776453 * lw25 + -473.269785487 * lw16 +
               15.3213264134 * lw17 + -3282.8510348085 * lw11 * lw21 + 164.0438603974 * lw12 * lw22 +
               -5.2778800755 * lw13 * lw23 + 0.0929379305 * lw14 * lw24 + -0.0006826817 * lw15 * lw25;
    double pre = -(b + c * d);
    double prob = pre <= floor_pre ? floor_prob : 1.0 / (1 + exp(pre));
    if (prob >= floor_prob) {
        b = 6770.9351457442 + -5933.7589419767 * lw11 + -2976.2879986855 * lw21 + 3279.7524685865 * lw12 +
            1602.7544794819 * lw22 + -967.2906583423 * lw13 + -462.0149190219 * lw23 + 159.8317289682 * lw14 +
            74.4884405822 * lw24 + -14.0267151808 * lw15 + -6.3644917671 * lw25 + 0.5108811613 * lw16 +
            0.2252455343 * lw26 + 0.965040193 * lw12 * lw22 + -0.0546309127 * lw13 * lw23 +
            0.0012917084 * lw14 * lw24 + -1.14383e-05 * lw15 * lw25;
        c = 39406.5712626297 + -77863.1741143294 * lw11 + 9586.8761567725 * lw21 + 55360.1701572325 * lw12 +
            -5825.2491611377 * lw22 + -21887.8400068324 * lw13 + 1751.6803621934 * lw23 + 5158.3764225203 * lw14 +
            -290.1765894829 * lw24 + -724.0348081819 * lw15 + 25.364646181 * lw25 + 56.0522105105 * lw16 +
            -0.9172073892 * lw26 + -1.8470088417 * lw17 + 449.4660736502 * lw11 * lw21 +
            -24.4141920625 * lw12 * lw22 + 0.8465834103 * lw13 * lw23 + -0.0158943762 * lw14 * lw24 +
            0.0001235384 * lw15 * lw25;
        pre = -(b + c * d);
        prob = pre <= floor_pre ? 1.0 / (1 + exp(pre)) : floor_prob;
    }
    return prob;
}

double orc_logit_cutoff(double cutoff) { return log((1.0 / (1. - cutoff)) - 1.0); }

/* Distance and probability of given pairs (pairs[2p], pairs[2p+1]):
 * cuda/Cuda2.cu:192-241 for the pre-probability, sigmoid as at 255. */
void orc_pair_scores(const float* tnf, const double* logsize, const uint64_t* pairs, uint64_t m, double* dist,
                     double* prob, int threads) {
    int nt = resolve_threads(threads);
    (void)nt;
#pragma omp parallel for schedule(static) num_threads(nt)
    for (int64_t p = 0; p < (int64_t)m; ++p) {
        const uint64_t i = pairs[2 * p], j = pairs[2 * p + 1];
        const double d = orc_tnf_distance(tnf + i * 136, tnf + j * 136);
        const double pre = orc_pre_prob_from_d(logsize[i], logsize[j], d);
        dist[p] = d;
        prob[p] = 1. - 1. / (1. + exp(pre));
    }
}

uint64_t orc_tnf_graph(const float* tnf, const double* logsize, uint64_t n, double cutoff, uint32_t max_edges,
                       uint64_t row0, uint64_t row1, uint64_t* from, uint64_t* to, double* stnf, uint64_t cap,
                       int threads) {
    return orc_tnf_graph_nz(tnf, logsize, n, cutoff, max_edges, row0, row1, from, to, stnf, cap, threads, nullptr);
}

uint64_t orc_tnf_graph_nz(const float* tnf, const double* logsize, uint64_t n, double cutoff, uint32_t max_edges,
                          uint64_t row0, uint64_t row1, uint64_t* from, uint64_t* to, double* stnf, uint64_t cap,
                          int threads, const uint8_t* low) {
    if (row1 > n) row1 = n;
    if (row0 >= row1) return 0;
    const double floor_cut = orc_logit_cutoff(cutoff);
    uint64_t nr = row1 - row0;
    std::vector<std::vector<std::pair<uint64_t, double>>> per_row(nr);
    int nt = resolve_threads(threads);
    (void)nt;
#pragma omp parallel for schedule(dynamic, 1) num_threads(nt)
    for (int64_t r = 0; r < (int64_t)nr; ++r) {
        uint64_t i = row0 + (uint64_t)r;
        EdgeHeap heap;
        row_heap(tnf, logsize, n, floor_cut, max_edges, i, heap, low);
        /* emission rule of cuda/Cuda2.cu:936-946: only i < j */
        while (!heap.empty()) {
            std::pair<uint64_t, double> e = heap.top();
            if (i < e.first) per_row[r].push_back(e);
            heap.pop();
        }
    }
    uint64_t total = 0;
    for (uint64_t r = 0; r < nr; ++r) {
        for (auto& e : per_row[r]) {
            if (total < cap) {
                from[total] = row0 + r;
                to[total] = e.first;
                stnf[total] = e.second;
            }
            ++total;
        }
    }
    return total;
}

/* gen_tnf_graph (cuda/Cuda2.cu:861-946) for a given list of rows only, in
 * the order given: each row's heap over all n columns, then its i < j edges.
 * A device's share of the reference's row tiles (888-891) is such a list. */
uint64_t orc_tnf_graph_rows(const float* tnf, const double* logsize, uint64_t n, double cutoff, uint32_t max_edges,
                            const uint64_t* rows, uint64_t nr, uint64_t* from, uint64_t* to, double* stnf,
                            uint64_t cap, int threads) {
    const double floor_cut = orc_logit_cutoff(cutoff);
    std::vector<std::vector<std::pair<uint64_t, double>>> per_row(nr);
    int nt = resolve_threads(threads);
    (void)nt;
#pragma omp parallel for schedule(dynamic, 1) num_threads(nt)
    for (int64_t r = 0; r < (int64_t)nr; ++r) {
        const uint64_t i = rows[r];
        EdgeHeap heap;
        row_heap(tnf, logsize, n, floor_cut, max_edges, i, heap, nullptr);
        while (!heap.empty()) {
            std::pair<uint64_t, double> e = heap.top();
            if (i < e.first) per_row[r].push_back(e);
            heap.pop();
        }
    }
    uint64_t total = 0;
    for (uint64_t r = 0; r < nr; ++r)
        for (auto& e : per_row[r]) {
            if (total < cap) {
                from[total] = rows[r];
                to[total] = e.first;
                stnf[total] = e.second;
            }
            ++total;
        }
    return total;
}

uint64_t orc_tnf_topk_rows(const float* tnf, const double* logsize, uint64_t n, double cutoff, uint32_t max_edges,
                           uint64_t row0, uint64_t row1, uint64_t* row_ptr, uint64_t* cols, double* sims, uint64_t cap,
                           int threads) {
    return orc_tnf_topk_rows_nz(tnf, logsize, n, cutoff, max_edges, row0, row1, row_ptr, cols, sims, cap, threads,
                                nullptr);
}

uint64_t orc_tnf_topk_rows_nz(const float* tnf, const double* logsize, uint64_t n, double cutoff,
                              uint32_t max_edges, uint64_t row0, uint64_t row1, uint64_t* row_ptr, uint64_t* cols,
                              double* sims, uint64_t cap, int threads, const uint8_t* low) {
    if (row1 > n) row1 = n;
    if (row0 >= row1) {
        row_ptr[0] = 0;
        return 0;
    }
    const double floor_cut = orc_logit_cutoff(cutoff);
    uint64_t nr = row1 - row0;
    std::vector<std::vector<std::pair<uint64_t, double>>> per_row(nr);
    int nt = resolve_threads(threads);
    (void)nt;
#pragma omp parallel for schedule(dynamic, 1) num_threads(nt)
    for (int64_t r = 0; r < (int64_t)nr; ++r) {
        EdgeHeap heap;
        row_heap(tnf, logsize, n, floor_cut, max_edges, row0 + (uint64_t)r, heap, low);
        while (!heap.empty()) {
            per_row[r].push_back(heap.top());
            heap.pop();
        }
    }
    uint64_t total = 0;
    for (uint64_t r = 0; r < nr; ++r) {
        row_ptr[r] = total;
        for (auto& e : per_row[r]) {
            if (total < cap) {
                cols[total] = e.first;
                sims[total] = e.second;
            }
            ++total;
        }
    }
    row_ptr[nr] = total;
    return total;
}

/* cuda/Cuda2.cu:281-314: position b of the permutation against every other
 * position; the running max starts at DBL_MIN (a tiny positive number), so a
 * contig whose pre-probabilities are all <= 0 reports sigmoid(DBL_MIN)=0.5. */
void orc_max_prob(const float* tnf, const double* logsize, uint64_t n, const uint64_t* contigs, uint64_t m,
                  double* out, int threads) {
    int nt = resolve_threads(threads);
    (void)nt;
#pragma omp parallel for schedule(dynamic, 1) num_threads(nt)
    for (int64_t b = 0; b < (int64_t)m; ++b) {
        uint64_t ci = contigs[b];
        double local_max = DBL_MIN;
        for (uint64_t i = 0; i < n; ++i) {
            if (i == (uint64_t)b) continue;
            double pre = orc_pre_prob(logsize[ci], logsize[contigs[i]], tnf + ci * 136, tnf + contigs[i] * 136);
            if (pre > local_max) local_max = pre;
        }
        out[b] = 1. - (1. / (1. + exp(local_max)));
    }
}

void orc_srand(uint32_t seed) { srand(seed); }
int orc_rand(void) { return rand(); }

/* gen_tnf_graph_sample (cuda/Cuda2.cu:972-1025). */
static double ptnf_sample(const float* tnf, const double* logsize, uint64_t n, double coverage, bool full,
                          int threads) {
    uint64_t m = full ? n : std::min(n, (uint64_t)2500);
    std::vector<uint64_t> idx(n);
    std::iota(idx.begin(), idx.end(), (uint64_t)0);
    /* random_unique, cuda/Cuda2.cu:500-511 */
    {
        uint64_t left = n;
        uint64_t* begin = idx.data();
        uint64_t k = m;
        while (k--) {
            uint64_t* r = begin + (uint64_t)rand() % left;
            std::swap(*begin, *r);
            ++begin;
            --left;
        }
    }
    std::vector<double> mx(m);
    orc_max_prob(tnf, logsize, n, idx.data(), m, mx.data(), threads);
    std::sort(mx.begin(), mx.end(), std::greater<double>());
    uint64_t p = 999, pp = 1000;
    double cov = 0, pcov = 0;
    uint64_t counton = 0;
    for (; p > 700;) {
        double cutoff = (double)p / 1000.;
        while (counton < m && mx[counton] >= cutoff) counton++;
        cov = (double)counton / m;
        if (cov >= coverage) {
            if (cov - coverage > coverage - pcov) {
                p = pp;
                cov = pcov;
            }
            break;
        }
        pp = p;
        pcov = cov;
        if (p > 990)
            p -= rand() % 3 + 1;
        else if (p > 900)
            p -= rand() % 3 + 3;
        else
            p -= rand() % 3 + 9;
    }
    return (double)p;
}

/* driver, cuda/Cuda2.cu:1885-1901 */
double orc_ptnf_search(const float* tnf, const double* logsize, uint64_t n, double coverage, int threads) {
    double ptnf = 0;
    if (n <= 25000) return ptnf_sample(tnf, logsize, n, coverage, true, threads);
    for (int i = 0; i < 10; ++i) {
        double minp = ptnf_sample(tnf, logsize, n, coverage, false, threads);
        if (minp < 701) minp = 700.;
        ptnf += minp;
        if (i == 1 && ptnf / 2 < 701) {
            ptnf = 700.;
            break;
        }
        if (i == 9) ptnf /= 10.;
    }
    return ptnf;
}

/* ----------------------------------------------------------- abundance --
 * Coverage side of the edge score.  abd and var are n x nabd row-major
 * matrices: mean depth and depth variance of contig r in sample i (the
 * reference's ABD(r, i) and ABD_VAR(r, i)). */

/* A contig is "low" when none of its depths exceeds 1; is_nz
 * (cuda/Cuda2.cu:845-856, fixed threshold 1) rejects a pair of two low
 * contigs. */
void orc_abd_low(const double* abd, uint64_t n, uint32_t nabd, uint8_t* low) {
    for (uint64_t r = 0; r < n; ++r) {
        bool any = false;
        for (uint32_t i = 0; i < nabd; ++i) any = any || abd[r * nabd + i] > 1.;
        low[r] = (nabd > 0 && !any) ? 1 : 0;
    }
}

}  // extern "C"

namespace {

/* The reference evaluates boost::math::cdf(normal_distribution(mean, sd), x)
 * (Boost.Math, a dependency that is not part of the MdeT sources).  Its
 * published definition: erfc(-(x - mean) / (sd * sqrt(2))) / 2. */
double normal_cdf(double mean, double sd, double x) {
    const double z = (x - mean) / (sd * 1.4142135623730951);
    return erfc(-z) / 2;
}

/* cal_abd_dist2 (cuda/Cuda2.cu:667-700): the overlap of two normal densities,
 * from the crossing points k1 <= k2 of the densities; the narrower
 * distribution is evaluated first. */
double abd_dist2(double m1, double s1, double m2, double s2) {
    const double v1 = s1 * s1, v2 = s2 * s2;
    double k1, k2;
    if (fabs(v2 - v1) < 1e-4) {
        k1 = k2 = (m1 + m2) / 2;
    } else {
        const double t = sqrt(v1 * v2 * ((m1 - m2) * (m1 - m2) - 2 * (v1 - v2) * log(sqrt(v2 / v1))));
        k1 = (t - m1 * v2 + m2 * v1) / (v1 - v2);
        k2 = (t + m1 * v2 - m2 * v1) / (v2 - v1);
    }
    if (k1 > k2) std::swap(k1, k2);
    double ma = m1, sa = s1, mb = m2, sb = s2;
    if (v1 > v2) {
        std::swap(ma, mb);
        std::swap(sa, sb);
    }
    if (k1 == k2) return fabs(normal_cdf(ma, sa, k1) - normal_cdf(mb, sb, k1));
    return fabs(normal_cdf(ma, sa, k2) - normal_cdf(ma, sa, k1) + normal_cdf(mb, sb, k1) - normal_cdf(mb, sb, k2));
}

/* cal_abd_dist (cuda/Cuda2.cu:702-719) for sample i; *nz is set when either
 * depth exceeds min_cv. */
double abd_dist(const double* abd, const double* var, uint32_t nabd, uint64_t r1, uint64_t r2, uint32_t i,
                double min_cv, bool* nz) {
    double d = 0;
    double m1 = abd[r1 * nabd + i], m2 = abd[r2 * nabd + i];
    if (m1 > min_cv || m2 > min_cv) {
        *nz = true;
        m1 = std::max(m1, 1e-6);
        m2 = std::max(m2, 1e-6);
        if (m1 != m2) {
            const double w1 = var[r1 * nabd + i], w2 = var[r2 * nabd + i];
            const double v1 = w1 < 1 ? 1 : w1, v2 = w2 < 1 ? 1 : w2;
            d = abd_dist2(m1, sqrt(v1), m2, sqrt(v2));
        }
    }
    return std::min(std::max(d, 1e-6), 1. - 1e-6);
}

/* cal_abd_corr (cuda/Cuda2.cu:1219-1245): Pearson correlation of the two
 * depth profiles with running (Welford) means and co-moments. */
double abd_corr(const double* abd, uint32_t nabd, uint64_t r1, uint64_t r2) {
    double sxx = 0, syy = 0, sxy = 0, mx = 0, my = 0;
    for (uint32_t i = 0; i < nabd; ++i) {
        const double x = abd[r1 * nabd + i], y = abd[r2 * nabd + i];
        if (i == 0) {
            mx = x;
            my = y;
            continue;
        }
        const double ratio = i / (i + 1.0);
        const double dx = x - mx, dy = y - my;
        sxx += dx * dx * ratio;
        syy += dy * dy * ratio;
        sxy += dx * dy * ratio;
        mx += dx / (i + 1.0);
        my += dy / (i + 1.0);
    }
    return sxy / (sqrt(sxx) * sqrt(syy));
}

/* rank(v, w, "min" | "max") (cuda/ranker.h:56-80): 1-based ranks in
 * ascending order; a run of equal values gets its first ("min") or last
 * ("max") rank. */
void rank_ties(const double* v, uint64_t n, bool last, std::vector<double>& r) {
    std::vector<uint64_t> ord(n);
    std::iota(ord.begin(), ord.end(), (uint64_t)0);
    std::sort(ord.begin(), ord.end(), [&](uint64_t a, uint64_t b) { return v[a] < v[b]; });
    r.resize(n);
    for (uint64_t c = 0; c < n;) {
        uint64_t k = 1;
        while (c + k < n && v[ord[c]] == v[ord[c + k]]) ++k;
        for (uint64_t q = 0; q < k; ++q) r[ord[c + q]] = (double)(last ? c + k : c + 1);
        c += k;
    }
}

}  // namespace

extern "C" {

/* sTNF -> sSCR (cuda/Cuda2.cu:1921-1971): per edge the mean abundance
 * similarity over the samples where either contig is covered (nnz of them);
 * sTNF, and with nabd >= min_sample the depth correlation, are mapped by
 * rank onto the sorted abundance similarities; the score is their weighted
 * geometric mean.  Edge e joins to[e] (r1) and from[e] (r2), in that order.
 * nabd == 0: sSCR = sTNF. */
void orc_sscr(const uint64_t* from, const uint64_t* to, const double* stnf, uint64_t ne, const double* abd,
              const double* var, uint32_t nabd, double min_cv, uint32_t min_sample, double* sscr, int threads) {
    if (nabd == 0) {
        for (uint64_t e = 0; e < ne; ++e) sscr[e] = stnf[e];
        return;
    }
    int nt = resolve_threads(threads);
    (void)nt;
    std::vector<double> raw(ne, 0.0);
    std::vector<int> nnz(ne, 0);
#pragma omp parallel for schedule(static) num_threads(nt)
    for (int64_t e = 0; e < (int64_t)ne; ++e) {
        for (uint32_t i = 0; i < nabd; ++i) {
            bool nz = false;
            const double a = 1. - abd_dist(abd, var, nabd, to[e], from[e], i, min_cv, &nz);
            if (nz) {
                raw[e] += a;
                ++nnz[e];
            }
        }
        raw[e] /= nnz[e];
    }
    std::vector<double> distr(raw);
    std::sort(distr.begin(), distr.end());
    std::vector<double> rt, rc;
    rank_ties(stnf, ne, false, rt);
    const bool corr = nabd >= min_sample;
    if (corr) {
        std::vector<double> c(ne);
#pragma omp parallel for schedule(static) num_threads(nt)
        for (int64_t e = 0; e < (int64_t)ne; ++e) c[e] = abd_corr(abd, nabd, to[e], from[e]);
        rank_ties(c.data(), ne, true, rc);
    }
#pragma omp parallel for schedule(static) num_threads(nt)
    for (int64_t e = 0; e < (int64_t)ne; ++e) {
        const double t = distr[(uint64_t)round(rt[e]) - 1];
        const double w = 1. / (1 + nnz[e]);
        if (corr) {
            const double c = distr[(uint64_t)round(rc[e]) - 1];
            sscr[e] = pow(pow(raw[e], 1. - w) * pow(t, w) * c, 1. / 2.);
        } else {
            sscr[e] = pow(raw[e], 1. - w) * pow(t, w);
        }
    }
}

}  // extern "C"

// ------------------------------------------------ leftover recruiting ----

namespace {

/* rank(rowMat, rowMat) on a float row (cuda/ranker.h:56-68, method
 * "average"): 1-based ranks in ascending order; a run of equal values gets
 * the mean of its ranks, formed in float as the reference's S = float. */
void rank_average_f(float* v, uint32_t n) {
    std::vector<uint32_t> ord(n);
    std::iota(ord.begin(), ord.end(), 0u);
    std::sort(ord.begin(), ord.end(), [&](uint32_t a, uint32_t b) { return v[a] < v[b]; });
    std::vector<float> w(n);
    for (uint32_t c = 0; c < n;) {
        uint32_t k = 1;
        while (c + k < n && v[ord[c]] == v[ord[c + k]]) ++k;
        for (uint32_t q = 0; q < k; ++q) w[ord[c + q]] = (float)(2 * c + k - 1) / 2 + 1;
        c += k;
    }
    std::copy(w.begin(), w.end(), v);
}

/* cal_abd_corr (cuda/Cuda2.cu:1219-1245) between row r1 of a and row r2 of b
 * (float matrices, values read as double). */
double corr_f(const float* a, const float* b, uint32_t nabd, uint64_t r1, uint64_t r2) {
    double sxx = 0, syy = 0, sxy = 0, mx = 0, my = 0;
    for (uint32_t i = 0; i < nabd; ++i) {
        const double x = a[r1 * nabd + i], y = b[r2 * nabd + i];
        if (i == 0) {
            mx = x;
            my = y;
            continue;
        }
        const double ratio = i / (i + 1.0);
        const double dx = x - mx, dy = y - my;
        sxx += dx * dx * ratio;
        syy += dy * dy * ratio;
        sxy += dx * dy * ratio;
        mx += dx / (i + 1.0);
        my += dy / (i + 1.0);
    }
    return sxy / (sqrt(sxx) * sqrt(syy));
}

}  // namespace

extern "C" {

/* Dissolving small bins and recruiting leftover and small contigs
 * (cuda/Cuda2.cu:2064-2283, after label propagation).  Bins are the label
 * groups of the large contigs, members in ascending index; a bin whose
 * sizes sum below min_cls_size is dissolved and its members become
 * leftovers.  The depth rows are replaced by their average ranks (Spearman).
 * Bins with at least 10 members get the mean pairwise correlation of their
 * members (cls_corr).  A leftover (a small contig) joins bin k when its mean
 * correlation with the first 10 members, and then with all members, is at
 * least cls_corr[k] -- and only when exactly one bin qualifies (the
 * reference stops at a second one and keeps none).  The leftovers are added
 * when their bases are under 10 % of the binned bases, the small contigs when
 * theirs are under 15 % of small_total (the reference's totalSize1, which it
 * only sums in verbose runs; 0 rejects every small recruit).  Out: the bin
 * label of every large contig (-1: dissolved and not recruited) and of every
 * small contig (-1: none).  stats: [0] kept bins, [1] scored bins,
 * [2] leftovers, [3] leftovers matched, [4] smalls matched, [5] leftovers
 * accepted, [6] smalls accepted.  abd and small_abd are overwritten by their
 * ranks, as in the reference. */
void orc_recruit(float* abd, float* small_abd, uint64_t n, uint64_t n1, uint32_t nabd, const int64_t* label,
                 const uint64_t* sizes, const uint64_t* small_sizes, uint64_t min_cls_size, uint64_t small_total,
                 int64_t* out, int64_t* small_out, uint64_t* stats) {
    std::map<int64_t, std::vector<uint64_t>> cls;
    for (uint64_t i = 0; i < n; ++i) cls[label[i]].push_back(i);
    std::vector<uint64_t> leftovers;
    for (auto it = cls.begin(); it != cls.end();) {
        uint64_t s = 0;
        for (uint64_t m : it->second) s += sizes[m];
        if (s < min_cls_size) {
            leftovers.insert(leftovers.end(), it->second.begin(), it->second.end());
            it = cls.erase(it);
        } else {
            ++it;
        }
    }
    for (uint64_t i = 0; i < n; ++i) out[i] = -1;
    for (uint64_t i = 0; i < n1; ++i) small_out[i] = -1;
    for (auto& kv : cls)
        for (uint64_t m : kv.second) out[m] = kv.first;
    for (int k = 0; k < 7; ++k) stats[k] = 0;
    stats[0] = cls.size();
    stats[2] = leftovers.size();
    if (leftovers.empty() && n1 == 0) return;
    const size_t minCS = 10;
    for (uint64_t r = 0; r < n; ++r) rank_average_f(abd + r * nabd, nabd);
    uint64_t binned = 0;
    for (auto& kv : cls)
        for (uint64_t m : kv.second) binned += sizes[m];
    std::map<int64_t, double> cls_corr;
    for (auto& kv : cls) {
        const auto& c = kv.second;
        const size_t cs = c.size();
        if (cs < minCS) continue;
        double corr = 0;
        for (size_t i = 0; i < cs; ++i)
            for (size_t j = i + 1; j < cs; ++j) corr += corr_f(abd, abd, nabd, c[i], c[j]);
        cls_corr[kv.first] = corr / (cs * (cs - 1) / 2);
        ++stats[1];
    }
    // the bin a contig joins: the single qualifying bin, or -1
    auto assign = [&](const float* other, uint64_t r) -> int64_t {
        int64_t best = -1;
        for (auto& kv : cls) {
            const auto& c = kv.second;
            const size_t cs = c.size();
            if (cs < minCS) continue;
            const double th = cls_corr[kv.first];
            double corr = 0;
            size_t i = 0;
            for (; i < minCS; ++i) corr += corr_f(abd, other, nabd, c[i], r);
            if (corr / minCS < th) continue;
            for (; i < cs; ++i) corr += corr_f(abd, other, nabd, c[i], r);
            corr /= cs;
            if (corr >= th) {
                if (best > -1) return -1;
                best = kv.first;
            }
        }
        return best;
    };
    std::vector<int64_t> lb(leftovers.size());
    for (size_t l = 0; l < leftovers.size(); ++l) lb[l] = assign(abd, leftovers[l]);
    std::vector<int64_t> sb(n1, -1);
    if (n1 > 0) {
        for (uint64_t r = 0; r < n1; ++r) rank_average_f(small_abd + r * nabd, nabd);
        for (uint64_t s = 0; s < n1; ++s) sb[s] = assign(small_abd, s);
    }
    unsigned long long added = 0;
    for (size_t l = 0; l < leftovers.size(); ++l)
        if (lb[l] > -1) {
            added += sizes[leftovers[l]];
            ++stats[3];
        }
    if (added > 0 && (double)added / binned < .10) {
        stats[5] = 1;
        for (size_t l = 0; l < leftovers.size(); ++l)
            if (lb[l] > -1) out[leftovers[l]] = lb[l];
    }
    added = 0;
    for (uint64_t s = 0; s < n1; ++s)
        if (sb[s] > -1) {
            added += small_sizes[s];
            ++stats[4];
        }
    if (added > 0 && (double)added / small_total < .15) {
        stats[6] = 1;
        for (uint64_t s = 0; s < n1; ++s) small_out[s] = sb[s];
    }
}

}  // extern "C"

extern "C" {

/* The reference reader's record split (cuda/Cuda2.cu:1507-1544), read
 * sequentially: a '>' starts a record wherever it stands (a '>' inside the
 * record's own name line belongs to the name); the name is the rest of that
 * line cut at its first space; the sequence view runs from after the name
 * line's newline to the next record's '>' (or the end), inner newlines kept,
 * and drops one trailing newline; size = the view's bytes before that drop
 * minus its newlines.  A name line with no newline before the end of the
 * buffer ends the scan (the reference would read past its buffer there).
 * Every record is returned (no size classes); at most cap are written. */
uint64_t orc_fasta_index(const char* b, uint64_t nbytes, uint64_t cap, uint64_t* seq_off, uint64_t* seq_len,
                         uint64_t* size, uint64_t* name_off, uint32_t* name_len) {
    uint64_t nr = 0, i = 0;
    while (i < nbytes) {
        const char* gt = (const char*)memchr(b + i, '>', nbytes - i);
        if (!gt) break;
        const uint64_t p = (uint64_t)(gt - b);
        const char* nl = (const char*)memchr(b + p + 1, '\n', nbytes - p - 1);
        if (!nl) break;
        const uint64_t h = (uint64_t)(nl - b);
        uint64_t nlen = h - (p + 1);
        const char* sp = (const char*)memchr(b + p + 1, ' ', nlen);
        if (sp) nlen = (uint64_t)(sp - (b + p + 1));
        const uint64_t s0 = h + 1;
        const char* nx = (const char*)memchr(b + s0, '>', nbytes - s0);
        const uint64_t s1 = nx ? (uint64_t)(nx - b) : nbytes;
        uint64_t lines = 0;
        for (uint64_t q = s0; q < s1; ++q) lines += b[q] == '\n';
        uint64_t view = s1 - s0;
        const uint64_t sz = view - lines;
        if (view > 0 && b[s1 - 1] == '\n') --view;
        if (nr < cap) {
            seq_off[nr] = s0;
            seq_len[nr] = view;
            size[nr] = sz;
            name_off[nr] = p + 1;
            name_len[nr] = (uint32_t)nlen;
        }
        ++nr;
        i = s1;
    }
    return nr;
}

}  // extern "C"

/* ------------------------------------------------------------------------
 * Label propagation over the scored edge graph (cuda/Cuda2.cu:1980-2061, the
 * traversal of main, and label_propagation, cuda/Cuda2.cu:569-656),
 * restated.  The chi-squared CDF (float-float, lpf::chi2_cdf), and the log
 * of 1 - sSCR (double, lpm::log), are the
 * project's own host/device functions of mdet_gb300/csrc/lp_math.h (the
 * reference calls Boost's CDF and the C library's log; Boost is not used
 * here), so that the device form can be held to the last bit.  The
 * per-contig label tallies are std::unordered_map / unordered_set, as in the
 * reference: the label picked among exact ties is the first in that map's
 * iteration order.
 * ---------------------------------------------------------------------- */
#include <climits>
#include <unordered_map>
#include <unordered_set>

#include "../mdet_gb300/csrc/lp_math.h"

namespace {

struct LpGraph {
    std::vector<uint64_t> from, to;   // to: the edge's first contig (ii), from: the second (jj)
    std::vector<double> lw;           // log(1 - sSCR)
    std::vector<std::vector<uint64_t>> inc;
};

struct LpFact {
    std::vector<lpf::F2> t;
    const lpf::F2* at(uint64_t c) {
        if (t.size() <= c) {
            t.resize(std::max<uint64_t>(c + 1, 2 * t.size()));
            lpf::log_factorials(t.data(), (uint32_t)t.size());
        }
        return t.data();
    }
};

/* One call of label_propagation (cuda/Cuda2.cu:569-656): Gauss-Seidel sweeps
 * over `order`; each contig takes the neighbour label with the largest
 * Fisher-combined CDF; a contig that moves back to a label it held earlier
 * in this call is frozen; the sweeps stop when no contig moved to a new
 * label, or after 10 sweeps in a row without a new low of such moves. */
void lp_call(LpGraph& g, std::vector<uint64_t>& mem, const std::vector<uint64_t>& order, LpFact& lf,
             uint64_t* sweeps, uint64_t* frozen, uint64_t* ties) {
    std::unordered_map<uint64_t, std::unordered_set<uint64_t>> held;
    std::unordered_set<uint64_t> stuck;
    uint64_t low = INT_MAX, attempt = 0;
    bool again = true;
    while (again) {
        again = false;
        uint64_t moved = 0;
        ++*sweeps;
        for (uint64_t v : order) {
            std::unordered_map<uint64_t, double> score;
            std::unordered_map<uint64_t, uint64_t> cnt;
            for (uint64_t e : g.inc[v]) {
                const uint64_t k = mem[g.from[e] == v ? g.to[e] : g.from[e]];
                if (score.find(k) == score.end()) {
                    score[k] = 0.;
                    cnt[k] = 0;
                }
                score[k] += g.lw[e];
                cnt[k]++;
            }
            if (score.empty()) continue;
            for (auto& kv : score) {
                const uint64_t c = cnt[kv.first];
                kv.second = lpf::chi2_cdf(2.0 * (double)c, -2.0 * kv.second, lf.at(c));
            }
            auto best = score.begin();
            for (auto it = score.begin(); it != score.end(); ++it)
                if (best->second < it->second) best = it;
            uint64_t at_top = 0;
            for (auto& kv : score) at_top += kv.second == best->second;
            *ties += at_top > 1;
            if (mem[v] != best->first && stuck.find(v) == stuck.end()) {
                mem[v] = best->first;
                auto& h = held[v];
                if (h.insert(best->first).second) {
                    ++moved;
                    again = true;
                } else {
                    stuck.insert(v);
                }
            }
        }
        if (moved < low) {
            low = moved;
            attempt = 0;
        } else if (++attempt >= 10) {
            break;
        }
    }
    *frozen += stuck.size();
}

}  // namespace

extern "C" {

/* The binning traversal (cuda/Cuda2.cu:1980-2061): edges in decreasing sSCR
 * (equal scores in edge order; the reference's std::sort leaves their order
 * open); every contig starts in its own bin; an edge whose two contigs are
 * in different bins connects them (first-seen order: to before from) and,
 * when its score is above min_s, joins the traversal graph -- the first such
 * edge at or below min_s ends the traversal.  Label propagation runs each
 * time the connected share of the n contigs reaches max_p/10 * (1..10), and
 * at the last edge; at most 10 times.  mem_out: the bin of every contig.
 * stats: [0] propagation calls, [1] sweeps, [2] traversal-graph edges,
 * [3] connected contigs, [4] frozen contigs (summed over calls), [5] contig
 * updates decided among exactly tied labels. */
void orc_label_prop(const uint64_t* from, const uint64_t* to, const double* sscr, uint64_t ne, uint64_t n,
                    double max_p, double min_s, uint64_t* mem_out, uint64_t* stats) {
    for (int k = 0; k < 6; ++k) stats[k] = 0;
    std::vector<uint64_t> ord(ne);
    std::iota(ord.begin(), ord.end(), 0);
    std::stable_sort(ord.begin(), ord.end(), [&](uint64_t a, uint64_t b) { return sscr[a] > sscr[b]; });
    std::vector<double> sched;
    for (int i = 1; i <= 10; ++i) sched.push_back(max_p / 10 * i);
    std::vector<uint64_t> mem(n);
    std::iota(mem.begin(), mem.end(), 0);
    std::vector<char> seen(n, 0);
    std::vector<uint64_t> order;
    LpGraph g;
    g.inc.resize(n);
    LpFact lf;
    size_t which = 0;
    for (uint64_t i = 0; i < ne; ++i) {
        const uint64_t e = ord[i];
        const uint64_t ii = to[e], jj = from[e];
        if (mem[ii] != mem[jj]) {
            if (!seen[ii]) {
                seen[ii] = 1;
                order.push_back(ii);
            }
            if (!seen[jj]) {
                seen[jj] = 1;
                order.push_back(jj);
            }
            const double s = sscr[e];
            if (s > min_s) {
                g.from.push_back(jj);
                g.to.push_back(ii);
                g.lw.push_back(lpm::log(1. - s));
                g.inc[ii].push_back(g.from.size() - 1);
                g.inc[jj].push_back(g.from.size() - 1);
            } else {
                i = ne - 1;
            }
        }
        if (!g.from.empty() && ((double)order.size() / (double)n >= sched[which] || i == ne - 1)) {
            ++stats[0];
            lp_call(g, mem, order, lf, &stats[1], &stats[4], &stats[5]);
            if (++which == sched.size()) break;
        }
    }
    stats[2] = g.from.size();
    stats[3] = order.size();
    for (uint64_t i = 0; i < n; ++i) mem_out[i] = mem[i];
}

/* Iteration order of std::unordered_map<uint64_t, ...> after inserting the
 * distinct keys keys[0..k) in turn (as this C++ library lays it out), for
 * checking the device form's emulation of that order. */
void orc_umap_order(const uint64_t* keys, uint64_t k, uint64_t* out) {
    std::unordered_map<uint64_t, double> m;
    for (uint64_t i = 0; i < k; ++i) m[keys[i]] = 0.;
    uint64_t j = 0;
    for (auto& kv : m) out[j++] = kv.first;
}

/* lp_math.h's functions, for checking them against independent references */
double orc_lp_log(double x) { return lpm::log(x); }
double orc_lp_exp(double x) { return lpm::exp(x); }
double orc_lp_chi2_cdf(uint64_t count, double x) {
    std::vector<lpf::F2> lf(count + 1);
    lpf::log_factorials(lf.data(), (uint32_t)lf.size());
    return lpf::chi2_cdf(2.0 * (double)count, x, lf.data());
}

}  // extern "C"

#include "../mdet_gb300/csrc/lp_umap.h"

extern "C" {
/* lp_umap.h's emulation of that order (the device form's tie rule), for
 * checking it against orc_umap_order. */
void orc_umap_emulated(const uint64_t* keys, uint64_t k, uint64_t* out) {
    std::vector<int32_t> nxt(k + 1), bb(lpu::buckets_for((uint32_t)k));
    int32_t p = lpu::order(keys, (uint32_t)k, nxt.data(), bb.data());
    uint64_t j = 0;
    while (p >= 0) {
        out[j++] = keys[p];
        p = nxt[p];
    }
}
}  // extern "C"
