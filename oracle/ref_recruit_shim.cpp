/*
 * ref_recruit_shim.cpp -- host shim around the reference's own dissolving and
 * recruiting code (test infrastructure).  oracle/build_ref.py cuts
 * cal_abd_corr (cuda/Cuda2.cu:1219-1245) and the block of main from the
 * grouping of contigs into bins after label propagation to the end of the
 * recruiting of leftover and small contigs (cuda/Cuda2.cu:2064-2283) out of
 * the mounted reference into _ref/cuda2_recruit.inc, and compiles it with the
 * reference's own cuda/ranker.h.  The definitions below are what those spans
 * expect from the rest of Cuda2.cu: the ublas float matrix and its row view
 * are stood in for by a row-major float array.
 */
#include <algorithm>
#include <cmath>
#include <cstddef>
#include <cstdint>
#include <cstdio>
#include <string>
#include <unordered_map>
#include <unordered_set>
#include <vector>

typedef double Distance;
typedef double Similarity;

#include "ranker.h"

struct FMat {
    float* p = nullptr;
    size_t rows = 0, cols = 0;
    size_t size1() const { return rows; }
    size_t size2() const { return cols; }
    float& operator()(size_t r, size_t c) { return p[r * cols + c]; }
    float operator()(size_t r, size_t c) const { return p[r * cols + c]; }
};
struct MatrixRowType {
    float* b;
    float* e;
    MatrixRowType(FMat& m, size_t r) : b(m.p + r * m.cols), e(m.p + (r + 1) * m.cols) {}
    float* begin() { return b; }
    float* end() { return e; }
};

typedef std::vector<int> ContigVector;
typedef std::unordered_map<int, ContigVector> ClassMap;

static FMat ABD, small_ABD;
static size_t nABD = 0, nobs = 0, nobs1 = 0, minClsSize = 200000, minSample = 3, minContig = 2500;
static bool noAdd = false, verbose = false;
static unsigned long long totalSize = 0, totalSize1 = 0;
static std::vector<size_t> sizes, small_sizes;
static void verbose_message(const char*, ...) {}

#include "cuda2_recruit.inc"

extern "C" {
/* The reference's block on the given bins; out[i] (large) and small_out[s]:
 * the final bin of each contig, -1 when none.  abd and small_abd are
 * replaced by their ranks, as in the reference.  verbose: the reference's
 * flag, which decides whether totalSize1 is summed before the small-contig
 * gate. */
void ref_recruit(float* abd, float* small_abd, uint64_t n, uint64_t n1, uint32_t nabd, const int64_t* label,
                 const uint64_t* sz, const uint64_t* small_sz, uint64_t min_cls_size, int verb, int64_t* out,
                 int64_t* small_out) {
    ABD.p = abd;
    ABD.rows = n;
    ABD.cols = nabd;
    small_ABD.p = small_abd;
    small_ABD.rows = n1;
    small_ABD.cols = nabd;
    nABD = nabd;
    nobs = n;
    nobs1 = n1;
    minClsSize = min_cls_size;
    verbose = verb != 0;
    totalSize = totalSize1 = 0;
    sizes.assign(sz, sz + n);
    small_sizes.assign(small_sz, small_sz + n1);
    std::vector<size_t> mems(label, label + n);
    ClassMap cls;
    recruit_block(cls, mems);
    for (uint64_t i = 0; i < n; ++i) out[i] = -1;
    for (uint64_t s = 0; s < n1; ++s) small_out[s] = -1;
    for (auto& kv : cls)
        for (int m : kv.second) {
            if ((size_t)m < n) out[m] = kv.first;
            else small_out[m - n] = kv.first;
        }
}
}
