/*
 * ref_prob_shim.cpp -- host shim around the reference's own probability
 * functions (test infrastructure).  oracle/build_ref.py cuts
 * cal_tnf_pre_dist_d with its coefficient tables (cuda/Cuda2.cu:170-241) and
 * cal_tnf_dist (cuda/Cuda2.cu:721-779) out of the mounted reference into
 * _ref/cuda2_prob.inc; the macros and globals below are what those spans
 * expect from the rest of Cuda2.cu, so they compile unchanged on the host.
 */
#include <cfloat>
#include <cmath>
#include <cstddef>
#include <vector>

#define __device__
#define __constant__
typedef double Distance;
typedef double Similarity;
#define LOG log
#define SQRT sqrt
#define EXP exp
static inline double min(double a, double b) { return a < b ? a : b; }
static inline double max(double a, double b) { return a > b ? a : b; }
static const size_t nTNF = 136;
static float* TNF;
static std::vector<Distance> logSizes;

#include "cuda2_prob.inc"

extern "C" {
double ref_pre_prob(double r1, double r2, const float* a, const float* b) {
    return cal_tnf_pre_dist_d(r1, r2, a, b);
}
double ref_tnf_dist(double r1, double r2, const float* a, const float* b) {
    static thread_local float buf[272];
    for (int k = 0; k < 136; ++k) {
        buf[k] = a[k];
        buf[136 + k] = b[k];
    }
    TNF = buf;
    logSizes.assign({r1, r2});
    return cal_tnf_dist(0, 1);
}
}
