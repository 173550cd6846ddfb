/*
 * ref_abd_shim.cpp -- host shim around the reference's own abundance-scoring
 * code (test infrastructure).  oracle/build_ref.py cuts cal_abd_dist2,
 * cal_abd_dist, is_nz, cal_abd_corr (cuda/Cuda2.cu:667-719, 845-856,
 * 1219-1245) and the sTNF -> sSCR block of main (cuda/Cuda2.cu:1921-1971) out
 * of the mounted reference into _ref/cuda2_abd.inc and includes the
 * reference's cuda/ranker.h; the definitions below are what those spans expect
 * from the rest of Cuda2.cu.  Boost is not available here, so its normal
 * distribution is stood in for by the published definition of its CDF,
 * erfc(-(x - mean) / (sd * sqrt(2))) / 2.
 */
#include <algorithm>
#include <cmath>
#include <cstddef>
#include <cstdint>
#include <string>
#include <vector>

typedef double Distance;
typedef double Similarity;
#define LOG log
#define SQRT sqrt
#define POW pow
#define FABS fabs

namespace boost {
namespace math {
template <class T>
class normal_distribution {
   public:
    normal_distribution(T m = 0, T s = 1) : m_(m), s_(s) {}
    T mean() const { return m_; }
    T standard_deviation() const { return s_; }

   private:
    T m_, s_;
};
template <class T>
T cdf(const normal_distribution<T>& d, const T& x) {
    const T diff = (x - d.mean()) / (d.standard_deviation() * 1.4142135623730951);
    return std::erfc(-diff) / 2;
}
}  // namespace math
}  // namespace boost
typedef boost::math::normal_distribution<Distance> Normal;

#include "ranker.h"

struct Mat {
    const double* p = nullptr;
    size_t cols = 0;
    double operator()(size_t r, size_t c) const { return p[r * cols + c]; }
};
static Mat ABD, ABD_VAR, small_ABD;
static size_t nABD = 0;
static Distance minCV = 1;
static size_t minSample = 3;
static std::string abdFile;
struct Graph {
    std::vector<size_t> from, to;
    std::vector<double> sTNF, sSCR;
};
static void verbose_message(const char*, ...) {}

#include "cuda2_abd.inc"

extern "C" {
void ref_sscr(const uint64_t* from, const uint64_t* to, const double* stnf, uint64_t ne, const double* abd,
              const double* var, uint32_t nabd, double min_cv, uint32_t min_sample, double* sscr) {
    ABD.p = abd;
    ABD.cols = nabd;
    ABD_VAR.p = var;
    ABD_VAR.cols = nabd;
    nABD = nabd;
    minCV = min_cv;
    minSample = min_sample;
    abdFile = nabd ? "abundance" : "";
    Graph g;
    g.from.assign(from, from + ne);
    g.to.assign(to, to + ne);
    g.sTNF.assign(stnf, stnf + ne);
    sscr_block(g, (size_t)ne);
    std::copy(g.sSCR.begin(), g.sSCR.end(), sscr);
}

int ref_is_nz(const double* abd, uint32_t nabd, uint64_t r1, uint64_t r2) {
    ABD.p = abd;
    ABD.cols = nabd;
    nABD = nabd;
    abdFile = nabd ? "abundance" : "";
    return is_nz((size_t)r1, (size_t)r2) ? 1 : 0;
}
}
