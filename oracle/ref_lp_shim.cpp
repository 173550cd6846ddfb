/*
 * ref_lp_shim.cpp -- host shim around the reference's own label propagation
 * (test infrastructure).  oracle/build_ref.py cuts label_propagation
 * (cuda/Cuda2.cu:569-656) and the block of main that traverses the scored
 * edges in decreasing order and calls it (cuda/Cuda2.cu:1980-2061) out of the
 * mounted reference into _ref/cuda2_lp.inc and compiles them with the
 * reference's own cuda/ranker.h.  What those spans expect from the rest of
 * Cuda2.cu is defined here: the Graph class's members, the option globals,
 * logging and memory-report helpers (no-ops), and in place of Boost --
 * which is not used here -- boost::math::chi_squared and its cdf,
 * computed by lp_math.h, whose functions are the ones the device form uses.
 * LOG, which the reference defines as the C library's log, is lp_math.h's
 * log for the same reason.
 */
#include <algorithm>
#include <cassert>
#include <climits>
#include <cmath>
#include <cstddef>
#include <cstdlib>
#include <cstdint>
#include <fstream>
#include <iostream>
#include <numeric>
#include <string>
#include <unordered_map>
#include <unordered_set>
#include <vector>

#include "lp_math.h"

using std::cerr;
using std::cout;
using std::endl;

typedef double Distance;
typedef double Similarity;
#define LOG lpm::log

#include "ranker.h"

namespace boost {
namespace math {
struct chi_squared {
    double dof;
    explicit chi_squared(double d) : dof(d) {}
};
inline double cdf(const chi_squared& d, double x) {
    static std::vector<lpf::F2> lf;
    const size_t c = (size_t)(d.dof * 0.5);
    if (lf.size() <= c) {
        lf.resize(std::max<size_t>(c + 1, 2 * lf.size()));
        lpf::log_factorials(lf.data(), (uint32_t)lf.size());
    }
    return lpf::chi2_cdf(d.dof, x, lf.data());
}
}  // namespace math
template <class T, class S>
T lexical_cast(const S& s) {
    return std::to_string(s);
}
}  // namespace boost

typedef std::vector<int> ContigVector;
typedef std::unordered_set<int> ContigSet;
typedef std::unordered_map<int, ContigVector> ClassMap;

// the members of the reference's Graph that the cut spans use
class Graph {
   public:
    size_t n;
    std::vector<size_t> from, to;
    std::vector<std::vector<size_t>> incs;
    std::vector<double> sTNF, sSCR;
    ContigSet connected_nodes;
    bool hasEdges;
    Graph(size_t num_nodes, bool has_edges = false) : n(num_nodes), hasEdges(has_edges) {
        if (has_edges) incs.resize(num_nodes);
    }
    size_t getNodeCount() { return n; }
    size_t getEdgeCount() { return from.size(); }
    size_t getOtherNode(size_t e, size_t v) { return from[e] == v ? to[e] : from[e]; }
};

static size_t nobs = 0;
static Similarity maxP = 0.95, minS = 0.60;
static bool debug = false;
static size_t lp_calls = 0;
// the traversal reports each propagation call with this message
static void verbose_message(const char* fmt, ...) {
    if (std::string(fmt).rfind("Building SCR Graph", 0) == 0) ++lp_calls;
}
static double getUsedPhysMem() { return 0; }
static double getTotalPhysMem() { return 0; }

#include "cuda2_lp.inc"

extern "C" {
/* The reference's traversal on the edges (from[e], to[e], sscr[e]) of n
 * contigs; max_p and min_s as fractions (the reference divides its percent
 * options by 100).  Returns the number of label propagation calls. */
uint64_t ref_label_prop(const uint64_t* from, const uint64_t* to, const double* sscr, uint64_t ne, uint64_t n,
                        double max_p, double min_s, uint64_t* mem_out) {
    nobs = n;
    maxP = max_p;
    minS = min_s;
    lp_calls = 0;
    Graph g(n);
    g.from.assign(from, from + ne);
    g.to.assign(to, to + ne);
    g.sSCR.assign(sscr, sscr + ne);
    std::vector<size_t> mems;
    lp_block(g, ne, mems);
    for (uint64_t i = 0; i < n; ++i) mem_out[i] = mems[i];
    return lp_calls;
}
}
