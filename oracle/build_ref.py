#!/usr/bin/env python3
"""Build the reference-side checkers into oracle/_ref/ (test infrastructure).

Two pieces of the MdeT sources are compiled where they lie, without copying
them into this repository:

* openmp/TNF.cpp, the reference's standalone OpenMP TNF counter, built as-is
  (oracle/Makefile target `ref`) -> oracle/_ref/omp_ex;
* the probability functions of cuda/Cuda2.cu -- the coefficient tables and
  cal_tnf_pre_dist_d (device form, cuda/Cuda2.cu:170-241) and cal_tnf_dist
  (host form, cuda/Cuda2.cu:721-779).  Cuda2.cu as a whole needs Boost and a
  GPU, so this script cuts those two spans out of the file at build time into
  oracle/_ref/cuda2_prob.inc and compiles them on the host behind the shim
  oracle/ref_prob_shim.cpp -> oracle/_ref/libref_prob.so;
* the abundance scoring of cuda/Cuda2.cu -- cal_abd_dist2, cal_abd_dist,
  is_nz, cal_abd_corr and the sTNF -> sSCR block of main -- cut the same way
  into oracle/_ref/cuda2_abd.inc and compiled with the reference's own
  cuda/ranker.h behind oracle/ref_abd_shim.cpp (which stands in for Boost's
  normal CDF) -> oracle/_ref/libref_abd.so;
* the dissolving of small bins and the recruiting of leftover and small
  contigs (cuda/Cuda2.cu:2064-2283) with cal_abd_corr, cut the same way into
  oracle/_ref/cuda2_recruit.inc and compiled with cuda/ranker.h behind
  oracle/ref_recruit_shim.cpp -> oracle/_ref/libref_recruit.so;
* label_propagation (cuda/Cuda2.cu:569-656) and the traversal of main that
  calls it (cuda/Cuda2.cu:1980-2061), cut the same way into
  oracle/_ref/cuda2_lp.inc and compiled with cuda/ranker.h behind
  oracle/ref_lp_shim.cpp (which supplies the chi-squared CDF and LOG of
  mdet_gb300/csrc/lp_math.h) -> oracle/_ref/libref_lp.so.

Only runs where the reference is mounted (MDET_REFERENCE or /root/reference).
"""
import os
import re
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REF = os.environ.get("MDET_REFERENCE", "/root/reference")
OUT = os.path.join(HERE, "_ref")


def extract_prob(src: str) -> str:
    start = src.index("__device__ __constant__ double _b1[18]")
    end = src.index("__global__ void get_tnf_graph2")
    dev = src[start:end]
    m = re.search(r"\nDistance cal_tnf_dist\(size_t r1, size_t r2\) \{", src)
    if not m:
        raise RuntimeError("cal_tnf_dist not found")
    i = m.start() + 1
    depth, j = 0, src.index("{", i)
    while True:
        if src[j] == "{":
            depth += 1
        elif src[j] == "}":
            depth -= 1
            if depth == 0:
                break
        j += 1
    host = src[i : j + 1]
    return dev + "\n" + host + "\n"


def cut_block(src: str, head: str) -> str:
    """The function that starts with `head`, through its closing brace."""
    i = src.index(head)
    depth, j = 0, src.index("{", i)
    while True:
        if src[j] == "{":
            depth += 1
        elif src[j] == "}":
            depth -= 1
            if depth == 0:
                return src[i : j + 1]
        j += 1


def extract_abd(src: str) -> str:
    """cal_abd_dist2, cal_abd_dist, is_nz, cal_abd_corr and the sTNF -> sSCR
    block of main, the latter wrapped as sscr_block(Graph&, size_t)."""
    funcs = [
        cut_block(src, "Distance cal_abd_dist2(Normal& p1, Normal& p2) {"),
        cut_block(src, "Distance cal_abd_dist(size_t r1, size_t r2, size_t i, bool& nz) {"),
        cut_block(src, "bool is_nz(size_t r1, size_t r2) {"),
        cut_block(src, "Distance cal_abd_corr(size_t r1, size_t r2, bool is_small = false) {"),
    ]
    a = src.index("// 3. convert sTNF to sSCR")
    b = src.index("std::vector<double>().swap(g.sTNF);", a)
    block = "static void sscr_block(Graph& g, size_t nEdges) {\n" + src[a:b] + "\n}\n"
    return "\n\n".join(funcs) + "\n\n" + block


def extract_recruit(src: str) -> str:
    """cal_abd_corr and the block of main that groups the contigs into bins
    after label propagation, dissolves the small bins and recruits leftover
    and small contigs, wrapped as recruit_block(ClassMap&, mems)."""
    corr = cut_block(src, "Distance cal_abd_corr(size_t r1, size_t r2, bool is_small = false) {")
    a = src.index("        for (size_t i = 0; i < nobs; ++i) {\n            cls[mems[i]].push_back(i);")
    b = src.index("        ABD.clear();", a)
    block = ("static void recruit_block(ClassMap& cls, std::vector<size_t>& mems) {\n" + src[a:b] + "\n}\n")
    return corr + "\n\n" + block


def extract_lp(src: str) -> str:
    """label_propagation and the block of main that traverses the scored
    edges and calls it, the latter wrapped as lp_block(Graph&, nEdges, mems)."""
    lp = cut_block(src, "int label_propagation(Graph& g, std::vector<size_t>& membership, "
                        "std::vector<size_t>& node_order) {")
    a = src.index("            // 4. build sequential graph covering")
    b = src.index("if (++which_p == p_schedule2.size()) break;", a)
    b = src.index("}", b)          # the propagation branch
    b = src.index("}", b + 1)      # the loop over the edges
    block = ("static int lp_block(Graph& g, size_t nEdges, std::vector<size_t>& mems) {\n" + src[a:b + 1]
             + "\n    return 0;\n}\n")
    return lp + "\n\n" + block


def main() -> int:
    cuda2 = os.path.join(REF, "cuda", "Cuda2.cu")
    if not os.path.exists(cuda2):
        print(f"reference not mounted at {REF}; nothing to build", file=sys.stderr)
        return 0
    os.makedirs(OUT, exist_ok=True)
    subprocess.check_call(["make", "-s", "-C", HERE, "all", "ref", f"REF={REF}"])
    with open(cuda2, "r", encoding="utf-8", errors="replace") as f:
        src = f.read()
    inc = os.path.join(OUT, "cuda2_prob.inc")
    with open(inc, "w") as f:
        f.write(extract_prob(src))
    subprocess.check_call([
        "g++", "-O2", "-std=c++17", "-ffp-contract=off", "-fPIC", "-shared",
        f"-I{OUT}", "-o", os.path.join(OUT, "libref_prob.so"),
        os.path.join(HERE, "ref_prob_shim.cpp"),
    ])
    inc = os.path.join(OUT, "cuda2_abd.inc")
    with open(inc, "w") as f:
        f.write(extract_abd(src))
    subprocess.check_call([
        "g++", "-O2", "-std=c++17", "-ffp-contract=off", "-fPIC", "-shared",
        f"-I{OUT}", f"-I{os.path.join(REF, 'cuda')}", "-o", os.path.join(OUT, "libref_abd.so"),
        os.path.join(HERE, "ref_abd_shim.cpp"),
    ])
    inc = os.path.join(OUT, "cuda2_recruit.inc")
    with open(inc, "w") as f:
        f.write(extract_recruit(src))
    subprocess.check_call([
        "g++", "-O2", "-std=c++17", "-ffp-contract=off", "-fPIC", "-shared", "-fopenmp",
        f"-I{OUT}", f"-I{os.path.join(REF, 'cuda')}", "-o", os.path.join(OUT, "libref_recruit.so"),
        os.path.join(HERE, "ref_recruit_shim.cpp"),
    ])
    inc = os.path.join(OUT, "cuda2_lp.inc")
    with open(inc, "w") as f:
        f.write(extract_lp(src))
    subprocess.check_call([
        "g++", "-O2", "-std=c++17", "-ffp-contract=off", "-fPIC", "-shared",
        f"-I{OUT}", f"-I{os.path.join(REF, 'cuda')}", f"-I{os.path.join(HERE, '..', 'mdet_gb300', 'csrc')}",
        "-o", os.path.join(OUT, "libref_lp.so"), os.path.join(HERE, "ref_lp_shim.cpp"),
    ])
    return 0


if __name__ == "__main__":
    sys.exit(main())
