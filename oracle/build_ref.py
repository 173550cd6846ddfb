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
  oracle/ref_prob_shim.cpp -> oracle/_ref/libref_prob.so.

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
    return 0


if __name__ == "__main__":
    sys.exit(main())
