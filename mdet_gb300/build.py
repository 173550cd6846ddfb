"""Build the native parts in-tree (nvcc / gcc / g++, no cmake).

Outputs (git-ignored):
  mdet_gb300/_lib/libmdet_tnf.so    CUDA kernels + C ABI (include/mdet_tnf.h)
  mdet_gb300/_lib/libmdet_synth.so  synthetic-assembly generator
  mdet_gb300/_lib/mdet_tnf          command-line host (MetaBAT2-style flags)

Translation units compile in parallel; a unit is skipped when its object is
newer than the unit and every header it may include.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
OBJ = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "_lib")
NVCC = os.environ.get("NVCC", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CU_UNITS = [
    "ctx",
    "tnf_count",
    "graph_prep",
    "graph_filter_simt",
    "graph_filter_tc",
    "graph_exact",
    "graph",
    "learned",
    "mlp_tc",
    "graph_learned",
    "graph_batch",
    "abundance",
    "fasta_index",
    "recruit",
    "labelprop",
]
# per-unit flags: the abundance, recruiting and label propagation units round
# every product and sum separately (no FMA contraction), as the reference's
# host arithmetic and the host checkers do
UNIT_FLAGS = {"abundance": ["-fmad=false"], "recruit": ["-fmad=false"], "labelprop": ["-fmad=false"]}


def _headers():
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    hs.append(os.path.join(ROOT, "include", "mdet_tnf.h"))
    return hs


def _stale(out, deps):
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"build step failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return r


def build(verbose: bool = False) -> str:
    os.makedirs(OBJ, exist_ok=True)
    os.makedirs(LIB, exist_ok=True)
    hdrs = _headers()
    jobs = []
    for u in CU_UNITS:
        src = os.path.join(CSRC, u + ".cu")
        obj = os.path.join(OBJ, u + ".o")
        if _stale(obj, [src] + hdrs):
            jobs.append([NVCC, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                         *UNIT_FLAGS.get(u, []), f"-I{os.path.join(ROOT, 'include')}", "-c", src, "-o", obj])
    with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 4)) as ex:
        for r in ex.map(_run, jobs):
            if verbose:
                print(r.stdout, r.stderr, end="")
    objs = [os.path.join(OBJ, u + ".o") for u in CU_UNITS]
    so = os.path.join(LIB, "libmdet_tnf.so")
    if _stale(so, objs):
        _run([NVCC, *ARCH, "-shared", "-o", so, *objs])
    synth_src = os.path.join(CSRC, "synth.c")
    synth_so = os.path.join(LIB, "libmdet_synth.so")
    if _stale(synth_so, [synth_src]):
        _run(["gcc", "-O2", "-ffp-contract=off", "-fPIC", "-shared", "-pthread", "-o", synth_so, synth_src, "-lm"])
    cli_src = os.path.join(CSRC, "host_main.cpp")
    cli = os.path.join(LIB, "mdet_tnf")
    if os.path.exists(cli_src) and _stale(cli, [cli_src, so]):
        _run(["g++", "-O2", "-std=c++17", f"-I{os.path.join(ROOT, 'include')}", "-o", cli, cli_src,
              f"-L{LIB}", "-lmdet_tnf", "-Wl,-rpath,$ORIGIN", "-pthread"])
    return so


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
