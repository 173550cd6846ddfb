#!/usr/bin/env python3
"""Regenerate the golden fixtures of tests/golden/ from the mounted reference.

Needs the MdeT sources (MDET_REFERENCE, default /root/reference) and runs
only here, never on the GPU machine; its outputs are committed.

  ref_tables.json     TN column order (openmp/TNF.cpp:14-24), TNmap_d and BN
                      tables (cuda/Cuda2.cu:149-168) parsed from the sources
  count_*.fa(.gz)     FASTA inputs: one synthetic, one of edge cases
  count_*_tnf.npy     TNF.bin written by the unmodified openmp/TNF.cpp
                      (built by oracle/build_ref.py) on that FASTA
  prob_golden.npz     pre-probabilities / probabilities of random pairs from
                      the reference's own cal_tnf_pre_dist_d and cal_tnf_dist
                      compiled on the host (oracle/_ref/libref_prob.so)
"""
import ctypes
import gzip
import json
import os
import re
import shutil
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
REF = os.environ.get("MDET_REFERENCE", "/root/reference")


def parse_tables():
    tnf_cpp = open(os.path.join(REF, "openmp", "TNF.cpp")).read()
    m = re.search(r"static const std::string TN\[\] = \{(.*?)\};", tnf_cpp, re.S)
    tn = re.findall(r'"([ACGT]{4})"', m.group(1))
    m = re.search(r"static const std::string TNP\[\] = \{(.*?)\};", tnf_cpp, re.S)
    tnp = re.findall(r'"([ACGT]{4})"', m.group(1))
    cuda2 = open(os.path.join(REF, "cuda", "Cuda2.cu")).read()
    m = re.search(r"const unsigned char TNmap_d\[256\] = \{(.*?)\};", cuda2, re.S)
    tnmap = [int(x) for x in re.findall(r"\d+", m.group(1))]
    m = re.search(r"const unsigned char BN\[256\] = \{(.*?)\};", cuda2, re.S)
    bn = [int(x) for x in re.findall(r"\d+", m.group(1))]
    assert len(tn) == 136 and len(tnp) == 16 and len(tnmap) == 256 and len(bn) == 256
    return {"tn_order": tn, "palindromes": tnp, "tnmap": tnmap, "bn": bn}


def edge_case_fasta() -> bytes:
    """Hand-made records that exercise the counting rules (LF endings)."""
    rng = np.random.default_rng(20240607)

    def bases(n, alphabet="ACGT"):
        return "".join(rng.choice(list(alphabet), n))

    def wrap(s, w):
        return "\n".join(s[i:i + w] for i in range(0, len(s), w)) + "\n"

    recs = []
    recs.append((">plain60 desc text", wrap(bases(3000), 60)))
    recs.append((">lower", wrap(bases(2800).lower(), 70)))
    mixed = list(bases(4000))
    for i in rng.choice(4000, 400, replace=False):
        mixed[i] = mixed[i].lower()
    recs.append((">mixedcase", wrap("".join(mixed), 80)))
    s = list(bases(3500))
    for start in (10, 500, 501, 2000):
        for k in range(start, start + 7):
            s[k] = "N"
    recs.append((">nruns", wrap("".join(s), 60)))
    s = list(bases(3200))
    for i in rng.choice(3200, 60, replace=False):
        s[i] = rng.choice(list("RYKMSWBDHVN"))
    recs.append((">iupac", wrap("".join(s), 61)))
    recs.append((">width1", wrap(bases(2600), 1)))
    recs.append((">width3", wrap(bases(2700), 3)))
    recs.append((">width4", wrap(bases(2650), 4)))
    recs.append((">oneline", bases(5000) + "\n"))
    recs.append((">long_multi_piece", wrap(bases(70000), 60)))
    recs.append((">poly_a", wrap("A" * 2600, 60)))
    recs.append((">blank_lines", "\n".join([bases(40), "", bases(1400), "", "", bases(1300)]) + "\n"))
    recs.append((">no_trailing_newline", wrap(bases(2900), 60)[:-1]))
    return "".join(h + "\n" + b for h, b in recs).encode()


def run_tnf_cpp(fasta_path: str) -> np.ndarray:
    exe = os.path.join(ROOT, "oracle", "_ref", "omp_ex")
    with tempfile.TemporaryDirectory() as d:
        subprocess.check_call([exe, "4", os.path.abspath(fasta_path)], cwd=d, stdout=subprocess.DEVNULL)
        raw = np.fromfile(os.path.join(d, "TNF.bin"), dtype=np.float64)
    return raw.reshape(-1, 136)


def main():
    subprocess.check_call([sys.executable, os.path.join(ROOT, "oracle", "build_ref.py")])
    subprocess.check_call([sys.executable, "-m", "mdet_gb300.build"], cwd=ROOT)
    with open(os.path.join(HERE, "ref_tables.json"), "w") as f:
        json.dump(parse_tables(), f)

    from mdet_gb300 import synth

    a = synth.generate(seed=11, n=120, genomes=8, max_len=20000, threads=4)
    fa = os.path.join(HERE, "count_synth.fa.gz")
    with open(fa, "wb") as raw, gzip.GzipFile(fileobj=raw, mode="wb", compresslevel=9, mtime=0) as f:
        f.write(a.data.tobytes())
    np.save(os.path.join(HERE, "count_synth_tnf.npy"), run_tnf_cpp(fa))

    ec = os.path.join(HERE, "count_edge.fa")
    with open(ec, "wb") as f:
        f.write(edge_case_fasta())
    np.save(os.path.join(HERE, "count_edge_tnf.npy"), run_tnf_cpp(ec))

    # reference probability functions on random pairs drawn from synthetic TNF rows
    ref = ctypes.CDLL(os.path.join(ROOT, "oracle", "_ref", "libref_prob.so"))
    for fn in ("ref_pre_prob", "ref_tnf_dist"):
        getattr(ref, fn).restype = ctypes.c_double
        getattr(ref, fn).argtypes = [ctypes.c_double, ctypes.c_double, ctypes.c_void_p, ctypes.c_void_p]
    from oracle import oracle

    b = synth.generate(seed=12, n=600, genomes=20, max_len=500000, threads=4)
    _, tnf = oracle.tnf_count(b.data, b.seq_off, b.seq_len)
    rng = np.random.default_rng(5)
    npairs = 1200
    i = rng.integers(0, b.sizes.size, npairs)
    j = rng.integers(0, b.sizes.size, npairs)
    same = b.genome[i] == b.genome[j]
    r1 = b.log_sizes[i].copy()
    r2 = b.log_sizes[j].copy()
    # a few exact-boundary sizes
    r1[:20] = np.log10(2500.0)
    r2[10:30] = np.log10(500000.0)
    A = tnf[i]
    B = tnf[j]
    pre = np.array([ref.ref_pre_prob(r1[k], r2[k], A[k].ctypes.data, B[k].ctypes.data) for k in range(npairs)])
    prob = np.array([ref.ref_tnf_dist(r1[k], r2[k], A[k].ctypes.data, B[k].ctypes.data) for k in range(npairs)])
    np.savez_compressed(os.path.join(HERE, "prob_golden.npz"), a=A, b=B, r1=r1, r2=r2, pre=pre, prob=prob, same=same)
    print("golden fixtures written; same-genome pairs:", int(same.sum()))


if __name__ == "__main__":
    main()
