#!/usr/bin/env python3
"""Golden vectors for label propagation (tests/golden/lp_golden.npz).

Runs the reference's own traversal and label_propagation -- cut out of
cuda/Cuda2.cu and compiled behind oracle/ref_lp_shim.cpp by
oracle/build_ref.py into oracle/_ref/libref_lp.so -- on seeded inputs, and
stores inputs and bins.  Scores are distinct within each case (the
reference's std::sort leaves the order of equal scores open).  Cases:
  planted   900 contigs in 12 planted groups, 6 draws each, 20 % of the
            in-group scores within 1e-9..1e-15 of 1 (saturated CDFs, exact ties)
  tnf       the TNF graph (cutoff 0.9, 200 edges) of a 1,000-contig synthetic
            assembly of 10 genomes, sSCR = sTNF
  strict    the tnf graph at max_p 0.9, min_s 0.95 (early stop)
Each case stores its graph's name, n, max_p, min_s, the reference's number of
propagation calls and its bins.
Run where the reference is mounted: python tests/golden/make_lp_golden.py
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from mdet_gb300 import synth  # noqa: E402
from oracle import oracle  # noqa: E402


def planted(seed, n, groups, draws, sat=0.2):
    rng = np.random.default_rng(seed)
    g = rng.integers(0, groups, n)
    fr, to, sc = [], [], []
    for v in range(n):
        for _ in range(draws):
            if rng.random() < 0.9:
                u = int(rng.choice(np.flatnonzero(g == g[v])))
                s = rng.uniform(0.7, 1.0)
                if rng.random() < sat:
                    s = 1 - 10 ** rng.uniform(-15, -9)
            else:
                u = int(rng.integers(0, n))
                s = rng.uniform(0.3, 0.85)
            if u != v:
                fr.append(min(u, v))
                to.append(max(u, v))
                sc.append(s)
    return distinct(np.array(fr, np.uint64), np.array(to, np.uint64), np.array(sc))


def distinct(fr, to, sc):
    _, first = np.unique(sc, return_index=True)
    keep = np.sort(first)
    return fr[keep], to[keep], sc[keep]


def main():
    graphs = {"planted": planted(7, 900, 12, 6)}
    a = synth.generate(seed=31, n=1000, genomes=10, max_len=60000, threads=4)
    _, tnf = oracle.tnf_count(a.data, a.seq_off, a.seq_len, threads=4)
    gf, gt, gs = oracle.graph(tnf, a.log_sizes, 0.9, 200)
    graphs["tnf"] = distinct(gf.astype(np.uint64), gt.astype(np.uint64), gs)
    cases = {"planted": ("planted", 900, 0.95, 0.60), "tnf": ("tnf", 1000, 0.95, 0.60),
             "strict": ("tnf", 1000, 0.90, 0.95)}
    out = {}
    for name, (f, t, s) in graphs.items():
        out[f"g_{name}_from"], out[f"g_{name}_to"], out[f"g_{name}_sscr"] = f, t, s
    for name, (gname, n, mp, ms) in cases.items():
        f, t, s = graphs[gname]
        mem, calls = oracle.ref_label_prop(f, t, s, n, mp, ms)
        out[f"{name}_graph"] = np.array(gname)
        out[f"{name}_params"] = np.array([n, mp, ms, calls], np.float64)
        out[f"{name}_mem"] = mem.astype(np.uint32)
        print(name, len(s), "edges,", calls, "calls,", len(np.unique(mem)), "bins")
    np.savez_compressed(os.path.join(os.path.dirname(os.path.abspath(__file__)), "lp_golden.npz"), **out)


if __name__ == "__main__":
    main()
