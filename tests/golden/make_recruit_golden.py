#!/usr/bin/env python3
"""Golden cases for dissolving small bins and recruiting leftover and small
contigs (cuda/Cuda2.cu:2064-2283), produced by the reference's own block
compiled here (oracle/_ref/libref_recruit.so, built by oracle/build_ref.py
where the reference is mounted).  Writes tests/golden/recruit_golden.npz.

Cases (seeded): coverage profiles per synthetic genome with per-contig noise;
labels = genome, plus contigs split off into tiny bins (the leftovers);
some coverage rounded to integers (rank ties), zero rows and constant rows
(undefined correlations), bins under and over ten members, small contigs
drawn from the genomes and from random profiles; the reference run with its
verbose flag on and off (the small-contig gate depends on it); one case whose
recruited leftovers exceed 10 % of the binned bases.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle import oracle  # noqa: E402


def case(seed, n, nabd, genomes, tiny_frac, n_small, small_random_frac, int_frac, min_cls=200000):
    rng = np.random.default_rng(seed)
    gen = rng.integers(0, genomes, n)
    prof = rng.gamma(2.0, 5.0, (genomes, nabd))
    abd = prof[gen] * rng.lognormal(0, 0.35, (n, nabd))
    ints = rng.random(n) < int_frac
    abd[ints] = np.round(abd[ints])
    abd[rng.random(n) < 0.01] = 0.0
    const = rng.random(n) < 0.01
    abd[const] = 3.0
    lab = gen.astype(np.int64)
    tiny = rng.random(n) < tiny_frac
    lab[tiny] = 100000 + np.arange(tiny.sum())
    sizes = rng.integers(2500, 60000, n).astype(np.uint64)
    sgen = rng.integers(0, genomes, n_small)
    small = prof[sgen] * rng.lognormal(0, 0.35, (n_small, nabd))
    rnd = rng.random(n_small) < small_random_frac
    small[rnd] = rng.gamma(2.0, 5.0, (int(rnd.sum()), nabd))
    sround = rng.random(n_small) < 0.3
    small[sround] = np.round(small[sround])
    ssz = rng.integers(1000, 2500, n_small).astype(np.uint64)
    return abd.astype(np.float32), small.astype(np.float32), lab, sizes, ssz, min_cls


def main():
    cases = {
        "a": case(1, 3000, 6, 40, 0.05, 3000, 0.9, 0.2),
        "b": case(2, 2500, 10, 25, 0.03, 400, 0.1, 0.0),
        "c": case(3, 1200, 3, 12, 0.25, 0, 0.0, 0.5),   # many leftovers: > 10 % of the binned bases
        "d": case(4, 900, 20, 70, 0.1, 800, 0.5, 0.1),  # bins under ten members
    }
    out = {}
    for name, (abd, small, lab, sz, ssz, min_cls) in cases.items():
        for verb in (0, 1):
            o, so = oracle.ref_recruit(abd, small, lab, sz, ssz, min_cls, verbose=bool(verb))
            out[f"{name}_out_v{verb}"] = o
            out[f"{name}_small_out_v{verb}"] = so
        out[f"{name}_abd"] = abd
        out[f"{name}_small"] = small
        out[f"{name}_label"] = lab
        out[f"{name}_sizes"] = sz
        out[f"{name}_small_sizes"] = ssz
        out[f"{name}_min_cls"] = np.array([min_cls], np.uint64)
    np.savez_compressed(os.path.join(HERE, "recruit_golden.npz"), **out)
    print("wrote", os.path.join(HERE, "recruit_golden.npz"))


if __name__ == "__main__":
    main()
