#!/usr/bin/env python3
"""Regenerate tests/golden/abd_golden.npz from the mounted reference.

The reference's own abundance scoring -- cal_abd_dist2, cal_abd_dist, is_nz,
cal_abd_corr and the sTNF -> sSCR block of main (cuda/Cuda2.cu:667-719,
845-856, 1219-1245, 1921-1971) with cuda/ranker.h -- compiled on the host by
oracle/build_ref.py into oracle/_ref/libref_abd.so (Boost's normal CDF stood
in for by its published erfc form), run on seeded inputs:

  abd, var        400 x 5 coverage (mean depth, variance) with edge cases:
                  depths below and at min_cv, zero depths, variances below 1,
                  equal depths and equal variances across a pair
  from_, to       ~2900 edges (no pair of two contigs without a depth above 1,
                  each with a depth above min_cv in the first two samples)
  stnf            sTNF values in (0.5, 1], a fifth of them rounded to 3
                  decimals so that ranks see ties
  sscr5, sscr2    the reference's sSCR with all 5 samples (correlation term
                  used, minSample 3) and with the first 2 (not used)
  nz_pairs, nz    is_nz of 2000 contig pairs

Needs MDET_REFERENCE (default /root/reference); runs here only, its output is
committed.
"""
import ctypes
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)


def ref_lib():
    L = ctypes.CDLL(os.path.join(ROOT, "oracle", "_ref", "libref_abd.so"))
    P, u64, u32, D = ctypes.c_void_p, ctypes.c_uint64, ctypes.c_uint32, ctypes.c_double
    L.ref_sscr.argtypes = [P, P, P, u64, P, P, u32, D, u32, P]
    L.ref_is_nz.argtypes = [P, u32, u64, u64]
    L.ref_is_nz.restype = ctypes.c_int
    return L


def make_inputs(seed=2024):
    from mdet_gb300 import synth

    rng = np.random.default_rng(seed)
    n, nabd, ne = 400, 5, 3000
    genome = rng.integers(0, 12, n)
    abd, var = synth.abundance(genome, nabd, seed, low_frac=0.08)
    abd[rng.random((n, nabd)) < 0.04] = 0.0                           # uncovered samples
    abd[rng.random((n, nabd)) < 0.04] = 1.0                           # exactly min_cv
    var[rng.random((n, nabd)) < 0.1] *= 0.01                          # variances below 1 (clamped)
    low = ~(abd > 1.0).any(1)
    i = rng.integers(0, n, 4 * ne)
    j = rng.integers(0, n, 4 * ne)
    keep = (i != j) & ~(low[i] & low[j])
    i, j = i[keep][:ne], j[keep][:ne]
    fr, to = np.minimum(i, j).astype(np.uint64), np.maximum(i, j).astype(np.uint64)
    # equal depths / equal variances in some pairs' samples
    for e in range(0, ne, 37):
        k = e % nabd
        abd[to[e], k] = abd[fr[e], k]
    for e in range(5, ne, 41):
        k = e % nabd
        var[to[e], k] = var[fr[e], k]
    # float-valued, as the reference's ABD / ABD_VAR matrices are
    abd = abd.astype(np.float32).astype(np.float64)
    var = var.astype(np.float32).astype(np.float64)
    # every edge needs a sample above min_cv in both cases (else the
    # reference divides 0 by 0)
    cov = lambda k: ((abd[to, :k] > 1.0) | (abd[fr, :k] > 1.0)).any(1)
    ok = cov(nabd) & cov(2)
    fr, to = fr[ok], to[ok]
    ne = fr.size
    stnf = rng.uniform(0.5, 1.0, ne)
    q = rng.random(ne) < 0.2
    stnf[q] = np.round(stnf[q], 3)
    return abd, var, fr, to, stnf


def ref_sscr(L, fr, to, stnf, abd, var, min_cv=1.0, min_sample=3):
    abd = np.ascontiguousarray(abd)
    var = np.ascontiguousarray(var)
    out = np.zeros(stnf.size)
    L.ref_sscr(fr.ctypes.data, to.ctypes.data, stnf.ctypes.data, stnf.size, abd.ctypes.data, var.ctypes.data,
               abd.shape[1], min_cv, min_sample, out.ctypes.data)
    return out


def main():
    L = ref_lib()
    abd, var, fr, to, stnf = make_inputs()
    sscr5 = ref_sscr(L, fr, to, stnf, abd, var)
    sscr2 = ref_sscr(L, fr, to, stnf, abd[:, :2], var[:, :2])
    rng = np.random.default_rng(9)
    pairs = rng.integers(0, abd.shape[0], (2000, 2)).astype(np.uint64)
    nz = np.array([L.ref_is_nz(abd.ctypes.data, abd.shape[1], int(a), int(b)) for a, b in pairs], np.uint8)
    np.savez_compressed(os.path.join(HERE, "abd_golden.npz"), abd=abd, var=var, from_=fr, to=to, stnf=stnf,
                        sscr5=sscr5, sscr2=sscr2, nz_pairs=pairs, nz=nz)
    print("abd_golden.npz written:", stnf.size, "edges; pairs rejected by is_nz:", int((nz == 0).sum()))


if __name__ == "__main__":
    main()
