"""Edge-set parity of a GPU graph against the oracle, row by row.

TEST INFRASTRUCTURE ONLY: used by tests/ and by the CPU-baseline leg of
bench.py (which already runs the oracle over the rows it compares).

The contract (cuda/Cuda2.cu:921-946): the reference emits (i, j, sTNF) for
i < j when j is among row i's top-`max_edges` columns by similarity (strict
'>' replacement, nonzero similarities above the cutoff only).  Every edge is
therefore attributable to its row i = from, and a set of rows can be checked
on its own.  Edge sets must agree except for pairs whose probability lies
within BAND of the cutoff or of row i's top-k cutoff; common edges must
agree on sTNF within SIM_TOL.
"""
from __future__ import annotations

import numpy as np

from oracle import oracle

BAND = 1e-5     # probability band around the cutoff and each row's k-th similarity
SIM_TOL = 1e-9  # sTNF of an edge both sides emit


def compare_rows(gpu_from, gpu_to, gpu_sim, tnf, ls, cutoff, max_edges, row0=0, row1=None, low=None, threads=0,
                 ref=None):
    """Compares the GPU edges whose `from` lies in [row0, row1) with the
    oracle's top-k of those rows (`ref`: that oracle.topk_rows result when
    the caller already has it).  gpu_* may hold edges of other rows too
    (they are ignored).  Returns a dict: ref/got/common edge counts, the
    edges missed and extra, how many of those lie inside the band, the
    largest sTNF difference of common edges, recall and precision."""
    tnf = np.ascontiguousarray(tnf, np.float32)
    ls = np.ascontiguousarray(ls, np.float64)
    n = tnf.shape[0]
    row1 = n if row1 is None else min(row1, n)
    if ref is None:
        ref = oracle.topk_rows(tnf, ls, cutoff, max_edges, row0, row1, threads=threads, low=low)
    rp, cols, sims = ref
    rp = rp.astype(np.int64)
    counts = np.diff(rp)
    rows = np.repeat(np.arange(row0, row1, dtype=np.int64), counts)
    cols = cols[:rp[-1]].astype(np.int64)
    sims = sims[:rp[-1]]
    # k-th similarity of full rows (the row's top-k cutoff), -inf otherwise
    kth = np.full(row1 - row0, -np.inf)
    nonempty = counts > 0
    if nonempty.any():
        # per nonempty row: [start_k, start_{k+1}) is exactly that row's entries
        mins = np.minimum.reduceat(sims, rp[:-1][nonempty])
        full = counts[nonempty] == max_edges
        kth[np.flatnonzero(nonempty)[full]] = mins[full]
    keep = cols > rows
    ref_key = rows[keep] * n + cols[keep]
    ref_sim = sims[keep]
    f = np.asarray(gpu_from, np.int64)
    t = np.asarray(gpu_to, np.int64)
    s = np.asarray(gpu_sim, np.float64)
    sel = (f >= row0) & (f < row1)
    got_key = f[sel] * n + t[sel]
    got_sim = s[sel]
    assert np.all(t[sel] > f[sel]), "GPU edge with to <= from"
    assert np.unique(got_key).size == got_key.size, "duplicate edges in GPU output"
    o_r = np.argsort(ref_key)
    ref_key, ref_sim = ref_key[o_r], ref_sim[o_r]
    o_g = np.argsort(got_key)
    got_key, got_sim = got_key[o_g], got_sim[o_g]
    common, ir, ig = np.intersect1d(ref_key, got_key, assume_unique=True, return_indices=True)
    missed = np.setdiff1d(ref_key, got_key, assume_unique=True)
    extra = np.setdiff1d(got_key, ref_key, assume_unique=True)
    diff = np.concatenate([missed, extra])
    exempt = 0
    n_outside = 0
    outside = []
    if diff.size:
        pairs = np.stack([diff // n, diff % n], axis=1).astype(np.uint64)
        _, p = oracle.pair_scores(tnf, ls, pairs, threads=threads)
        k = kth[(diff // n) - row0]
        near = (np.abs(p - cutoff) <= BAND) | (np.abs(p - k) <= BAND)
        exempt = int(near.sum())
        n_outside = int((~near).sum())
        outside = [(int(a // n), int(a % n), float(pp)) for a, pp, nr in zip(diff, p, near) if not nr][:10]
    max_sim_diff = float(np.abs(ref_sim[ir] - got_sim[ig]).max()) if common.size else 0.0
    n_ref, n_got = int(ref_key.size), int(got_key.size)
    return {
        "rows": int(row1 - row0),
        "ref_edges": n_ref,
        "gpu_edges": n_got,
        "common": int(common.size),
        "missed": int(missed.size),
        "extra": int(extra.size),
        "band_exempt": exempt,
        "n_outside_band": n_outside,
        "outside_band": outside,
        "max_sim_diff": max_sim_diff,
        "recall": (common.size / n_ref) if n_ref else 1.0,
        "precision": (common.size / n_got) if n_got else 1.0,
    }


def assert_rows_match(res, max_exempt_frac=1e-3):
    """The parity contract on a compare_rows result."""
    assert not res["outside_band"], f"edges differ outside the band: {res['outside_band']}"
    assert res["max_sim_diff"] <= SIM_TOL, f"sTNF differs by {res['max_sim_diff']}"
    assert res["band_exempt"] <= max(2, int(max_exempt_frac * max(res["ref_edges"], 1))), res
