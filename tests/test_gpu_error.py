"""Error of the exact stage against the FP64 oracle: distance and
probability of 10^6 seeded random pairs plus every pair within 1e-3 of the
cutoff or of its row's top-k cutoff, on a 2*10^4-contig, 50-genome set.
The exact stage carries its sums in float-float (about 48 significant
bits).  The distance error stays near 1e-14.  The logistic model sums
polynomial terms of magnitude ~1e5-1e6 down to values of order 10, so even
an FP64 evaluation carries absolute errors near 1e-10 in the
pre-probability; the probability bound asserted is 1e-9."""
import os
import sys

import numpy as np
import pytest

sys.path.insert(0, os.path.dirname(__file__))

from oracle import oracle

pytestmark = pytest.mark.gpu

CUTOFF, K = 0.95, 200


def test_exact_stage_error_vs_fp64(gpu_ctx):
    torch = pytest.importorskip("torch")
    from gpu_util import synth_set

    a, _, tnf = synth_set(seed=31, n=20000, genomes=50)
    ls = a.log_sizes
    n = tnf.shape[0]
    rng = np.random.default_rng(5)
    rnd = rng.integers(0, n, (1_000_000, 2))
    rnd = rnd[rnd[:, 0] != rnd[:, 1]]
    # every pair above cutoff - 1e-3 (no row here has 4096 of them)
    g = gpu_ctx.tnf_graph(tnf, ls, CUTOFF - 1e-3, 4096, mode="bf16")
    fr, to, sim = g.from_.astype(np.int64), g.to.astype(np.int64), g.sTNF
    near = np.abs(sim - CUTOFF) <= 1e-3
    # per-row k-th best probability over both directions
    rows = np.concatenate([fr, to])
    sims2 = np.concatenate([sim, sim])
    order = np.lexsort((-sims2, rows))
    rows_s, sims_s = rows[order], sims2[order]
    start = np.searchsorted(rows_s, np.arange(n))
    cnt = np.bincount(rows_s, minlength=n)
    kth = np.full(n, -1.0)
    has = cnt >= K
    kth[has] = sims_s[start[has] + K - 1]
    band = (np.abs(sim - kth[fr]) <= 1e-3) | (np.abs(sim - kth[to]) <= 1e-3)
    pairs = np.concatenate([rnd, np.stack([fr, to], 1)[near | band]]).astype(np.uint64)
    m = pairs.shape[0]
    dev = torch.device("cuda:0")
    d_tnf = torch.from_numpy(np.ascontiguousarray(tnf)).to(dev)
    d_ls = torch.from_numpy(np.ascontiguousarray(ls)).to(dev)
    d_pairs = torch.from_numpy(pairs.view(np.int64)).to(dev)
    d_dist = torch.zeros(m, dtype=torch.float64, device=dev)
    d_prob = torch.zeros(m, dtype=torch.float64, device=dev)
    torch.cuda.synchronize()
    gpu_ctx.pair_scores_dev(d_tnf.data_ptr(), d_ls.data_ptr(), n, d_pairs.data_ptr(), m, d_dist.data_ptr(),
                            d_prob.data_ptr())
    gd, gp = d_dist.cpu().numpy(), d_prob.cpu().numpy()
    od, op = oracle.pair_scores(tnf, ls, pairs)
    ed, ep = np.abs(gd - od), np.abs(gp - op)
    print(f"pairs {m} (random {rnd.shape[0]}, near cutoff {int(near.sum())}, near top-k {int(band.sum())}): "
          f"max |d err| {ed.max():.3e}, max rel d err {(ed / np.maximum(od, 1e-300)).max():.3e}, "
          f"max |p err| {ep.max():.3e}")
    assert ed.max() <= 1e-12
    assert ep.max() <= 1e-9
