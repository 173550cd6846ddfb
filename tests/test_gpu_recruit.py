"""Dissolving small bins and recruiting leftover / small contigs on the GPU
(mdet_recruit) against the reference's own block (golden cases) and against
the oracle on a larger seeded set: bin labels identical for every contig
(the correlations and their sums are computed in the reference's order, so
the >= tests decide identically)."""
import os

import numpy as np
import pytest

from oracle import oracle

pytestmark = pytest.mark.gpu

G = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "recruit_golden.npz")


@pytest.mark.parametrize("name", ["a", "b", "c", "d"])
@pytest.mark.parametrize("verbose", [0, 1])
def test_recruit_golden(gpu_ctx, name, verbose):
    z = np.load(G)
    ssz = z[f"{name}_small_sizes"]
    out, sout, st = gpu_ctx.recruit(z[f"{name}_abd"], z[f"{name}_small"], z[f"{name}_label"], z[f"{name}_sizes"],
                                    ssz, int(z[f"{name}_min_cls"][0]), int(ssz.sum()) if verbose else 0)
    assert np.array_equal(out, z[f"{name}_out_v{verbose}"])
    assert np.array_equal(sout, z[f"{name}_small_out_v{verbose}"])


@pytest.mark.parametrize("nabd", [10, 48])
def test_recruit_synthetic_vs_oracle(gpu_ctx, nabd):
    """Also checks that the FP32 prefilter decides most pairs (10 samples:
    the contig's row kept in registers; 48: read from memory)."""
    from mdet_gb300 import synth

    a = synth.generate(seed=61, n=12000, genomes=60, threads=8)
    rng = np.random.default_rng(5)
    n1 = 3000
    sg = rng.integers(0, 60, n1).astype(np.uint32)
    both, _ = synth.abundance(np.concatenate([a.genome, sg]), nabd, 61)  # one depth profile per genome
    abd, sabd = both[:a.genome.size], both[a.genome.size:]
    label = a.genome.astype(np.int64)
    tiny = rng.random(label.size) < 0.02
    label[tiny] = 10000 + np.arange(tiny.sum())
    ssz = rng.integers(1000, 2500, n1)
    sizes = a.sizes.astype(np.uint64)
    for small_total in (0, int(ssz.sum()) * 20):
        want, swant, wst = oracle.recruit(abd, sabd, label, sizes, ssz, 200000, small_total)
        got, sgot, st = gpu_ctx.recruit(abd, sabd, label, sizes, ssz, 200000, small_total)
        assert np.array_equal(got, want)
        assert np.array_equal(sgot, swant)
        assert st["n_leftovers"] == wst["leftovers"] and st["n_leftovers_matched"] == wst["leftovers_matched"]
        assert st["n_small_matched"] == wst["small_matched"]
        assert st["pairs_tested"] == (wst["leftovers"] + n1) * st["n_bins_scored"]
        assert st["n_leftovers_matched"] + st["n_small_matched"] <= st["pairs_exact"] < st["pairs_tested"] // 4
    assert wst["leftovers_matched"] > 0 and wst["small_matched"] > 0


def test_recruit_rejects_bad_sizes(gpu_ctx):
    from mdet_gb300 import MdetError

    with pytest.raises(MdetError):
        gpu_ctx.recruit(np.zeros((4, 300), np.float32), np.zeros((0, 300), np.float32), np.zeros(4, np.int64),
                        np.ones(4, np.uint64), np.zeros(0, np.uint64))


@pytest.mark.parametrize("scale,cap", [("1e5", "0"), ("1e10", "0"), ("1e10", "30000"), ("1e10", "10000")])
def test_recruit_refined_means(gpu_ctx, scale, cap, monkeypatch):
    """Tests decided with the bins' refined means: estimate intervals
    widened 10^5-fold leave many tests to the FP64-term estimates, widened
    10^10-fold to the exact means -- with the term buffer at its default, at
    30,000 terms (200-member bins of 19,900 terms, one run each) and at
    10,000 (every bin by the large-bin warp) -- the same bins as the oracle
    every time."""
    from mdet_gb300 import synth

    a = synth.generate(seed=62, n=6000, genomes=30, threads=8)
    rng = np.random.default_rng(6)
    n1 = 800
    sg = rng.integers(0, 30, n1).astype(np.uint32)
    both, _ = synth.abundance(np.concatenate([a.genome, sg]), 12, 62)
    abd, sabd = both[:a.genome.size], both[a.genome.size:]
    label = a.genome.astype(np.int64)
    tiny = rng.random(label.size) < 0.03
    label[tiny] = -1 - np.arange(tiny.sum())
    ssz = rng.integers(1000, 2500, n1)
    sizes = a.sizes.astype(np.uint64)
    small_total = int(ssz.sum()) * 20
    want, swant, _ = oracle.recruit(abd, sabd, label, sizes, ssz, 200000, small_total)
    got, sgot, st0 = gpu_ctx.recruit(abd, sabd, label, sizes, ssz, 200000, small_total)
    assert np.array_equal(got, want) and np.array_equal(sgot, swant)
    monkeypatch.setenv("MDET_RECRUIT_EPS_SCALE", scale)
    if cap != "0":
        monkeypatch.setenv("MDET_RECRUIT_TERM_CAP", cap)
    got, sgot, st = gpu_ctx.recruit(abd, sabd, label, sizes, ssz, 200000, small_total)
    assert np.array_equal(got, want) and np.array_equal(sgot, swant)
    assert st["n_leftovers_matched"] > 0
    assert st["pairs_undecided"] > st0["pairs_undecided"]
    if scale == "1e10":
        assert st["bins_exact"] > st0["bins_exact"]


def test_recruit_degenerate_rows(gpu_ctx):
    """Constant depth rows (sx = 0: the reference's correlations with them
    are NaN) in some bins and among the leftovers: those bins get their exact
    means, and the bins equal the oracle's."""
    rng = np.random.default_rng(8)
    n, nabd = 3000, 8
    label = rng.integers(0, 12, n).astype(np.int64)
    prof = rng.lognormal(2, 1, (12, nabd))
    abd = (prof[label] * rng.lognormal(0, 0.2, (n, nabd))).astype(np.float32)
    abd[rng.random(n) < 0.01] = 3.0
    lone = rng.random(n) < 0.05
    label[lone] = 100 + np.arange(lone.sum())
    sizes = rng.integers(20000, 60000, n).astype(np.uint64)
    sabd = (prof[rng.integers(0, 12, 300)] * rng.lognormal(0, 0.2, (300, nabd))).astype(np.float32)
    sabd[:5] = 0
    ssz = rng.integers(1000, 2500, 300).astype(np.uint64)
    small_total = int(ssz.sum()) * 20
    want, swant, _ = oracle.recruit(abd, sabd, label, sizes, ssz, 200000, small_total)
    got, sgot, st = gpu_ctx.recruit(abd, sabd, label, sizes, ssz, 200000, small_total)
    assert np.array_equal(got, want) and np.array_equal(sgot, swant)
    assert st["bins_exact"] > 0 and st["n_leftovers_matched"] > 0
