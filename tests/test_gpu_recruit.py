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


def test_recruit_synthetic_vs_oracle(gpu_ctx):
    from mdet_gb300 import synth

    a = synth.generate(seed=61, n=12000, genomes=60, threads=8)
    rng = np.random.default_rng(5)
    n1 = 3000
    sg = rng.integers(0, 60, n1).astype(np.uint32)
    both, _ = synth.abundance(np.concatenate([a.genome, sg]), 10, 61)  # one depth profile per genome
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
    assert wst["leftovers_matched"] > 0 and wst["small_matched"] > 0


def test_recruit_rejects_bad_sizes(gpu_ctx):
    from mdet_gb300 import MdetError

    with pytest.raises(MdetError):
        gpu_ctx.recruit(np.zeros((4, 300), np.float32), np.zeros((0, 300), np.float32), np.zeros(4, np.int64),
                        np.ones(4, np.uint64), np.zeros(0, np.uint64))
