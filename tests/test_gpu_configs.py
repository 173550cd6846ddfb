"""Edge-set parity at the workload configurations' own sizes.

Config 0: 20,000 contigs from 50 Markov genomes (generator seed 0), the whole
graph against the oracle, at the pinned cutoff (--pTNF 95) and at the cutoff
the pTNF search finds (maxP 95), in the tensor-core form and, at the pinned
cutoff, the plain form.  Config 1: 200,000 contigs from 500 genomes (seed 1),
counts of a contig sample bit-exact against the oracle, and 2,000 rows in
four seeded blocks of 500 -- each row's top-200 against all 200,000 columns
-- against the oracle.  Both: edges identical outside the 1e-5 band (the
band's exemptions are counted), sTNF within 1e-9."""
import numpy as np
import pytest

from oracle import oracle, parity

pytestmark = pytest.mark.gpu

K = 200


@pytest.fixture(scope="module")
def config0():
    from mdet_gb300 import synth

    a = synth.generate(seed=0, n=20000, genomes=50, threads=16)
    counts, tnf = oracle.tnf_count(a.data, a.seq_off, a.seq_len)
    return a, counts, tnf


def test_config0_counts(gpu_ctx, config0):
    a, counts, tnf = config0
    c, t = gpu_ctx.tnf_count(a.data, a.seq_off, a.seq_len)
    assert np.array_equal(c, counts)
    assert np.allclose(t, tnf, rtol=1e-6, atol=0)


@pytest.mark.parametrize("mode", ["bf16", "tf32", "plain"])
def test_config0_graph_pinned_cutoff(gpu_ctx, config0, mode):
    a, _, tnf = config0
    g = gpu_ctx.tnf_graph(tnf, a.log_sizes, 0.95, K, mode=mode)
    r = parity.compare_rows(g.from_, g.to, g.sTNF, tnf, a.log_sizes, 0.95, K)
    parity.assert_rows_match(r)
    assert r["recall"] >= 0.999 and r["ref_edges"] > 100000
    print(mode, {k: v for k, v in r.items() if k != "outside_band"})


def test_config0_graph_searched_cutoff(gpu_ctx, config0):
    a, _, tnf = config0
    want = oracle.ptnf_search(tnf, a.log_sizes, 0.95, seed=1234)
    oracle.srand(1234)
    p = gpu_ctx.ptnf_search(tnf, a.log_sizes, 0.95, mode="bf16")
    assert p == want
    cut = p / 1000.0
    g = gpu_ctx.tnf_graph(tnf, a.log_sizes, cut, K, mode="bf16")
    r = parity.compare_rows(g.from_, g.to, g.sTNF, tnf, a.log_sizes, cut, K)
    parity.assert_rows_match(r)
    assert r["recall"] >= 0.999
    print(p, {k: v for k, v in r.items() if k != "outside_band"})


def test_config1_sampled_rows(gpu_ctx):
    from mdet_gb300 import synth

    n = 200000
    a = synth.generate(seed=1, n=n, genomes=500, threads=16)
    counts, tnf = gpu_ctx.tnf_count(a.data, a.seq_off, a.seq_len)
    rng = np.random.default_rng(11)
    sample = np.sort(rng.choice(n, 3000, replace=False))
    oc, ot = oracle.tnf_count(a.data, a.seq_off[sample], a.seq_len[sample])
    assert np.array_equal(counts[sample], oc)
    assert np.allclose(tnf[sample], ot, rtol=1e-6, atol=0)
    g = gpu_ctx.tnf_graph(tnf, a.log_sizes, 0.95, K, mode="bf16")
    total = {"ref_edges": 0, "common": 0, "band_exempt": 0}
    for r0 in np.sort(rng.choice(n - 500, 4, replace=False)):
        r = parity.compare_rows(g.from_, g.to, g.sTNF, tnf, a.log_sizes, 0.95, K, int(r0), int(r0) + 500)
        parity.assert_rows_match(r)
        for k in total:
            total[k] += r[k]
    assert total["ref_edges"] > 10000
    assert total["common"] / total["ref_edges"] >= 0.999
    print(total)
