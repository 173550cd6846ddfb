"""Row shards of the graph (mdet_tnf_graph_shard): every shard's edges come
from its own block of size-sorted rows, match the oracle for those rows, and
the shards together equal the whole graph bit for bit."""
import numpy as np
import pytest

from oracle import oracle

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def set_s():
    from mdet_gb300 import synth

    a = synth.generate(seed=44, n=2600, genomes=30, threads=8)
    _, tnf = oracle.tnf_count(a.data, a.seq_off, a.seq_len)
    return a, tnf


@pytest.mark.parametrize("mode", ["bf16", "plain"])
@pytest.mark.parametrize("nshards", [1, 2, 3, 7])
def test_shards_make_the_whole_graph(gpu_ctx, set_s, mode, nshards):
    from mdet_gb300 import shard

    a, tnf = set_s
    full = gpu_ctx.tnf_graph(tnf, a.log_sizes, 0.9, 60, mode=mode)
    want = dict(zip(zip(full.from_.tolist(), full.to.tolist()), full.sTNF.tolist()))
    got = {}
    for k in range(nshards):
        g = gpu_ctx.tnf_graph_shard(tnf, a.log_sizes, 0.9, 60, mode, k, nshards)
        rows = set(shard.shard_rows(a.log_sizes, k, nshards).tolist())
        assert set(g.from_.tolist()) <= rows
        for f, t, s in zip(g.from_.tolist(), g.to.tolist(), g.sTNF.tolist()):
            assert (f, t) not in got
            got[(f, t)] = s
    assert got == want


def test_shard_matches_oracle_rows(gpu_ctx, set_s):
    from mdet_gb300 import shard

    a, tnf = set_s
    rows = shard.shard_rows(a.log_sizes, 1, 3)
    g = gpu_ctx.tnf_graph_shard(tnf, a.log_sizes, 0.95, 200, "bf16", 1, 3)
    fr, to, st = oracle.graph_rows(tnf, a.log_sizes, 0.95, 200, rows)
    assert set(zip(g.from_.tolist(), g.to.tolist())) == set(zip(fr.tolist(), to.tolist()))


def test_shard_arguments(gpu_ctx, set_s):
    from mdet_gb300 import MdetError

    a, tnf = set_s
    with pytest.raises(MdetError):
        gpu_ctx.tnf_graph_shard(tnf, a.log_sizes, 0.9, 60, "bf16", 3, 3)
    with pytest.raises(MdetError):
        gpu_ctx.tnf_graph_shard(tnf, a.log_sizes, 0.9, 600, "bf16", 0, 2)
