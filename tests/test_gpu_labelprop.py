"""Label propagation on the GPU (mdet_label_propagation): bins equal to the
reference's own traversal (golden vectors from the reference compiled here)
and to the oracle restatement -- with exact ties broken by the map order, a
contig with more than 2,048 traversal edges (the global-memory sort), equal
scores (taken in edge order by both), early stops and degenerate inputs."""
import os
import sys

import numpy as np
import pytest

sys.path.insert(0, os.path.dirname(__file__))

from oracle import oracle
from test_lp_oracle import G, _case, _planted

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", ["planted", "tnf", "strict"])
def test_equals_reference_golden(gpu_ctx, name):
    z = np.load(G)
    f, t, s, n, mp, ms, calls, want = _case(z, name)
    mem, st = gpu_ctx.label_propagation(f, t, s, n, mp, ms)
    assert st["calls"] == calls
    assert np.array_equal(mem, want.astype(np.uint64))


@pytest.mark.parametrize("seed", [1, 2, 3, 4])
def test_equals_oracle_with_ties(gpu_ctx, seed):
    f, t, s = _planted(seed, 400 + 200 * seed, 4 + seed, 6, 0.4)
    n = 400 + 200 * seed
    ties = 0
    for mp, ms in [(0.95, 0.6), (0.8, 0.75)]:
        want, ost = oracle.label_prop(f, t, s, n, mp, ms)
        got, st = gpu_ctx.label_propagation(f, t, s, n, mp, ms)
        assert np.array_equal(got, want)
        for k in ("calls", "sweeps", "graph_edges", "connected", "frozen"):
            assert st[k] == ost[k], (k, st, ost)
        ties += st["ties"]
    assert ties > 0   # exact ties were broken by the map order on the GPU


def test_equal_scores_in_edge_order(gpu_ctx):
    rng = np.random.default_rng(9)
    f, t, s = _planted(9, 700, 7, 6, 0.2)
    s = np.round(s, 2)   # many equal scores
    want, _ = oracle.label_prop(f, t, s, 700)
    got, _ = gpu_ctx.label_propagation(f, t, s, 700)
    assert np.array_equal(got, want)
    perm = rng.permutation(s.size)   # another edge order: both follow it
    want, _ = oracle.label_prop(f[perm], t[perm], s[perm], 700)
    got, _ = gpu_ctx.label_propagation(f[perm], t[perm], s[perm], 700)
    assert np.array_equal(got, want)


def test_hub_contig_uses_global_sort(gpu_ctx):
    """Contig 0's 3,000 edges score highest, so all join the traversal graph
    before the first propagation run (at 10 % of 40,000 contigs): more edges
    than a block sorts in shared memory.  The other contigs pair up within 400
    groups at lower scores."""
    rng = np.random.default_rng(21)
    n, hub = 40000, 3000
    fr = [0] * hub
    to = list(range(1, hub + 1))
    sc = list(rng.uniform(0.97, 0.999, hub))
    grp = rng.integers(0, 400, n)
    for v in range(1, n):
        u = int(rng.integers(1, n))
        u = u if grp[u] == grp[v] else int(rng.choice(np.flatnonzero(grp == grp[v])[:50]))
        if u not in (0, v):
            fr.append(min(u, v))
            to.append(max(u, v))
            sc.append(rng.uniform(0.7, 0.95))
    f, t, s = np.array(fr, np.uint64), np.array(to, np.uint64), np.array(sc)
    want, ost = oracle.label_prop(f, t, s, n, 1.0, 0.6)
    got, st = gpu_ctx.label_propagation(f, t, s, n, 1.0, 0.6)
    assert st["degree_max"] > 2048
    assert np.array_equal(got, want)


def test_tnf_graph_scale(gpu_ctx):
    """The oracle's TNF graph of a 6,000-contig assembly, sSCR = sTNF."""
    from gpu_util import synth_set

    a, _, tnf = synth_set(seed=77, n=6000, genomes=40, max_len=100000)
    f, t, s = oracle.graph(tnf, a.log_sizes, 0.9, 200)
    want, ost = oracle.label_prop(f, t, s, 6000)
    got, st = gpu_ctx.label_propagation(f, t, s, 6000)
    assert np.array_equal(got, want)
    assert st["calls"] == ost["calls"] and st["sweeps"] == ost["sweeps"]


def test_config0_scored_graph(gpu_ctx):
    """The plain config's assembly (20,000 contigs, 50 genomes) through the
    whole binning front: the GPU's gated graph and its sSCR with 10 samples of
    depths, then label propagation -- bins equal to the oracle's on the same
    edges, at the reference's defaults and at a stricter minS."""
    from gpu_util import synth_set

    from mdet_gb300 import synth

    a, _, tnf = synth_set(seed=7, n=20000, genomes=50)
    abd, var = synth.abundance(a.genome, 10, 77)
    gpu_ctx.set_abundance(abd, var)
    g = gpu_ctx.tnf_graph(tnf, a.log_sizes, 0.95, 200, mode="bf16")
    sc = gpu_ctx.edges_sscr(g.from_, g.to, g.sTNF)
    gpu_ctx.set_abundance(None, None)
    assert np.allclose(sc, oracle.sscr(g.from_, g.to, g.sTNF, abd, var), rtol=1e-12, atol=1e-12)
    for mp, ms in [(0.95, 0.60), (0.95, 0.80)]:
        want, ost = oracle.label_prop(g.from_, g.to, sc, 20000, mp, ms)
        got, st = gpu_ctx.label_propagation(g.from_, g.to, sc, 20000, mp, ms)
        assert np.array_equal(got, want)
        assert st["calls"] == ost["calls"] and st["sweeps"] == ost["sweeps"]
        assert len(np.unique(got)) < 20000


def test_repeated_edges_and_self_pairs(gpu_ctx):
    """Edges listed twice (both copies join while their contigs' bins differ)
    and an edge of a contig with itself (never joins) are taken as the
    reference takes them."""
    f, t, s = _planted(12, 500, 5, 5, 0.2)
    rng = np.random.default_rng(12)
    dup = rng.choice(s.size, 300, replace=False)
    f2 = np.concatenate([f, f[dup], [7, 9]])
    t2 = np.concatenate([t, t[dup], [7, 9]])
    s2 = np.concatenate([s, s[dup] - 1e-9, [0.99, 0.7]])
    want, ost = oracle.label_prop(f2, t2, s2, 500)
    got, st = gpu_ctx.label_propagation(f2, t2, s2, 500)
    assert np.array_equal(got, want)
    assert st["graph_edges"] == ost["graph_edges"]


def test_degenerate_inputs(gpu_ctx):
    mem, st = gpu_ctx.label_propagation([], [], [], 5)
    assert mem.tolist() == list(range(5)) and st["calls"] == 0
    mem, st = gpu_ctx.label_propagation([0, 1], [1, 2], [0.3, 0.5], 4)
    assert mem.tolist() == list(range(4)) and st["calls"] == 0
    mem, st = gpu_ctx.label_propagation([0], [1], [0.9], 2)
    assert st["calls"] == 1 and mem[0] == mem[1]
    mem, st = gpu_ctx.label_propagation([0], [1], [1.0], 2)   # log(0): a CDF of 1
    want, _ = oracle.label_prop([0], [1], [1.0], 2)
    assert np.array_equal(mem, want)
    import mdet_gb300 as m

    with pytest.raises(m.MdetError):
        gpu_ctx.label_propagation([0], [1], [1.5], 2)
    with pytest.raises(m.MdetError):
        gpu_ctx.label_propagation([0], [7], [0.9], 2)


def test_device_entry(gpu_ctx):
    torch = pytest.importorskip("torch")
    f, t, s = _planted(5, 800, 8, 5, 0.3)
    want, _ = oracle.label_prop(f, t, s, 800)
    df = torch.from_numpy(f.astype(np.int64)).cuda()
    dt = torch.from_numpy(t.astype(np.int64)).cuda()
    ds = torch.from_numpy(s).cuda()
    dm = torch.zeros(800, dtype=torch.int64, device="cuda")
    torch.cuda.synchronize()
    st = gpu_ctx.label_propagation_dev(df.data_ptr(), dt.data_ptr(), ds.data_ptr(), s.size, 800, dm.data_ptr())
    assert np.array_equal(dm.cpu().numpy().astype(np.uint64), want)
    assert st["ms_total"] > 0
