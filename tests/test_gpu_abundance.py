"""The abundance side on the GPU: sTNF -> sSCR against the reference's own
code (golden fixture) and the oracle, and the is_nz pair gate of the graph
against the oracle's gated graph."""
import os
import sys

import numpy as np
import pytest

sys.path.insert(0, os.path.dirname(__file__))
from gpu_util import compare_graph, synth_set  # noqa: E402
from oracle import oracle  # noqa: E402

pytestmark = pytest.mark.gpu
G = os.path.join(os.path.dirname(__file__), "golden")
# the crossing points and the correlations are the reference's FP64
# arithmetic in its order (CUDA's log and pow may differ from the host's libm
# by a few ulps); the four normal CDFs per sample come from a float-float
# erfc (about 1e-13 absolute near erfc ~ 1 after its float-float Horner
# steps), so sSCR (in [0, 1]) agrees within 1e-12 relative or 1e-12 absolute
RTOL = 1e-12
ATOL = 1e-12


@pytest.fixture
def abd_ctx(gpu_ctx):
    yield gpu_ctx
    gpu_ctx.set_abundance(None, None)


@pytest.mark.parametrize("k", [5, 2])
def test_sscr_matches_reference_golden(abd_ctx, k):
    g = np.load(os.path.join(G, "abd_golden.npz"))
    abd_ctx.set_abundance(g["abd"][:, :k], g["var"][:, :k])
    got = abd_ctx.edges_sscr(g["from_"], g["to"], g["stnf"])
    assert np.allclose(got, g[f"sscr{k}"], rtol=RTOL, atol=ATOL)


@pytest.mark.parametrize("nabd,min_cv", [(10, 1.0), (3, 1.0), (2, 0.5), (1, 2.0)])
def test_sscr_vs_oracle(abd_ctx, nabd, min_cv):
    from mdet_gb300 import synth

    rng = np.random.default_rng(nabd)
    n, ne = 5000, 60000
    abd, var = synth.abundance(rng.integers(0, 40, n), nabd, 100 + nabd, low_frac=0.05)
    i, j = rng.integers(0, n, (2, 2 * ne))
    cov = ((abd[i] > min_cv) | (abd[j] > min_cv)).any(1) & (i != j)
    fr, to = i[cov][:ne].astype(np.uint64), j[cov][:ne].astype(np.uint64)
    st = np.round(rng.uniform(0.5, 1.0, fr.size), 5)  # ties
    abd_ctx.set_abundance(abd, var)
    got = abd_ctx.edges_sscr(fr, to, st, min_cv=min_cv)
    ref = oracle.sscr(fr, to, st, abd, var, min_cv=min_cv)
    assert np.allclose(got, ref, rtol=RTOL, atol=ATOL)


def test_sscr_device_path_and_empty(abd_ctx):
    torch = pytest.importorskip("torch")
    g = np.load(os.path.join(G, "abd_golden.npz"))
    abd_ctx.set_abundance(g["abd"], g["var"])
    host = abd_ctx.edges_sscr(g["from_"], g["to"], g["stnf"])
    dev = torch.device("cuda:0")
    f = torch.from_numpy(g["from_"].astype(np.int64)).to(dev)
    t = torch.from_numpy(g["to"].astype(np.int64)).to(dev)
    s = torch.from_numpy(g["stnf"]).to(dev)
    out = torch.empty_like(s)
    abd_ctx.edges_sscr_dev(f.data_ptr(), t.data_ptr(), s.data_ptr(), s.numel(), out.data_ptr())
    torch.cuda.synchronize()
    assert np.array_equal(out.cpu().numpy(), host)
    assert abd_ctx.edges_sscr(g["from_"][:0], g["to"][:0], g["stnf"][:0]).size == 0


def test_sscr_without_abundance_copies_stnf(gpu_ctx):
    g = np.load(os.path.join(G, "abd_golden.npz"))
    gpu_ctx.set_abundance(None, None)
    assert np.array_equal(gpu_ctx.edges_sscr(g["from_"], g["to"], g["stnf"]), g["stnf"])


def test_sscr_rejects_bad_edges(abd_ctx):
    from mdet_gb300 import MdetError

    g = np.load(os.path.join(G, "abd_golden.npz"))
    abd_ctx.set_abundance(g["abd"], g["var"])
    n = g["abd"].shape[0]
    fr, to = g["from_"].copy(), g["to"].copy()
    to[7] = n  # out of range
    with pytest.raises(MdetError):
        abd_ctx.edges_sscr(fr, to, g["stnf"])
    # an edge with no sample above min_cv (the reference would divide 0 by 0)
    with pytest.raises(MdetError):
        abd_ctx.edges_sscr(g["from_"], g["to"], g["stnf"], min_cv=1e9)
    # the context stays usable
    assert np.allclose(abd_ctx.edges_sscr(g["from_"], g["to"], g["stnf"]), g["sscr5"], rtol=RTOL, atol=ATOL)


@pytest.mark.parametrize("mode", ["bf16", "plain"])
def test_gated_graph_vs_oracle(abd_ctx, mode):
    from mdet_gb300 import synth

    a, _, tnf = synth_set(21, 3000, 30)
    abd, var = synth.abundance(a.genome, 4, 5, low_frac=0.25)
    low = oracle.abd_low(abd)
    abd_ctx.set_abundance(abd, var)
    gr = abd_ctx.tnf_graph(tnf, a.log_sizes, 0.9, 60, mode=mode)
    assert not np.any(low[gr.from_].astype(bool) & low[gr.to].astype(bool))
    compare_graph(gr.from_, gr.to, gr.sTNF, tnf, a.log_sizes, 0.9, 60, low=low)
    # a different contig count than the abundance covers is an error
    from mdet_gb300 import MdetError

    with pytest.raises(MdetError):
        abd_ctx.tnf_graph(tnf[:100], a.log_sizes[:100], 0.9, 60, mode=mode)
    # cleared: the ungated graph again
    abd_ctx.set_abundance(None, None)
    g0 = abd_ctx.tnf_graph(tnf, a.log_sizes, 0.9, 60, mode=mode)
    assert np.any(low[g0.from_].astype(bool) & low[g0.to].astype(bool))
    compare_graph(g0.from_, g0.to, g0.sTNF, tnf, a.log_sizes, 0.9, 60)
