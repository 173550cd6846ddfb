"""Pairwise stage on the GPU against the oracle: edge sets identical outside
the 1e-5 tolerance band, sTNF within 1e-9; the tensor-core form equal to
the plain form; max-probability sample and pTNF search equal to the oracle."""
import numpy as np
import sys, os
sys.path.insert(0, os.path.dirname(__file__))
import pytest

from gpu_util import compare_graph, synth_set
from oracle import oracle

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def set_a():
    return synth_set(seed=21, n=1800, genomes=30)


@pytest.mark.parametrize("cutoff,k", [(0.95, 200), (0.95, 5), (0.8, 40), (0.999, 200)])
def test_plain_vs_oracle(gpu_ctx, set_a, cutoff, k):
    a, _, tnf = set_a
    g = gpu_ctx.tnf_graph(tnf, a.log_sizes, cutoff, k, mode="plain")
    common, exempt = compare_graph(g.from_, g.to, g.sTNF, tnf, a.log_sizes, cutoff, k)
    assert common > 0 or cutoff > 0.99
    assert exempt <= max(2, common // 1000)
    # output order: rows ascending, similarity descending inside a row
    assert np.all(np.diff(g.from_.astype(np.int64)) >= 0)


@pytest.mark.parametrize("cutoff,k", [(0.95, 200), (0.9, 10)])
def test_bf16_equals_plain(gpu_ctx, set_a, cutoff, k):
    a, _, tnf = set_a
    p = gpu_ctx.tnf_graph(tnf, a.log_sizes, cutoff, k, mode="plain")
    t = gpu_ctx.tnf_graph(tnf, a.log_sizes, cutoff, k, mode="bf16")
    assert np.array_equal(p.from_, t.from_)
    assert np.array_equal(p.to, t.to)
    assert np.array_equal(p.sTNF, t.sTNF)
    assert t.stats["n_candidates"] >= t.stats["n_above_cutoff"]


@pytest.mark.parametrize("cutoff,k", [(0.95, 200), (0.9, 10), (0.8, 40)])
def test_tf32_equals_plain(gpu_ctx, set_a, cutoff, k):
    """The TF32 tcgen05 filter is conservative like the BF16 one (its rows'
    rounding errors enter the bound), so the graph equals the plain form's bit
    for bit; its tighter rounding keeps fewer candidates than BF16."""
    a, _, tnf = set_a
    p = gpu_ctx.tnf_graph(tnf, a.log_sizes, cutoff, k, mode="plain")
    t = gpu_ctx.tnf_graph(tnf, a.log_sizes, cutoff, k, mode="tf32")
    b = gpu_ctx.tnf_graph(tnf, a.log_sizes, cutoff, k, mode="bf16")
    assert np.array_equal(p.from_, t.from_) and np.array_equal(p.to, t.to) and np.array_equal(p.sTNF, t.sTNF)
    assert t.stats["n_above_cutoff"] <= t.stats["n_candidates"] <= b.stats["n_candidates"]
    assert t.stats["tile_m_n"] == 128128


def test_tf32_sample_passes(gpu_ctx, set_a):
    """Max-probability and pTNF requests in the TF32 form give the BF16/plain
    results (the sample passes run the BF16 filter; the maxima are exact)."""
    a, _, tnf = set_a
    idx = np.arange(0, tnf.shape[0], 5)
    assert np.array_equal(gpu_ctx.max_prob(tnf, a.log_sizes, idx, mode="tf32"),
                          gpu_ctx.max_prob(tnf, a.log_sizes, idx, mode="plain"))
    from oracle import oracle as _o
    _o.srand(77)
    p1 = gpu_ctx.ptnf_search(tnf, a.log_sizes, 0.95, mode="tf32")
    _o.srand(77)
    p2 = gpu_ctx.ptnf_search(tnf, a.log_sizes, 0.95, mode="bf16")
    assert p1 == p2


@pytest.mark.parametrize("shape", [128256, 128128, 256128])
def test_every_tile_shape_equals_plain(gpu_ctx, set_a, shape):
    a, _, tnf = set_a
    p = gpu_ctx.tnf_graph(tnf, a.log_sizes, 0.9, 40, mode="plain")
    gpu_ctx.set_autotune(shape)
    try:
        t = gpu_ctx.tnf_graph(tnf, a.log_sizes, 0.9, 40, mode="bf16")
        m = gpu_ctx.max_prob(tnf, a.log_sizes, np.arange(0, tnf.shape[0], 7), mode="bf16")
    finally:
        gpu_ctx.set_autotune(True)
    assert t.stats["tile_m_n"] == shape
    assert np.array_equal(p.from_, t.from_) and np.array_equal(p.to, t.to) and np.array_equal(p.sTNF, t.sTNF)
    mp = gpu_ctx.max_prob(tnf, a.log_sizes, np.arange(0, tnf.shape[0], 7), mode="plain")
    assert np.array_equal(m, mp)


def test_identical_contigs_big_rows(gpu_ctx):
    # 1500 copies of a handful of profiles: rows with > 1024 tied edges
    a, _, tnf = synth_set(seed=22, n=40, genomes=2, max_len=30000)
    rep = np.repeat(np.arange(4), 375)
    t2 = tnf[rep]
    ls = a.log_sizes[rep]
    for mode in ("plain", "bf16"):
        g = gpu_ctx.tnf_graph(t2, ls, 0.9, 300, mode=mode)
        compare_graph(g.from_, g.to, g.sTNF, t2, ls, 0.9, 300)


def test_tiny_inputs(gpu_ctx):
    a, _, tnf = synth_set(seed=23, n=3, genomes=1, max_len=200000)
    for n in (0, 1, 2, 3):
        g = gpu_ctx.tnf_graph(tnf[:n], a.log_sizes[:n], 0.7, 200, mode="plain")
        fr, to, st = oracle.graph(tnf[:n], a.log_sizes[:n], 0.7, 200) if n else ([], [], [])
        assert sorted(zip(g.from_.tolist(), g.to.tolist())) == sorted(zip(list(map(int, fr)), list(map(int, to))))


def test_capacity_error(gpu_ctx, set_a):
    import ctypes

    from mdet_gb300 import tnf as T

    a, _, tnf = set_a
    lib = T.load_library()
    n = tnf.shape[0]
    fr = np.zeros(4, np.uint64)
    ne = ctypes.c_uint64(0)
    t32 = np.ascontiguousarray(tnf)
    rc = lib.mdet_tnf_graph(gpu_ctx.h, t32.ctypes.data, a.log_sizes.ctypes.data, n, 0.9, 200, 0, fr.ctypes.data,
                            fr.ctypes.data, fr.ctypes.data, 4, ctypes.byref(ne), None)
    assert rc == T.ERR_CAPACITY and ne.value > 4


@pytest.mark.parametrize("mode", ["plain", "bf16"])
def test_max_prob_vs_oracle(gpu_ctx, set_a, mode):
    a, _, tnf = set_a
    n = tnf.shape[0]
    rng = np.random.default_rng(3)
    perm = rng.permutation(n).astype(np.uint64)
    m = 250
    ref = oracle.max_prob(tnf, a.log_sizes, perm, m)
    got = gpu_ctx.max_prob(tnf, a.log_sizes, perm, m, mode=mode, floor_prob=0.7)
    hi = ref >= 0.7
    assert np.abs(got[hi] - ref[hi]).max() <= 1e-9
    assert np.all(got[~hi] < 0.7)
    exact = gpu_ctx.max_prob(tnf, a.log_sizes, perm, 60, mode="plain", floor_prob=0.0)
    assert np.abs(exact - ref[:60]).max() <= 1e-9


@pytest.mark.parametrize("genomes", [50, 2000])
def test_ptnf_search_sampled_vs_oracle(gpu_ctx, genomes):
    """Above 25,000 contigs the search samples 2,500 rows ten times.  Each pass
    scores maxima at a floor just below the previous cutoff first and rescores
    the rows below it only when the search goes there: with 50 genomes the
    cutoff stays high, with 2,000 it drops below the first floor (0.9), so
    both branches run; the result must equal the oracle's."""
    a, _, tnf = synth_set(seed=5, n=26000, genomes=genomes)
    want = oracle.ptnf_search(tnf, a.log_sizes, 0.95, seed=77)
    oracle.srand(77)
    got = gpu_ctx.ptnf_search(tnf, a.log_sizes, 0.95, mode="bf16")
    assert got == want
    if genomes == 2000:
        assert want < 900


@pytest.mark.parametrize("mode", ["plain", "bf16"])
def test_ptnf_search_vs_oracle(gpu_ctx, set_a, mode):
    a, _, tnf = set_a
    want = oracle.ptnf_search(tnf, a.log_sizes, 0.95, seed=77)
    oracle.srand(77)
    got = gpu_ctx.ptnf_search(tnf, a.log_sizes, 0.95, mode=mode)
    assert got == want


def test_prep_reuse_follows_contents(gpu_ctx):
    """Calls on the same device buffers reuse the size-sorted preparation only
    while the contents are unchanged and no count ran in between: results
    must always equal a fresh context's on the current contents."""
    torch = pytest.importorskip("torch")
    import mdet_gb300 as m

    dev = torch.device("cuda:0")
    a1, _, t1 = synth_set(seed=41, n=1500, genomes=20)
    a2, _, t2 = synth_set(seed=42, n=1500, genomes=20)
    n = 1500
    d_tnf = torch.from_numpy(t1).to(dev)
    d_ls = torch.from_numpy(a1.log_sizes.copy()).to(dev)
    cap = n * 40
    outs = [torch.empty(cap, dtype=t, device=dev) for t in (torch.int64, torch.int64, torch.float64)]

    def run(ctx):
        ne, _ = ctx.tnf_graph_dev(d_tnf.data_ptr(), d_ls.data_ptr(), n, 0.9, 40, "bf16", outs[0].data_ptr(),
                                  outs[1].data_ptr(), outs[2].data_ptr(), cap)
        torch.cuda.synchronize()
        return [o[:ne].cpu().numpy().copy() for o in outs]

    def fresh():
        with m.Context(0) as c:
            return run(c)

    r1 = run(gpu_ctx)
    r1b = run(gpu_ctx)  # same contents: the preparation is reused
    for x, y in zip(r1, r1b):
        assert np.array_equal(x, y)
    # new contents in the same buffers
    d_tnf.copy_(torch.from_numpy(t2))
    d_ls.copy_(torch.from_numpy(a2.log_sizes.copy()))
    r2 = run(gpu_ctx)
    f2 = fresh()
    for x, y in zip(r2, f2):
        assert np.array_equal(x, y)
    assert not np.array_equal(r1[0], r2[0]) or not np.array_equal(r1[1], r2[1])
    # a count into the same TNF buffer invalidates it even when it writes the same rows
    d_bytes = torch.zeros(a2.data.size + 64, dtype=torch.uint8, device=dev)
    d_bytes[:a2.data.size].copy_(torch.from_numpy(a2.data))
    d_off = torch.from_numpy(a2.seq_off.astype(np.int64)).to(dev)
    d_len = torch.from_numpy(a2.seq_len.astype(np.int64)).to(dev)
    d_cnt = torch.empty((n, 136), dtype=torch.int32, device=dev)
    gpu_ctx.tnf_count_dev(d_bytes.data_ptr(), a2.data.size, d_off.data_ptr(), d_len.data_ptr(), n, d_cnt.data_ptr(),
                          d_tnf.data_ptr())
    r3 = run(gpu_ctx)
    f3 = fresh()
    for x, y in zip(r3, f3):
        assert np.array_equal(x, y)
