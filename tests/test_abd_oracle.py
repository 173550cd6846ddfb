"""The abundance side of the oracle pinned against the reference: sTNF ->
sSCR and the is_nz pair gate against the reference's own code
(tests/golden/abd_golden.npz, made by tests/golden/make_abd_golden.py from
cuda/Cuda2.cu compiled on the host), and -- where the reference is mounted --
against that compiled code on fresh random inputs."""
import ctypes
import os

import numpy as np
import pytest

from oracle import oracle

G = os.path.join(os.path.dirname(__file__), "golden")
REF_ABD = os.path.join(os.path.dirname(oracle.__file__), "_ref", "libref_abd.so")


def golden():
    return np.load(os.path.join(G, "abd_golden.npz"))


@pytest.mark.parametrize("k", [5, 2])
def test_sscr_reproduces_reference(k):
    g = golden()
    got = oracle.sscr(g["from_"], g["to"], g["stnf"], g["abd"][:, :k], g["var"][:, :k])
    ref = g[f"sscr{k}"]
    # the same arithmetic in the same order; only libm's erfc/log/pow may
    # differ by an ulp between machines
    assert np.allclose(got, ref, rtol=1e-12, atol=0)
    assert np.all((got > 0) & (got < 1))


def test_is_nz_gate_reproduces_reference():
    g = golden()
    low = oracle.abd_low(g["abd"]).astype(bool)
    p = g["nz_pairs"]
    assert np.array_equal((~(low[p[:, 0]] & low[p[:, 1]])).astype(np.uint8), g["nz"])


def test_sscr_without_abundance_is_stnf():
    g = golden()
    empty = np.zeros((g["abd"].shape[0], 0))
    assert np.array_equal(oracle.sscr(g["from_"], g["to"], g["stnf"], empty, empty), g["stnf"])


def test_sscr_depends_on_stnf_only_by_rank():
    """sTNF enters by rank ("min" ties): a strictly increasing transform of
    it leaves sSCR unchanged, and merging values into ties changes it."""
    g = golden()
    st = g["stnf"]
    base = oracle.sscr(g["from_"], g["to"], st, g["abd"], g["var"])
    assert np.array_equal(oracle.sscr(g["from_"], g["to"], st ** 3 - 0.1, g["abd"], g["var"]), base)
    merged = oracle.sscr(g["from_"], g["to"], np.round(st, 1), g["abd"], g["var"])
    assert not np.array_equal(merged, base)


def test_gated_graph_has_no_low_pairs():
    from mdet_gb300 import synth

    a = synth.generate(seed=77, n=400, genomes=10, max_len=20000, threads=4)
    abd, var = synth.abundance(a.genome, 4, 3, low_frac=0.2)
    low = oracle.abd_low(abd)
    _, tnf = oracle.tnf_count(a.data, a.seq_off, a.seq_len)
    f, t, _ = oracle.graph(tnf, a.log_sizes, 0.85, 30, low=low)
    assert not np.any(low[f].astype(bool) & low[t].astype(bool))
    f0, t0, s0 = oracle.graph(tnf, a.log_sizes, 0.85, 30)
    assert np.any(low[f0].astype(bool) & low[t0].astype(bool))  # the gate had something to drop
    f1, t1, s1 = oracle.graph(tnf, a.log_sizes, 0.85, 30, low=np.zeros_like(low))
    assert np.array_equal(f0, f1) and np.array_equal(t0, t1) and np.array_equal(s0, s1)


@pytest.mark.skipif(not os.path.exists(REF_ABD), reason="reference not compiled here")
@pytest.mark.parametrize("seed,nabd", [(1, 3), (2, 8), (3, 1)])
def test_sscr_against_reference_code(seed, nabd):
    from mdet_gb300 import synth

    L = ctypes.CDLL(REF_ABD)
    P, u64, u32, D = ctypes.c_void_p, ctypes.c_uint64, ctypes.c_uint32, ctypes.c_double
    L.ref_sscr.argtypes = [P, P, P, u64, P, P, u32, D, u32, P]
    rng = np.random.default_rng(seed)
    n, ne = 300, 2000
    abd, var = synth.abundance(rng.integers(0, 9, n), nabd, seed, low_frac=0.05)
    i, j = rng.integers(0, n, (2, 3 * ne))
    cov = ((abd[i] > 1.0) | (abd[j] > 1.0)).any(1) & (i != j)
    fr, to = i[cov][:ne].astype(np.uint64), j[cov][:ne].astype(np.uint64)
    st = np.round(rng.uniform(0.5, 1.0, fr.size), 4)
    ref = np.zeros(fr.size)
    L.ref_sscr(fr.ctypes.data, to.ctypes.data, st.ctypes.data, fr.size, abd.ctypes.data, var.ctypes.data, nabd,
               1.0, 3, ref.ctypes.data)
    got = oracle.sscr(fr, to, st, abd, var)
    assert np.allclose(got, ref, rtol=1e-12, atol=0)


def test_overlap_is_stationary_in_the_crossing_points():
    """The GPU forms cal_abd_dist2's crossing points in float-float where the
    variances differ by at least 1e-3 of the larger (mdet_gb300/csrc/
    abundance.cu, abd_dist2_ff).  That rests on the overlap
    d = |Pa(k2) - Pa(k1) + Pb(k1) - Pb(k2)| being stationary in k1 and k2
    (the densities are equal there): moving both by 1e-9 sd, far more than
    float-float's error, moves d by less than 1e-16 -- checked here in
    50-digit arithmetic on seeded normal pairs in that regime."""
    mp = pytest.importorskip("mpmath")
    mp.mp.dps = 50
    rng = np.random.default_rng(17)
    for _ in range(200):
        m1, m2 = rng.lognormal(2, 1.2, 2)
        v1 = max(1.0, m1 * rng.uniform(0.3, 3))
        v2 = max(1.0, m2 * rng.uniform(0.3, 3))
        if abs(v1 - v2) < 1e-3 * max(v1, v2):
            continue
        m1, m2, v1, v2 = (mp.mpf(float(x)) for x in (m1, m2, v1, v2))
        t = mp.sqrt(v1 * v2 * ((m1 - m2) ** 2 - 2 * (v1 - v2) * mp.log(mp.sqrt(v2 / v1))))
        k1, k2 = sorted([(t - m1 * v2 + m2 * v1) / (v1 - v2), (t + m1 * v2 - m2 * v1) / (v2 - v1)])
        (ma, va), (mb, vb) = sorted([(m1, v1), (m2, v2)], key=lambda p: p[1])

        def cdf(m, v, x):
            return mp.erfc(-(x - m) / mp.sqrt(2 * v)) / 2

        def d(a, b):
            return abs(cdf(ma, va, b) - cdf(ma, va, a) + cdf(mb, vb, a) - cdf(mb, vb, b))

        sd = mp.sqrt(min(va, vb))
        for e1, e2 in [(1, 1), (1, -1), (-1, 1)]:
            moved = d(k1 + e1 * mp.mpf("1e-9") * sd, k2 + e2 * mp.mpf("1e-9") * sd)
            assert abs(moved - d(k1, k2)) < 1e-16
