"""Label propagation on the host: the oracle restatement against the
reference's own traversal and label_propagation (compiled here from
cuda/Cuda2.cu:569-656 and 1980-2061; tests/golden/make_lp_golden.py), the
emulated std::unordered_map order that breaks exact ties, and the accuracy
of the project's exp, log and chi-squared CDF (mdet_gb300/csrc/lp_math.h)."""
import os

import numpy as np
import pytest

from oracle import oracle

G = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "lp_golden.npz")


def _case(z, name):
    g = str(z[f"{name}_graph"])
    n, mp, ms, calls = z[f"{name}_params"]
    return (z[f"g_{g}_from"], z[f"g_{g}_to"], z[f"g_{g}_sscr"], int(n), float(mp), float(ms), int(calls),
            z[f"{name}_mem"])


@pytest.mark.parametrize("name", ["planted", "tnf", "strict"])
def test_oracle_equals_reference_golden(name):
    z = np.load(G)
    f, t, s, n, mp, ms, calls, want = _case(z, name)
    mem, st = oracle.label_prop(f, t, s, n, mp, ms)
    assert st["calls"] == calls
    assert np.array_equal(mem, want.astype(np.uint64))
    assert len(np.unique(mem)) < n  # bins formed


def _planted(seed, n, groups, draws, sat):
    rng = np.random.default_rng(seed)
    g = rng.integers(0, groups, n)
    fr, to, sc = [], [], []
    for v in range(n):
        for _ in range(draws):
            if rng.random() < 0.9:
                u = int(rng.choice(np.flatnonzero(g == g[v])))
                s = rng.uniform(0.7, 1.0) if rng.random() >= sat else 1 - 10 ** rng.uniform(-15, -9)
            else:
                u, s = int(rng.integers(0, n)), rng.uniform(0.3, 0.85)
            if u != v:
                fr.append(min(u, v))
                to.append(max(u, v))
                sc.append(s)
    fr, to, sc = np.array(fr, np.uint64), np.array(to, np.uint64), np.array(sc)
    _, first = np.unique(sc, return_index=True)
    keep = np.sort(first)
    return fr[keep], to[keep], sc[keep]


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_oracle_equals_reference_built_here(seed):
    if not os.path.exists(oracle.REF_LP):
        pytest.skip("reference label propagation not built (oracle/build_ref.py)")
    f, t, s = _planted(seed, 300 + 150 * seed, 5 + seed, 5, 0.3)
    n = 300 + 150 * seed
    for mp, ms in [(0.95, 0.6), (0.7, 0.8)]:
        a, st = oracle.label_prop(f, t, s, n, mp, ms)
        b, calls = oracle.ref_label_prop(f, t, s, n, mp, ms)
        assert np.array_equal(a, b) and st["calls"] == calls


def test_ties_are_exercised():
    """Saturated CDFs give exactly tied labels, which the map order breaks."""
    f, t, s = _planted(4, 600, 6, 8, 0.5)
    _, st = oracle.label_prop(f, t, s, 600)
    assert st["ties"] > 0


def test_no_edges_and_all_below_min_s():
    mem, st = oracle.label_prop([], [], [], 5)
    assert mem.tolist() == list(range(5)) and st["calls"] == 0
    mem, st = oracle.label_prop([0, 1], [1, 2], [0.3, 0.5], 4)
    assert mem.tolist() == list(range(4)) and st["calls"] == 0
    mem, st = oracle.label_prop([0], [1], [0.9], 2)   # one edge: both contigs, one bin
    assert st["calls"] == 1 and mem[0] == mem[1]


@pytest.mark.parametrize("seed", range(4))
def test_map_order_emulation(seed):
    rng = np.random.default_rng(seed)
    for _ in range(150):
        k = int(rng.integers(1, 40 if rng.random() < 0.8 else 3000))
        rg = [50, 1000, 10 ** 6, 2 ** 31][int(rng.integers(0, 4))]
        keys = rng.choice(rg, size=min(k, rg), replace=False)
        assert np.array_equal(oracle.umap_order(keys), oracle.umap_emulated(keys))


def test_lp_math_accuracy():
    mp = pytest.importorskip("mpmath")
    mp.mp.dps = 40
    L = oracle.lib()
    rng = np.random.default_rng(5)
    xs = np.concatenate([rng.random(400), np.exp(rng.uniform(-700, 700, 400)), 1 + rng.normal(0, 1e-6, 100)])
    for x in xs:
        r = mp.log(mp.mpf(float(x)))
        assert abs(mp.mpf(L.orc_lp_log(float(x))) - r) <= 3e-16 * abs(r) + 1e-300
    for z in rng.uniform(-700, 700, 400):
        r = mp.exp(mp.mpf(float(z)))
        assert abs(mp.mpf(L.orc_lp_exp(float(z))) - r) <= 3e-16 * r
    # the CDF (float-float) against the regularised lower incomplete gamma:
    # its exponent c log y - y - log c! carries ~2^-48 of terms of size ~c y
    for _ in range(300):
        c = int(rng.integers(1, 2000))
        y = float(c * rng.uniform(0.3, 3.0))
        r = mp.gammainc(c, 0, y, regularized=True)
        assert abs(mp.mpf(L.orc_lp_chi2_cdf(c, 2 * y)) - r) < 3e-10
    for _ in range(300):
        c = int(rng.integers(1, 50))
        y = float(c * rng.uniform(0.1, 5.0))
        r = mp.gammainc(c, 0, y, regularized=True)
        assert abs(mp.mpf(L.orc_lp_chi2_cdf(c, 2 * y)) - r) < 1e-12
    assert L.orc_lp_chi2_cdf(3, float("inf")) == 1.0
    assert L.orc_lp_chi2_cdf(3, 0.0) == 0.0
