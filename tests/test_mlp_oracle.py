"""The network oracle itself (CPU): its analytic gradient against central
finite differences, and its parameter layout against the library's."""
import numpy as np

from oracle import mlp_ref as R


def _setup(seed=5, rows=24, npairs=20):
    rng = np.random.default_rng(seed)
    p = np.zeros(R.NPARAM, np.float64)
    p[R.W1:R.B1] = rng.normal(0, np.sqrt(2 / R.IN), R.H1 * R.IN)
    p[R.B1:R.W2] = rng.normal(0, 0.1, R.H1)
    p[R.W2:R.B2] = rng.normal(0, np.sqrt(2 / R.H1), R.H2 * R.H1)
    p[R.B2:R.W3] = rng.normal(0, 0.1, R.H2)
    p[R.W3:R.B3] = rng.normal(0, np.sqrt(2 / R.H2), R.OUT * R.H2)
    p[R.B3:R.MU] = rng.normal(0, 0.1, R.OUT)
    p[R.SCALE] = 1.0
    x = rng.normal(0, 1.0, (rows, R.IN))
    pairs = rng.integers(0, rows, (npairs, 2))
    pairs[pairs[:, 0] == pairs[:, 1], 1] = (pairs[pairs[:, 0] == pairs[:, 1], 1] + 1) % rows
    y = (rng.random(npairs) < 0.5).astype(np.float64)
    e = np.linalg.norm(R.embed(p, x[pairs[:, 0]]) - R.embed(p, x[pairs[:, 1]]), axis=1)
    return p, x, pairs, y, 0.7 * np.median(e), 1.3 * np.median(e)


def test_gradient_matches_finite_differences():
    p, x, pairs, y, mp, mn = _setup()
    _, g = R.loss_and_grad(p, x, pairs, y, mp, mn, rounded=False)
    rng = np.random.default_rng(9)
    for lo, hi in [(R.W1, R.B1), (R.B1, R.W2), (R.W2, R.B2), (R.B2, R.W3), (R.W3, R.B3), (R.B3, R.MU)]:
        for k in rng.integers(lo, hi, 6):
            h = 1e-6
            q = p.copy()
            q[k] += h
            lp, _ = R.loss_and_grad(q, x, pairs, y, mp, mn, rounded=False)
            q[k] -= 2 * h
            lm, _ = R.loss_and_grad(q, x, pairs, y, mp, mn, rounded=False)
            fd = (lp - lm) / (2 * h)
            assert abs(fd - g[k]) <= 1e-6 + 1e-5 * abs(fd), (k, fd, g[k])


def test_bf16_rounding_is_nearest_even():
    v = np.array([1.0, 1.00390625, 1.005859375, 1.0078125, -2.5e-3, 3.0e38], np.float32)
    r = R.bf16_round(v)
    assert r[0] == 1.0 and r[1] == 1.0          # tie -> even
    assert r[2] == 1.0078125                    # above the tie -> up
    assert r[3] == 1.0078125                    # representable
    assert abs(r[4] - (-2.5e-3)) < 2e-5


def test_layout_matches_library():
    from mdet_gb300 import tnf as T

    assert T.Network.param_count() == R.NPARAM == 76362
