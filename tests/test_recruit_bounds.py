"""The error bounds behind recruiting's FP32 estimates (mdet_gb300/csrc/
recruit.cu), checked numerically on the CPU: for rank rows (the only rows the
entry point correlates), the FP32 correlation formed as the kernels form it
-- dx_i * ratio_i rounded to FP32 for the member row, dx_i for the other, a
fused dot product, and the two rows' rounded inverse root sums -- stays
within (m + 10.2) * 1.02 u of the reference's FP64 correlation (u = 2^-24),
and an FP32 first-ten mean within (1.02 m + 20.5) u of the FP64 one.  The
FP64 side follows cal_abd_corr (cuda/Cuda2.cu:1219-1245) step by step.
The fused multiply-add is emulated as an FP64 product-sum rounded once to
FP32 (the product of two floats is exact in FP64)."""
import numpy as np
import pytest

U = 2.0 ** -24
f32 = np.float32


def rank_average(row):
    """Average ranks (1-based) of a row, ties sharing the mean of their ranks,
    formed in float as the reference's ranker does."""
    order = np.argsort(row, kind="stable")
    v = row[order]
    out = np.empty(row.size, np.float32)
    c = 0
    while c < row.size:
        k = 1
        while c + k < row.size and v[c] == v[c + k]:
            k += 1
        out[order[c:c + k]] = f32((2 * c + k - 1) / 2 + 1)
        c += k
    return out


def prep(row):
    """k_corr_rows: deviations from the running mean and the root sum, FP64."""
    nabd = row.size
    dx = np.zeros(nabd - 1)
    mx = float(row[0])
    sxx = 0.0
    for i in range(1, nabd):
        ratio = i / (i + 1.0)
        d = float(row[i]) - mx
        sxx += d * d * ratio
        mx += d / (i + 1.0)
        dx[i - 1] = d
    return dx, np.sqrt(sxx)


def corr64(a, b):
    """The reference's correlation from two prepared rows."""
    (dx, sx), (dy, sy) = a, b
    sxy = 0.0
    for i in range(dx.size):
        sxy += dx[i] * dy[i] * ((i + 1) / (i + 2.0))
    return sxy / (sx * sy)


def corr32(a, b):
    """The kernels' FP32 correlation: member row a in the xw form."""
    (dx, sx), (dy, sy) = a, b
    xw = np.array([f32(f32(dx[i]) * f32((i + 1) / (i + 2.0))) for i in range(dx.size)], np.float32)
    yf = dy.astype(np.float32)
    s = f32(0.0)
    for i in range(dx.size):
        s = f32(float(xw[i]) * float(yf[i]) + float(s))  # fma: one rounding
    ix, iy = f32(f32(1.0) / f32(sx)), f32(f32(1.0) / f32(sy))
    return f32(s * f32(ix * iy))


@pytest.mark.parametrize("nabd", [3, 10, 48, 200])
def test_fp32_correlation_bounds(nabd):
    rng = np.random.default_rng(nabd)
    rows = []
    for k in range(60):
        if k % 3 == 0:
            r = rng.integers(0, 4, nabd).astype(np.float32)  # many ties
        else:
            r = rng.lognormal(2, 1, nabd).astype(np.float32)
        r = rank_average(r)
        if np.all(r == r[0]):
            continue  # constant rows take the exact path
        rows.append(prep(r))
    m = nabd - 1
    worst = 0.0
    for i in range(len(rows)):
        for j in range(len(rows)):
            if i == j:
                continue
            e = abs(float(corr32(rows[i], rows[j])) - corr64(rows[i], rows[j]))
            worst = max(worst, e / U)
            assert e <= (m + 10.2) * 1.02 * U
    # first-ten means: ten members against one contig row
    for c in range(len(rows) - 10):
        y = rows[c]
        mem = rows[c + 1:c + 11]
        s32 = f32(0.0)
        s64 = 0.0
        for x in mem:
            s32 = f32(s32 + corr32(x, y))
            s64 += corr64(x, y)
        assert abs(float(f32(s32 / f32(10))) - s64 / 10) <= (1.02 * m + 20.5) * U
    assert worst > 0  # the FP32 form does differ: the bound is exercised
