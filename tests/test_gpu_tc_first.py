"""Smallest tensor-core case first: one and a few tiles against the plain form."""
import os
import sys

import numpy as np
import pytest

sys.path.insert(0, os.path.dirname(__file__))
from gpu_util import synth_set  # noqa: E402

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n", [100, 300, 700])
def test_bf16_small(gpu_ctx, n):
    a, _, tnf = synth_set(seed=31 + n, n=n, genomes=6, max_len=80000)
    p = gpu_ctx.tnf_graph(tnf, a.log_sizes, 0.9, 200, mode="plain")
    t = gpu_ctx.tnf_graph(tnf, a.log_sizes, 0.9, 200, mode="bf16")
    assert p.from_.size > 0
    assert np.array_equal(p.from_, t.from_) and np.array_equal(p.to, t.to) and np.array_equal(p.sTNF, t.sTNF)
