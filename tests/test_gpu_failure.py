"""Failure detection on the device side, without a GPU fault: a bounded wait
that nothing completes runs out, the kernel raises the context's error flag
and returns, the call reports MDET_ERR_TIMEOUT, and the same context then
counts and builds a graph correctly (the budget is a few thousand cycles;
nothing else is in flight while the probe waits)."""
import ctypes

import numpy as np
import pytest

from oracle import oracle

pytestmark = pytest.mark.gpu


def test_bounded_wait_runs_out_and_context_stays_usable(gpu_ctx):
    from mdet_gb300 import synth
    from mdet_gb300 import tnf as T

    lib = T.load_library()
    for budget in (1000, 200000):
        rc = lib.mdet_ctx_check_wait(gpu_ctx.h, budget)
        assert rc == T.ERR_TIMEOUT
        assert b"bounded device wait" in lib.mdet_last_error(gpu_ctx.h)
    assert lib.mdet_ctx_check_wait(gpu_ctx.h, 1 << 40) == T.ERR_INVALID
    a = synth.generate(seed=91, n=400, genomes=6, max_len=60000, threads=8)
    counts, tnf = gpu_ctx.tnf_count(a.data, a.seq_off, a.seq_len)
    oc, ot = oracle.tnf_count(a.data, a.seq_off, a.seq_len)
    assert np.array_equal(counts, oc)
    g = gpu_ctx.tnf_graph(ot, a.log_sizes, 0.9, 50, mode="bf16")
    fr, to, _ = oracle.graph(ot, a.log_sizes, 0.9, 50)
    assert set(zip(g.from_.tolist(), g.to.tolist())) == set(zip(fr.tolist(), to.tolist()))
