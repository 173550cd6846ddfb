"""Batched graphs (mdet_tnf_graph_batched): many assemblies of uneven sizes,
cutoffs and max_edges in one pass must give, assembly by assembly, exactly
the edges of the single-assembly entry point (same exact stage, same
selection), and a short capacity must be reported for that assembly only."""
import os
import sys

import numpy as np
import pytest

sys.path.insert(0, os.path.dirname(__file__))

pytestmark = pytest.mark.gpu

SPECS = [  # (n, genomes, cutoff, max_edges)
    (3000, 12, 0.9, 200),
    (257, 3, 0.95, 10),
    (40, 2, 0.8, 50),
    (9000, 30, 0.9, 200),
    (1, 1, 0.9, 5),
    (5000, 20, 0.99, 300),
    (700, 5, 0.7, 512),
]


@pytest.fixture(scope="module")
def batch_inputs():
    torch = pytest.importorskip("torch")
    from gpu_util import synth_set

    out = []
    for i, (n, G, cut, k) in enumerate(SPECS):
        a, _, tnf = synth_set(seed=900 + i, n=max(n, 2), genomes=G, max_len=150000)
        tnf, ls = tnf[:n], a.log_sizes[:n]
        out.append(dict(tnf=tnf, ls=ls, d_tnf=torch.from_numpy(np.ascontiguousarray(tnf)).cuda(),
                        d_ls=torch.from_numpy(np.ascontiguousarray(ls)).cuda(), n=n, cutoff=cut, max_edges=k))
    torch.cuda.synchronize()
    return out


def _outputs(torch, n, k, cap=None):
    cap = max(1, n * k) if cap is None else cap
    return (torch.zeros(cap, dtype=torch.int64, device="cuda"), torch.zeros(cap, dtype=torch.int64, device="cuda"),
            torch.zeros(cap, dtype=torch.float64, device="cuda"), cap)


def _single(ctx, torch, x, mode):
    fr, to, st, cap = _outputs(torch, x["n"], x["max_edges"])
    ne, _ = ctx.tnf_graph_dev(x["d_tnf"].data_ptr(), x["d_ls"].data_ptr(), x["n"], x["cutoff"], x["max_edges"], mode,
                              fr.data_ptr(), to.data_ptr(), st.data_ptr(), cap)
    return fr[:ne].cpu().numpy(), to[:ne].cpu().numpy(), st[:ne].cpu().numpy()


@pytest.mark.parametrize("mode", ["bf16", "plain"])
def test_batch_equals_single(gpu_ctx, batch_inputs, mode):
    import torch

    outs, items = [], []
    for x in batch_inputs:
        o = _outputs(torch, x["n"], x["max_edges"])
        outs.append(o)
        items.append(dict(d_tnf=x["d_tnf"].data_ptr(), d_ls=x["d_ls"].data_ptr(), n=x["n"], cutoff=x["cutoff"],
                          max_edges=x["max_edges"], d_from=o[0].data_ptr(), d_to=o[1].data_ptr(),
                          d_stnf=o[2].data_ptr(), capacity=o[3]))
    res, stats = gpu_ctx.tnf_graph_batched(items, mode=mode)
    assert stats["gpu_launches"] > 0
    total = 0
    for x, (status, ne), o in zip(batch_inputs, res, outs):
        assert status == 0
        f, t, s = _single(gpu_ctx, torch, x, mode)
        assert ne == f.size
        assert np.array_equal(o[0][:ne].cpu().numpy(), f)
        assert np.array_equal(o[1][:ne].cpu().numpy(), t)
        assert np.array_equal(o[2][:ne].cpu().numpy(), s)
        total += ne
    assert total > 0 and stats["n_edges"] == total


def test_recorded_batch_replays_with_new_data(gpu_ctx, batch_inputs):
    """Three calls with the same buffers: the first runs the sized path and
    records the batch, the next two replay the recording.  Then the inputs
    change in place (same sizes) and the replay must follow them."""
    import torch

    outs, items = [], []
    for x in batch_inputs:
        o = _outputs(torch, x["n"], x["max_edges"])
        outs.append(o)
        items.append(dict(d_tnf=x["d_tnf"].data_ptr(), d_ls=x["d_ls"].data_ptr(), n=x["n"], cutoff=x["cutoff"],
                          max_edges=x["max_edges"], d_from=o[0].data_ptr(), d_to=o[1].data_ptr(),
                          d_stnf=o[2].data_ptr(), capacity=o[3]))
    singles = [_single(gpu_ctx, torch, x, "bf16") for x in batch_inputs]
    r0 = gpu_ctx.graph_replays()
    for call in range(3):
        res, _ = gpu_ctx.tnf_graph_batched(items, mode="bf16")
        for (status, ne), o, (f, t, st) in zip(res, outs, singles):
            assert status == 0 and ne == f.size
            assert np.array_equal(o[1][:ne].cpu().numpy(), t) and np.array_equal(o[2][:ne].cpu().numpy(), st)
    assert gpu_ctx.graph_replays() == r0 + 2
    # new data in the same buffers: reverse the rows of every assembly
    saved = [(x["d_tnf"].clone(), x["d_ls"].clone()) for x in batch_inputs]
    try:
        for x in batch_inputs:
            x["d_tnf"].copy_(torch.flip(x["d_tnf"], [0]))
            x["d_ls"].copy_(torch.flip(x["d_ls"], [0]))
        torch.cuda.synchronize()
        res, _ = gpu_ctx.tnf_graph_batched(items, mode="bf16")
        assert gpu_ctx.graph_replays() == r0 + 3
        for x, (status, ne), o in zip(batch_inputs, res, outs):
            f, t, st = _single(gpu_ctx, torch, x, "bf16")
            assert status == 0 and ne == f.size
            assert np.array_equal(o[0][:ne].cpu().numpy(), f)
            assert np.array_equal(o[1][:ne].cpu().numpy(), t) and np.array_equal(o[2][:ne].cpu().numpy(), st)
    finally:
        for x, (a, b) in zip(batch_inputs, saved):
            x["d_tnf"].copy_(a)
            x["d_ls"].copy_(b)
        torch.cuda.synchronize()


def test_replays_on_the_legacy_default_stream(batch_inputs):
    """A context whose stream is the legacy default stream (what a caller
    handing over torch's default stream gives it) still records the batch --
    on its own capture stream -- and replays it on the caller's stream."""
    import torch

    import mdet_gb300 as m

    with m.Context(0) as ctx:
        ctx.set_stream(0)
        outs, items = [], []
        for x in batch_inputs:
            o = _outputs(torch, x["n"], x["max_edges"])
            outs.append(o)
            items.append(dict(d_tnf=x["d_tnf"].data_ptr(), d_ls=x["d_ls"].data_ptr(), n=x["n"], cutoff=x["cutoff"],
                              max_edges=x["max_edges"], d_from=o[0].data_ptr(), d_to=o[1].data_ptr(),
                              d_stnf=o[2].data_ptr(), capacity=o[3]))
        singles = [_single(ctx, torch, x, "bf16") for x in batch_inputs]
        r0 = ctx.graph_replays()
        for call in range(3):
            res, _ = ctx.tnf_graph_batched(items, mode="bf16")
            for (status, ne), o, (f, t, st) in zip(res, outs, singles):
                assert status == 0 and ne == f.size
                assert np.array_equal(o[0][:ne].cpu().numpy(), f) and np.array_equal(o[2][:ne].cpu().numpy(), st)
        assert ctx.graph_replays() == r0 + 2


def test_batch_capacity_shortfall(gpu_ctx, batch_inputs):
    import torch

    x0, x1 = batch_inputs[0], batch_inputs[3]
    f0, _, _ = _single(gpu_ctx, torch, x0, "bf16")
    small = _outputs(torch, 1, 1, cap=max(1, f0.size // 2))
    big = _outputs(torch, x1["n"], x1["max_edges"])
    items = [dict(d_tnf=x0["d_tnf"].data_ptr(), d_ls=x0["d_ls"].data_ptr(), n=x0["n"], cutoff=x0["cutoff"],
                  max_edges=x0["max_edges"], d_from=small[0].data_ptr(), d_to=small[1].data_ptr(),
                  d_stnf=small[2].data_ptr(), capacity=small[3]),
             dict(d_tnf=x1["d_tnf"].data_ptr(), d_ls=x1["d_ls"].data_ptr(), n=x1["n"], cutoff=x1["cutoff"],
                  max_edges=x1["max_edges"], d_from=big[0].data_ptr(), d_to=big[1].data_ptr(),
                  d_stnf=big[2].data_ptr(), capacity=big[3])]
    res, _ = gpu_ctx.tnf_graph_batched(items, mode="bf16")
    from mdet_gb300.tnf import ERR_CAPACITY

    assert res[0] == (ERR_CAPACITY, f0.size)
    f1, t1, s1 = _single(gpu_ctx, torch, x1, "bf16")
    assert res[1] == (0, f1.size)
    assert np.array_equal(big[1][:f1.size].cpu().numpy(), t1)
