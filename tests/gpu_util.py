"""Helpers shared by the GPU parity tests (comparison within the tolerance
band that the parity contract allows)."""
import numpy as np

from oracle import oracle

BAND = 1e-5  # probability band around the cutoff and each row's top-k cutoff


def synth_set(seed, n, genomes, max_len=500000):
    from mdet_gb300 import synth

    a = synth.generate(seed=seed, n=n, genomes=genomes, max_len=max_len, threads=8)
    counts, tnf = oracle.tnf_count(a.data, a.seq_off, a.seq_len)
    return a, counts, tnf


def exact_sim(tnf, ls, i, j):
    pre = oracle.pre_prob(ls[i], ls[j], tnf[i], tnf[j])
    return 1.0 - 1.0 / (1.0 + np.exp(pre)), pre


def compare_graph(gpu_from, gpu_to, gpu_sim, tnf, ls, cutoff, max_edges, low=None):
    """Edge sets must match except pairs whose probability lies within BAND of
    the cutoff or of either row's top-k cutoff; common edges must agree on
    sTNF.  low: the abundance pair gate of the oracle (optional).  Returns
    (n_common, n_band_exempt)."""
    n = tnf.shape[0]
    rp, cols, sims = oracle.topk_rows(tnf, ls, cutoff, max_edges, low=low)
    kth = np.full(n, -np.inf)
    for i in range(n):
        if rp[i + 1] - rp[i] == max_edges:
            kth[i] = sims[rp[i]:rp[i + 1]].min()
    ref = {}
    for i in range(n):
        for c, s in zip(cols[rp[i]:rp[i + 1]], sims[rp[i]:rp[i + 1]]):
            if i < c:
                ref[(i, int(c))] = s
    got = {(int(f), int(t)): s for f, t, s in zip(gpu_from, gpu_to, gpu_sim)}
    assert len(got) == len(gpu_from), "duplicate edges in GPU output"
    exempt = 0
    for key in set(ref) ^ set(got):
        i, j = key
        s, _ = exact_sim(tnf, ls, i, j)
        near = abs(s - cutoff) <= BAND or abs(s - kth[i]) <= BAND
        assert near, f"edge {key} sim={s:.12f} differs outside the band (cutoff {cutoff}, kth {kth[i]})"
        exempt += 1
    common = set(ref) & set(got)
    for key in common:
        assert abs(ref[key] - got[key]) <= 1e-9, (key, ref[key], got[key])
    return len(common), exempt
