"""The edge-set comparison used by the config-scale parity tests and the
bench's recall figure, checked on the CPU: the oracle's own graph matches
itself; a dropped edge, an extra edge and a changed sTNF are caught."""
import numpy as np

from oracle import oracle, parity


def _set():
    from mdet_gb300 import synth

    a = synth.generate(seed=31, n=900, genomes=15, max_len=80000, threads=4)
    _, tnf = oracle.tnf_count(a.data, a.seq_off, a.seq_len)
    return a, tnf


def test_oracle_graph_matches_itself_and_mistakes_are_caught():
    a, tnf = _set()
    ls = a.log_sizes
    fr, to, st = oracle.graph(tnf, ls, 0.9, 40)
    r = parity.compare_rows(fr, to, st, tnf, ls, 0.9, 40)
    assert r["recall"] == 1.0 and r["precision"] == 1.0 and r["ref_edges"] == fr.size
    parity.assert_rows_match(r)
    # a row range alone
    r2 = parity.compare_rows(fr, to, st, tnf, ls, 0.9, 40, 100, 400)
    assert r2["common"] == int(((fr >= 100) & (fr < 400)).sum())
    # a dropped edge far from the band
    sims = st.copy()
    far = np.flatnonzero(np.abs(sims - 0.9) > 1e-3)
    k = int(far[len(far) // 2])
    r3 = parity.compare_rows(np.delete(fr, k), np.delete(to, k), np.delete(st, k), tnf, ls, 0.9, 40)
    assert r3["missed"] == 1 and len(r3["outside_band"]) == 1 and r3["recall"] < 1.0
    # an extra edge (a pair the oracle does not keep)
    ref = set(zip(fr.tolist(), to.tolist()))
    i, j = next((i, j) for i in range(5, 50) for j in range(i + 1, 900) if (i, j) not in ref)
    r4 = parity.compare_rows(np.append(fr, i), np.append(to, j), np.append(st, 0.5), tnf, ls, 0.9, 40)
    assert r4["extra"] == 1 and r4["precision"] < 1.0
    # a changed sTNF on a common edge
    st5 = st.copy()
    st5[k] += 1e-7
    r5 = parity.compare_rows(fr, to, st5, tnf, ls, 0.9, 40)
    assert r5["max_sim_diff"] > parity.SIM_TOL
