"""ctypes view of the CPU oracle (oracle/tnf_oracle.cpp).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline leg -- never by the product.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "liboracle.so")
REF_PROB = os.path.join(HERE, "_ref", "libref_prob.so")
REF_TNF = os.path.join(HERE, "_ref", "omp_ex")

P = ctypes.c_void_p
u64 = ctypes.c_uint64
D = ctypes.c_double
_lib = None


def build():
    subprocess.check_call(["make", "-s", "-C", HERE, "all"])


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            build()
        L = ctypes.CDLL(LIB)
        L.orc_tn_order.restype = ctypes.c_char_p
        L.orc_tnmap.argtypes = [P]
        L.orc_base_code.argtypes = [P]
        L.orc_tnf_count.argtypes = [P, P, P, u64, P, P, ctypes.c_int]
        L.orc_tnf_normalize_f64.argtypes = [P, u64, P]
        for f in ("orc_pre_prob", "orc_tnf_dist_cpu"):
            getattr(L, f).restype = D
            getattr(L, f).argtypes = [D, D, P, P]
        L.orc_tnf_distance.restype = D
        L.orc_tnf_distance.argtypes = [P, P]
        L.orc_pre_prob_from_d.restype = D
        L.orc_pre_prob_from_d.argtypes = [D, D, D]
        L.orc_pair_scores.argtypes = [P, P, P, u64, P, P, ctypes.c_int]
        L.orc_logit_cutoff.restype = D
        L.orc_logit_cutoff.argtypes = [D]
        L.orc_tnf_graph.restype = u64
        L.orc_tnf_graph.argtypes = [P, P, u64, D, ctypes.c_uint32, u64, u64, P, P, P, u64, ctypes.c_int]
        L.orc_tnf_topk_rows.restype = u64
        L.orc_tnf_topk_rows.argtypes = [P, P, u64, D, ctypes.c_uint32, u64, u64, P, P, P, u64, ctypes.c_int]
        L.orc_max_prob.argtypes = [P, P, u64, P, u64, P, ctypes.c_int]
        L.orc_srand.argtypes = [ctypes.c_uint32]
        L.orc_rand.restype = ctypes.c_int
        L.orc_ptnf_search.restype = D
        L.orc_ptnf_search.argtypes = [P, P, u64, D, ctypes.c_int]
        L.orc_tnf_graph_nz.restype = u64
        L.orc_tnf_graph_nz.argtypes = [P, P, u64, D, ctypes.c_uint32, u64, u64, P, P, P, u64, ctypes.c_int, P]
        L.orc_tnf_topk_rows_nz.restype = u64
        L.orc_tnf_topk_rows_nz.argtypes = [P, P, u64, D, ctypes.c_uint32, u64, u64, P, P, P, u64, ctypes.c_int, P]
        L.orc_abd_low.argtypes = [P, u64, ctypes.c_uint32, P]
        L.orc_sscr.argtypes = [P, P, P, u64, P, P, ctypes.c_uint32, D, ctypes.c_uint32, P, ctypes.c_int]
        L.orc_tnf_graph_rows.restype = u64
        L.orc_tnf_graph_rows.argtypes = [P, P, u64, D, ctypes.c_uint32, P, u64, P, P, P, u64, ctypes.c_int]
        L.orc_recruit.argtypes = [P, P, u64, u64, ctypes.c_uint32, P, P, P, u64, u64, P, P, P]
        L.orc_fasta_index.restype = u64
        L.orc_fasta_index.argtypes = [P, u64, u64, P, P, P, P, P]
        L.orc_label_prop.argtypes = [P, P, P, u64, u64, D, D, P, P]
        L.orc_umap_order.argtypes = [P, u64, P]
        L.orc_umap_emulated.argtypes = [P, u64, P]
        for f in ("orc_lp_log", "orc_lp_exp"):
            getattr(L, f).restype = D
            getattr(L, f).argtypes = [D]
        L.orc_lp_chi2_cdf.restype = D
        L.orc_lp_chi2_cdf.argtypes = [u64, D]
        _lib = L
    return _lib


def _p(a):
    return ctypes.c_void_p(a.ctypes.data)


def tnmap():
    m = np.zeros(256, np.uint8)
    lib().orc_tnmap(_p(m))
    return m


def tn_order():
    s = lib().orc_tn_order().decode()
    return [s[4 * i:4 * i + 4] for i in range(136)]


def tnf_count(data, off, ln, threads=0):
    data = np.ascontiguousarray(data, np.uint8)
    off = np.ascontiguousarray(off, np.uint64)
    ln = np.ascontiguousarray(ln, np.uint64)
    n = off.size
    c = np.zeros((n, 136), np.uint32)
    t = np.zeros((n, 136), np.float32)
    lib().orc_tnf_count(_p(data), _p(off), _p(ln), n, _p(c), _p(t), threads)
    return c, t


def normalize_f64(counts):
    counts = np.ascontiguousarray(counts, np.uint32)
    out = np.zeros(counts.shape, np.float64)
    lib().orc_tnf_normalize_f64(_p(counts), counts.shape[0], _p(out))
    return out


def pre_prob(r1, r2, a, b):
    a = np.ascontiguousarray(a, np.float32)
    b = np.ascontiguousarray(b, np.float32)
    return lib().orc_pre_prob(r1, r2, _p(a), _p(b))


def pair_scores(tnf, ls, pairs, threads=0):
    """(distance, probability) of index pairs (m x 2) in FP64."""
    tnf = np.ascontiguousarray(tnf, np.float32)
    ls = np.ascontiguousarray(ls, np.float64)
    pr = np.ascontiguousarray(pairs, np.uint64)
    m = pr.shape[0]
    d = np.zeros(m, np.float64)
    p = np.zeros(m, np.float64)
    lib().orc_pair_scores(_p(tnf), _p(ls), _p(pr), m, _p(d), _p(p), threads)
    return d, p


def _low_arg(low, n):
    if low is None:
        return None, None
    low = np.ascontiguousarray(low, np.uint8)
    assert low.size == n
    return low, _p(low)


def graph(tnf, ls, cutoff, max_edges=200, row0=0, row1=None, threads=0, low=None):
    """low (optional): per contig 1 when no depth exceeds 1 (the abundance
    pair gate, see abd_low)."""
    tnf = np.ascontiguousarray(tnf, np.float32)
    ls = np.ascontiguousarray(ls, np.float64)
    n = tnf.shape[0]
    row1 = n if row1 is None else row1
    cap = max(1, (row1 - row0) * max_edges)
    fr = np.zeros(cap, np.uint64)
    to = np.zeros(cap, np.uint64)
    st = np.zeros(cap, np.float64)
    low, lp = _low_arg(low, n)
    k = lib().orc_tnf_graph_nz(_p(tnf), _p(ls), n, cutoff, max_edges, row0, row1, _p(fr), _p(to), _p(st), cap,
                               threads, lp)
    return fr[:k], to[:k], st[:k]


def topk_rows(tnf, ls, cutoff, max_edges=200, row0=0, row1=None, threads=0, low=None):
    tnf = np.ascontiguousarray(tnf, np.float32)
    ls = np.ascontiguousarray(ls, np.float64)
    n = tnf.shape[0]
    row1 = n if row1 is None else row1
    cap = max(1, (row1 - row0) * max_edges)
    rp = np.zeros(row1 - row0 + 1, np.uint64)
    cols = np.zeros(cap, np.uint64)
    sims = np.zeros(cap, np.float64)
    low, lp = _low_arg(low, n)
    lib().orc_tnf_topk_rows_nz(_p(tnf), _p(ls), n, cutoff, max_edges, row0, row1, _p(rp), _p(cols), _p(sims), cap,
                               threads, lp)
    return rp, cols, sims


def abd_low(abd):
    """1 per contig none of whose depths exceeds 1 (is_nz's threshold)."""
    abd = np.ascontiguousarray(abd, np.float64)
    low = np.zeros(abd.shape[0], np.uint8)
    lib().orc_abd_low(_p(abd), abd.shape[0], abd.shape[1], _p(low))
    return low


def sscr(from_, to, stnf, abd, var, min_cv=1.0, min_sample=3, threads=0):
    """sTNF -> sSCR of edges (from_, to, stnf) with coverage abd / var (n x nabd)."""
    f = np.ascontiguousarray(from_, np.uint64)
    t = np.ascontiguousarray(to, np.uint64)
    s = np.ascontiguousarray(stnf, np.float64)
    abd = np.ascontiguousarray(abd, np.float64)
    var = np.ascontiguousarray(var, np.float64)
    out = np.zeros(s.size, np.float64)
    lib().orc_sscr(_p(f), _p(t), _p(s), s.size, _p(abd), _p(var), abd.shape[1], min_cv, min_sample, _p(out), threads)
    return out


def max_prob(tnf, ls, contigs, m, threads=0):
    tnf = np.ascontiguousarray(tnf, np.float32)
    ls = np.ascontiguousarray(ls, np.float64)
    c = np.ascontiguousarray(contigs, np.uint64)
    out = np.zeros(m, np.float64)
    lib().orc_max_prob(_p(tnf), _p(ls), tnf.shape[0], _p(c), m, _p(out), threads)
    return out


def ptnf_search(tnf, ls, coverage=0.95, seed=1, threads=0):
    tnf = np.ascontiguousarray(tnf, np.float32)
    ls = np.ascontiguousarray(ls, np.float64)
    lib().orc_srand(seed)
    return lib().orc_ptnf_search(_p(tnf), _p(ls), tnf.shape[0], coverage, threads)


def srand(seed):
    lib().orc_srand(seed)


def fasta_index(data):
    """Every record of a FASTA buffer: (seq_off, seq_len, size, name_off, name_len)."""
    data = np.ascontiguousarray(data, np.uint8)
    n = lib().orc_fasta_index(_p(data), data.size, 0, None, None, None, None, None)
    cap = max(1, n)
    so, sl, sz, no = (np.zeros(cap, np.uint64) for _ in range(4))
    nl = np.zeros(cap, np.uint32)
    lib().orc_fasta_index(_p(data), data.size, cap, _p(so), _p(sl), _p(sz), _p(no), _p(nl))
    return so[:n], sl[:n], sz[:n], no[:n], nl[:n]


REF_RECRUIT = os.path.join(HERE, "_ref", "libref_recruit.so")


def _recruit_args(abd, small_abd, label, sizes, small_sizes):
    abd = np.array(abd, np.float32, order="C", copy=True)  # ranked in place, as in the reference
    n, nabd = abd.shape
    small = np.array(small_abd, np.float32, order="C", copy=True).reshape(-1, nabd)
    lab = np.ascontiguousarray(label, np.int64)
    sz = np.ascontiguousarray(sizes, np.uint64)
    ssz = np.ascontiguousarray(small_sizes, np.uint64)
    assert lab.size == n and sz.size == n and ssz.size == small.shape[0]
    return abd, small, lab, sz, ssz, n, small.shape[0], nabd


def recruit(abd, small_abd, label, sizes, small_sizes, min_cls_size=200000, small_total=0):
    """Dissolving small bins and recruiting leftover / small contigs
    (orc_recruit).  Returns (bin of each large contig, bin of each small
    contig, stats dict); -1 = no bin."""
    abd, small, lab, sz, ssz, n, n1, nabd = _recruit_args(abd, small_abd, label, sizes, small_sizes)
    out = np.zeros(n, np.int64)
    sout = np.zeros(max(n1, 1), np.int64)
    st = np.zeros(7, np.uint64)
    lib().orc_recruit(_p(abd), _p(small), n, n1, nabd, _p(lab), _p(sz), _p(ssz), min_cls_size, small_total, _p(out),
                      _p(sout), _p(st))
    keys = ["bins", "bins_scored", "leftovers", "leftovers_matched", "small_matched", "leftovers_accepted",
            "small_accepted"]
    return out, sout[:n1], dict(zip(keys, (int(x) for x in st)))


def ref_recruit(abd, small_abd, label, sizes, small_sizes, min_cls_size=200000, verbose=False):
    """The reference's own block (oracle/_ref/libref_recruit.so, built where
    the reference is mounted)."""
    abd, small, lab, sz, ssz, n, n1, nabd = _recruit_args(abd, small_abd, label, sizes, small_sizes)
    L = ctypes.CDLL(REF_RECRUIT)
    L.ref_recruit.argtypes = [P, P, u64, u64, ctypes.c_uint32, P, P, P, u64, ctypes.c_int, P, P]
    out = np.zeros(n, np.int64)
    sout = np.zeros(max(n1, 1), np.int64)
    L.ref_recruit(_p(abd), _p(small), n, n1, nabd, _p(lab), _p(sz), _p(ssz), min_cls_size, 1 if verbose else 0,
                  _p(out), _p(sout))
    return out, sout[:n1]


def graph_rows(tnf, ls, cutoff, max_edges, rows, threads=0):
    """The reference's graph edges (i < j) of the listed rows only."""
    tnf = np.ascontiguousarray(tnf, np.float32)
    ls = np.ascontiguousarray(ls, np.float64)
    rows = np.ascontiguousarray(rows, np.uint64)
    cap = max(1, rows.size * max_edges)
    fr, to, st = np.zeros(cap, np.uint64), np.zeros(cap, np.uint64), np.zeros(cap, np.float64)
    k = lib().orc_tnf_graph_rows(_p(tnf), _p(ls), tnf.shape[0], cutoff, max_edges, _p(rows), rows.size, _p(fr), _p(to),
                                 _p(st), cap, threads)
    return fr[:k], to[:k], st[:k]


LP_STATS = ["calls", "sweeps", "graph_edges", "connected", "frozen", "ties"]
REF_LP = os.path.join(HERE, "_ref", "libref_lp.so")


def _lp_args(from_, to, sscr):
    fr = np.ascontiguousarray(from_, np.uint64)
    t = np.ascontiguousarray(to, np.uint64)
    s = np.ascontiguousarray(sscr, np.float64)
    assert fr.size == t.size == s.size
    return fr, t, s


def label_prop(from_, to, sscr, n, max_p=0.95, min_s=0.60):
    """The binning traversal and its label propagation calls
    (orc_label_prop).  Returns (bin of every contig, stats dict)."""
    fr, t, s = _lp_args(from_, to, sscr)
    mem = np.zeros(max(n, 1), np.uint64)
    st = np.zeros(6, np.uint64)
    lib().orc_label_prop(_p(fr), _p(t), _p(s), s.size, n, max_p, min_s, _p(mem), _p(st))
    return mem[:n], dict(zip(LP_STATS, (int(x) for x in st)))


def ref_label_prop(from_, to, sscr, n, max_p=0.95, min_s=0.60):
    """The reference's own traversal and label_propagation
    (oracle/_ref/libref_lp.so, built where the reference is mounted).
    Returns (bin of every contig, number of propagation calls)."""
    fr, t, s = _lp_args(from_, to, sscr)
    L = ctypes.CDLL(REF_LP)
    L.ref_label_prop.argtypes = [P, P, P, u64, u64, D, D, P]
    L.ref_label_prop.restype = u64
    mem = np.zeros(max(n, 1), np.uint64)
    calls = L.ref_label_prop(_p(fr), _p(t), _p(s), s.size, n, max_p, min_s, _p(mem))
    return mem[:n], int(calls)


def umap_order(keys):
    """Iteration order of this C++ library's unordered_map after inserting
    the distinct keys in turn."""
    k = np.ascontiguousarray(keys, np.uint64)
    out = np.zeros(max(k.size, 1), np.uint64)
    lib().orc_umap_order(_p(k), k.size, _p(out))
    return out[:k.size]


def umap_emulated(keys):
    """The same order from the emulation the device form uses (lp_umap.h)."""
    k = np.ascontiguousarray(keys, np.uint64)
    out = np.zeros(max(k.size, 1), np.uint64)
    lib().orc_umap_emulated(_p(k), k.size, _p(out))
    return out[:k.size]
