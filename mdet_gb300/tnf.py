"""Python host mirror of the reference's TNF-path interface over the C ABI.

The reference (cuda/Cuda2.cu) exposes its TNF path as free functions over
globals; this module gives the same operations as methods of a Context that
owns device memory, with the reference's names kept as aliases:

  calc_tnf            TNF loop of main            (cuda/Cuda2.cu:1825-1863)
  max_prob_sample     launch_tnf_max_prob_sample_kernel_multi (356-379)
  gen_tnf_graph_sample  pTNF search + driver    (972-1025, 1883-1904)
  gen_tnf_graph       gen_tnf_graph             (861-970)

Every call goes through libmdet_tnf.so (include/mdet_tnf.h).  There is no
CPU fallback: if the library is missing, loading raises.
"""
from __future__ import annotations

import ctypes
import os
from dataclasses import dataclass

import numpy as np

_LIB_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "_lib", "libmdet_tnf.so")

OK, ERR_INVALID, ERR_CUDA, ERR_NOMEM, ERR_CAPACITY, ERR_TIMEOUT, ERR_UNSUPPORTED = range(7)
MODES = {"plain": 0, "bf16": 1, "tf32": 2, "learned": 3}

u64 = ctypes.c_uint64
u32 = ctypes.c_uint32
P = ctypes.c_void_p
D = ctypes.c_double


class RecruitStats(ctypes.Structure):
    _fields_ = [("n_bins", u64), ("n_bins_scored", u64), ("n_leftovers", u64), ("n_leftovers_matched", u64),
                ("n_small_matched", u64), ("binned_bases", u64), ("leftover_bases", u64), ("small_bases", u64),
                ("leftovers_accepted", ctypes.c_int), ("small_accepted", ctypes.c_int), ("pairs_tested", u64),
                ("pairs_exact", u64), ("pairs_undecided", u64), ("bins_exact", u64)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class LpStats(ctypes.Structure):
    _fields_ = [("calls", u64), ("sweeps", u64), ("graph_edges", u64), ("connected", u64), ("frozen", u64),
                ("ties", u64), ("levels_max", u64), ("degree_max", u64), ("ms_total", D)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class FastaStats(ctypes.Structure):
    _fields_ = [("n_records", u64), ("n_large", u64), ("n_small", u64), ("ms_total", D)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class GraphStats(ctypes.Structure):
    _fields_ = [
        ("n_candidates", u64),
        ("n_above_cutoff", u64),
        ("n_edges", u64),
        ("tiles_total", u64),
        ("tiles_computed", u64),
        ("gpu_launches", u32),
        ("tile_m_n", u32),
        ("ms_prep", D),
        ("ms_filter", D),
        ("ms_exact", D),
        ("ms_select", D),
        ("ms_total", D),
    ]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class Assembly(ctypes.Structure):
    _fields_ = [
        ("d_tnf", P),
        ("d_log_size", P),
        ("n", u64),
        ("cutoff", D),
        ("max_edges", u32),
        ("status", ctypes.c_int32),
        ("d_from", P),
        ("d_to", P),
        ("d_stnf", P),
        ("capacity", u64),
        ("n_edges", u64),
    ]


class TrainParams(ctypes.Structure):
    _fields_ = [
        ("pairs", u64),
        ("candidate_fraction", D),
        ("label_cutoff", D),
        ("steps", u64),
        ("batch_pairs", u32),
        ("lr", ctypes.c_float),
        ("m_pos", ctypes.c_float),
        ("m_neg", ctypes.c_float),
        ("tau_quantile", D),
        ("seed", u64),
    ]


class TrainReport(ctypes.Structure):
    _fields_ = [
        ("steps", u64),
        ("pairs", u64),
        ("candidate_pairs", u64),
        ("held_pos", u64),
        ("held_neg", u64),
        ("final_loss", D),
        ("tau", D),
        ("pos_median", D),
        ("neg_median", D),
        ("neg_below_tau", D),
    ]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class LearnedReport(ctypes.Structure):
    _fields_ = [
        ("recall_target", D),
        ("recall_rows", u32),
        ("segment", u32),
        ("recall", D),
        ("fell_back", u32),
        ("order", u32),
        ("tiles_skipped", u64),
        ("tau", D),
        ("ms_embed", D),
        ("ms_order", D),
        ("ms_sample", D),
        ("tau_quantile", D),
    ]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


# (name, restype, argtypes) of every entry point in include/mdet_tnf.h
SIGNATURES = [
    ("mdet_ctx_create", ctypes.c_int, [ctypes.c_int, ctypes.POINTER(P)]),
    ("mdet_ctx_destroy", ctypes.c_int, [P]),
    ("mdet_last_error", ctypes.c_char_p, [P]),
    ("mdet_ctx_set_stream", ctypes.c_int, [P, P]),
    ("mdet_version", ctypes.c_char_p, []),
    ("mdet_ctx_set_timing", ctypes.c_int, [P, ctypes.c_int]),
    ("mdet_ctx_kernel_ms", ctypes.c_int, [P, ctypes.c_char_p, ctypes.POINTER(D), ctypes.POINTER(u32)]),
    ("mdet_ctx_launch_count", u64, [P]),
    ("mdet_ctx_set_autotune", ctypes.c_int, [P, ctypes.c_int]),
    ("mdet_tnf_count", ctypes.c_int, [P, P, u64, P, P, u64, P, P]),
    ("mdet_tnf_count_dev", ctypes.c_int, [P, P, u64, P, P, u64, P, P]),
    ("mdet_tnf_count_noalloc", ctypes.c_int, [P, u64, P, P, u64, P, P, P]),
    ("mdet_ctx_check_wait", ctypes.c_int, [P, u64]),
    ("mdet_recruit", ctypes.c_int, [P, P, P, u64, u64, ctypes.c_uint32, P, P, P, u64, u64, P, P, P]),
    ("mdet_label_propagation", ctypes.c_int, [P, P, P, P, u64, u64, D, D, P, ctypes.POINTER(LpStats)]),
    ("mdet_label_propagation_dev", ctypes.c_int, [P, P, P, P, u64, u64, D, D, P, ctypes.POINTER(LpStats)]),
    ("mdet_tnf_max_prob", ctypes.c_int, [P, P, P, u64, P, u64, ctypes.c_int, D, P]),
    ("mdet_tnf_max_prob_dev", ctypes.c_int, [P, P, P, u64, P, u64, ctypes.c_int, D, P]),
    ("mdet_tnf_ptnf_search", ctypes.c_int, [P, P, P, u64, D, ctypes.c_int, ctypes.POINTER(D)]),
    ("mdet_tnf_ptnf_search_dev", ctypes.c_int, [P, P, P, u64, D, ctypes.c_int, ctypes.POINTER(D)]),
    ("mdet_tnf_graph", ctypes.c_int,
     [P, P, P, u64, D, u32, ctypes.c_int, P, P, P, u64, ctypes.POINTER(u64), ctypes.POINTER(GraphStats)]),
    ("mdet_tnf_graph_dev", ctypes.c_int,
     [P, P, P, u64, D, u32, ctypes.c_int, P, P, P, u64, ctypes.POINTER(u64), ctypes.POINTER(GraphStats)]),
    ("mdet_tnf_pair_scores_dev", ctypes.c_int, [P, P, P, u64, P, u64, P, P]),
    ("mdet_tnf_graph_shard", ctypes.c_int,
     [P, P, P, u64, D, u32, ctypes.c_int, u32, u32, P, P, P, u64, ctypes.POINTER(u64), ctypes.POINTER(GraphStats)]),
    ("mdet_tnf_graph_shard_dev", ctypes.c_int,
     [P, P, P, u64, D, u32, ctypes.c_int, u32, u32, P, P, P, u64, ctypes.POINTER(u64), ctypes.POINTER(GraphStats)]),
    ("mdet_tnf_graph_batched", ctypes.c_int, [P, ctypes.POINTER(Assembly), u32, ctypes.c_int,
                                              ctypes.POINTER(GraphStats)]),
    ("mdet_ctx_set_graph_capture", ctypes.c_int, [P, ctypes.c_int]),
    ("mdet_ctx_graph_replays", u64, [P]),
    ("mdet_mlp_create", ctypes.c_int, [P, u64, ctypes.POINTER(P)]),
    ("mdet_mlp_destroy", ctypes.c_int, [P]),
    ("mdet_mlp_param_count", u64, []),
    ("mdet_mlp_get_params", ctypes.c_int, [P, P, P, u64]),
    ("mdet_mlp_set_params", ctypes.c_int, [P, P, P, u64]),
    ("mdet_mlp_embed_dev", ctypes.c_int, [P, P, P, u64, P]),
    ("mdet_mlp_grad", ctypes.c_int,
     [P, P, P, u64, P, P, u64, ctypes.c_float, ctypes.c_float, P, ctypes.POINTER(D)]),
    ("mdet_mlp_train", ctypes.c_int,
     [P, P, P, P, u64, ctypes.POINTER(TrainParams), ctypes.POINTER(TrainReport)]),
    ("mdet_ctx_set_learned", ctypes.c_int, [P, P, ctypes.POINTER(LearnedReport)]),
    ("mdet_ctx_set_abundance", ctypes.c_int, [P, P, P, u64, u32]),
    ("mdet_host_alloc", ctypes.c_int, [u64, ctypes.POINTER(P)]),
    ("mdet_host_free", ctypes.c_int, [P]),
    ("mdet_fasta_index", ctypes.c_int, [P, P, u64, u64, u64, P, P, P, P, P, P, ctypes.POINTER(FastaStats)]),
    ("mdet_fasta_index_dev", ctypes.c_int, [P, P, u64, u64, u64, P, P, P, P, P, P, ctypes.POINTER(FastaStats)]),
    ("mdet_tnf_count_fasta", ctypes.c_int, [P, P, u64, u64, u64, P, P, P, P, P, P, P, P, ctypes.POINTER(FastaStats)]),
    ("mdet_edges_sscr", ctypes.c_int, [P, P, P, P, u64, D, u32, P]),
    ("mdet_edges_sscr_dev", ctypes.c_int, [P, P, P, P, u64, D, u32, P]),
]

_lib = None


def load_library(path: str | None = None):
    """Load libmdet_tnf.so (raises OSError if it has not been built)."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or _LIB_PATH
    if not os.path.exists(p):
        raise OSError(f"{p} not found: build the CUDA extension first (python -m mdet_gb300.build)")
    lib = ctypes.CDLL(p)
    for name, res, args in SIGNATURES:
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    if path is None:
        _lib = lib
    return lib


class MdetError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"[mdet status {code}] {msg}")
        self.code = code


def _ptr(a: np.ndarray):
    return ctypes.c_void_p(a.ctypes.data)


@dataclass
class Graph:
    """Edge list of the TNF graph (the reference's Graph from/to/sTNF)."""
    n: int
    from_: np.ndarray
    to: np.ndarray
    sTNF: np.ndarray
    stats: dict

    def getEdgeCount(self) -> int:
        return int(self.from_.size)


class Context:
    """Owns a device, a CUDA stream and scratch memory (mdet_ctx)."""

    def __init__(self, device: int = 0):
        self.lib = load_library()
        h = P()
        rc = self.lib.mdet_ctx_create(device, ctypes.byref(h))
        if rc != OK:
            raise MdetError(rc, f"mdet_ctx_create(device={device}) failed")
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            self.lib.mdet_ctx_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc):
        if rc != OK:
            raise MdetError(rc, self.lib.mdet_last_error(self.h).decode())

    def set_stream(self, stream_handle: int):
        self._check(self.lib.mdet_ctx_set_stream(self.h, P(stream_handle)))

    def set_timing(self, enable: bool):
        self._check(self.lib.mdet_ctx_set_timing(self.h, 1 if enable else 0))

    def kernel_ms(self, kernel: str):
        ms = D()
        n = u32()
        self._check(self.lib.mdet_ctx_kernel_ms(self.h, kernel.encode(), ctypes.byref(ms), ctypes.byref(n)))
        return ms.value, n.value

    def set_autotune(self, mode):
        """True/False: tune or not; 128256, 128128, 256128: force that filter tile shape."""
        m = (1 if mode else 0) if isinstance(mode, bool) else int(mode)
        self._check(self.lib.mdet_ctx_set_autotune(self.h, m))

    def launch_count(self) -> int:
        return int(self.lib.mdet_ctx_launch_count(self.h))

    # ---- TNF counting -------------------------------------------------
    def tnf_count(self, data: np.ndarray, seq_off: np.ndarray, seq_len: np.ndarray, out=None):
        """Counts (n x 136 uint32) and TNF (n x 136 float32); `out` may give
        preallocated (e.g. pinned) output arrays.  out=(None, tnf): the TNF
        rows only (the counts are not copied back; counts is returned as None)."""
        data = np.ascontiguousarray(data, dtype=np.uint8)
        off = np.ascontiguousarray(seq_off, dtype=np.uint64)
        ln = np.ascontiguousarray(seq_len, dtype=np.uint64)
        n = off.size
        if out is None:
            counts = np.zeros((n, 136), np.uint32)
            tnf = np.zeros((n, 136), np.float32)
        else:
            counts, tnf = out
            assert counts is None or (counts.dtype == np.uint32 and counts.size >= n * 136
                                      and counts.flags.c_contiguous)
            assert tnf.dtype == np.float32 and tnf.size >= n * 136 and tnf.flags.c_contiguous
        self._check(self.lib.mdet_tnf_count(self.h, _ptr(data), data.size, _ptr(off), _ptr(ln), n,
                                            None if counts is None else _ptr(counts), _ptr(tnf)))
        return counts, tnf

    def tnf_count_dev(self, d_bytes: int, nbytes: int, d_off: int, d_len: int, n: int, d_counts: int, d_tnf: int):
        self._check(self.lib.mdet_tnf_count_dev(self.h, P(d_bytes), nbytes, P(d_off), P(d_len), n, P(d_counts),
                                                P(d_tnf)))

    # ---- max-probability sample --------------------------------------
    def max_prob(self, tnf, log_size, contigs, m=None, mode="bf16", floor_prob=0.7):
        tnf = np.ascontiguousarray(tnf, dtype=np.float32)
        ls = np.ascontiguousarray(log_size, dtype=np.float64)
        c = np.ascontiguousarray(contigs, dtype=np.uint64)
        n = tnf.shape[0]
        m = c.size if m is None else m
        out = np.zeros(m, np.float64)
        self._check(self.lib.mdet_tnf_max_prob(self.h, _ptr(tnf), _ptr(ls), n, _ptr(c), m, MODES[mode],
                                               float(floor_prob), _ptr(out)))
        return out

    def max_prob_dev(self, d_tnf, d_ls, n, d_contigs, m, mode, floor_prob, d_out):
        self._check(self.lib.mdet_tnf_max_prob_dev(self.h, P(d_tnf), P(d_ls), n, P(d_contigs), m, MODES[mode],
                                                   float(floor_prob), P(d_out)))

    def ptnf_search(self, tnf, log_size, coverage: float = 0.95, mode: str = "bf16") -> float:
        """pTNF in permille; consumes glibc rand() like the reference (seed it with srand)."""
        tnf = np.ascontiguousarray(tnf, dtype=np.float32)
        ls = np.ascontiguousarray(log_size, dtype=np.float64)
        out = D()
        self._check(self.lib.mdet_tnf_ptnf_search(self.h, _ptr(tnf), _ptr(ls), tnf.shape[0], coverage, MODES[mode],
                                                  ctypes.byref(out)))
        return out.value

    def ptnf_search_dev(self, d_tnf: int, d_ls: int, n: int, coverage: float = 0.95, mode: str = "bf16") -> float:
        out = D()
        self._check(self.lib.mdet_tnf_ptnf_search_dev(self.h, P(d_tnf), P(d_ls), n, coverage, MODES[mode],
                                                      ctypes.byref(out)))
        return out.value

    gen_tnf_graph_sample = ptnf_search

    # ---- graph ----------------------------------------------------------
    def tnf_graph(self, tnf, log_size, cutoff, max_edges=200, mode="bf16", out=None) -> Graph:
        """Edges (from < to) with sTNF; `out` may give preallocated (e.g.
        pinned) from/to/sTNF arrays, whose size is the capacity."""
        tnf = np.ascontiguousarray(tnf, dtype=np.float32)
        ls = np.ascontiguousarray(log_size, dtype=np.float64)
        n = tnf.shape[0]
        if out is None:
            cap = max(1, n * max_edges)
            fr = np.empty(cap, np.uint64)
            to = np.empty(cap, np.uint64)
            st = np.empty(cap, np.float64)
        else:
            fr, to, st = out
            cap = min(fr.size, to.size, st.size)
        ne = u64(0)
        stats = GraphStats()
        self._check(self.lib.mdet_tnf_graph(self.h, _ptr(tnf), _ptr(ls), n, float(cutoff), max_edges, MODES[mode],
                                            _ptr(fr), _ptr(to), _ptr(st), cap, ctypes.byref(ne),
                                            ctypes.byref(stats)))
        k = ne.value
        if out is not None:
            return Graph(n, fr[:k], to[:k], st[:k], stats.as_dict())
        return Graph(n, fr[:k].copy(), to[:k].copy(), st[:k].copy(), stats.as_dict())

    def tnf_graph_shard(self, tnf, log_size, cutoff, max_edges, mode, shard, nshards) -> Graph:
        """Row shard `shard` of `nshards` of the graph (mdet_tnf_graph_shard):
        the edges of the shard's block of size-sorted rows."""
        tnf = np.ascontiguousarray(tnf, dtype=np.float32)
        ls = np.ascontiguousarray(log_size, dtype=np.float64)
        n = tnf.shape[0]
        cap = max(1, ((n + nshards - 1) // nshards + 256) * max_edges)
        fr, to, st = np.empty(cap, np.uint64), np.empty(cap, np.uint64), np.empty(cap, np.float64)
        ne = u64(0)
        stats = GraphStats()
        self._check(self.lib.mdet_tnf_graph_shard(self.h, _ptr(tnf), _ptr(ls), n, float(cutoff), max_edges,
                                                  MODES[mode], shard, nshards, _ptr(fr), _ptr(to), _ptr(st), cap,
                                                  ctypes.byref(ne), ctypes.byref(stats)))
        k = ne.value
        return Graph(n, fr[:k].copy(), to[:k].copy(), st[:k].copy(), stats.as_dict())

    def tnf_graph_shard_dev(self, d_tnf, d_ls, n, cutoff, max_edges, mode, shard, nshards, d_from, d_to, d_stnf,
                            capacity):
        ne = u64(0)
        stats = GraphStats()
        self._check(self.lib.mdet_tnf_graph_shard_dev(self.h, P(d_tnf), P(d_ls), n, float(cutoff), max_edges,
                                                      MODES[mode], shard, nshards, P(d_from), P(d_to), P(d_stnf),
                                                      capacity, ctypes.byref(ne), ctypes.byref(stats)))
        return ne.value, stats.as_dict()

    def tnf_graph_dev(self, d_tnf, d_ls, n, cutoff, max_edges, mode, d_from, d_to, d_stnf, capacity):
        ne = u64(0)
        stats = GraphStats()
        self._check(self.lib.mdet_tnf_graph_dev(self.h, P(d_tnf), P(d_ls), n, float(cutoff), max_edges,
                                                MODES[mode], P(d_from), P(d_to), P(d_stnf), capacity,
                                                ctypes.byref(ne), ctypes.byref(stats)))
        return ne.value, stats.as_dict()

    def fasta_index(self, data, min_contig=2500, capacity=None):
        """The reference reader's record split of a FASTA buffer, on the GPU.
        Returns (seq_off, seq_len, sizes, log_sizes, names, stats) for the
        records with size >= min_contig, in file order."""
        data = np.ascontiguousarray(data, np.uint8)
        cap = int(capacity) if capacity is not None else max(1, data.size // 1000 + 16)
        while True:
            off, ln, sz, no = (np.empty(cap, np.uint64) for _ in range(4))
            ls = np.empty(cap, np.float64)
            nl = np.empty(cap, np.uint32)
            st = FastaStats()
            rc = self.lib.mdet_fasta_index(self.h, P(data.ctypes.data), data.size, int(min_contig), cap,
                                           P(off.ctypes.data), P(ln.ctypes.data), P(sz.ctypes.data),
                                           P(ls.ctypes.data), P(no.ctypes.data), P(nl.ctypes.data),
                                           ctypes.byref(st))
            if rc == ERR_CAPACITY and capacity is None and st.n_large > cap:
                cap = int(st.n_large)
                continue
            self._check(rc)
            break
        k = int(st.n_large)
        raw = data.tobytes() if k else b""
        names = [raw[int(o):int(o) + int(n)].decode(errors="replace") for o, n in zip(no[:k], nl[:k])]
        return off[:k], ln[:k], sz[:k], ls[:k], names, st.as_dict()

    def tnf_count_fasta(self, data, min_contig=2500, capacity=None):
        """Record split and TNF counting from FASTA bytes in one call.
        Returns (seq_off, seq_len, log_sizes, counts, tnf, stats) for the
        contigs with size >= min_contig, in file order."""
        data = np.ascontiguousarray(data, np.uint8)
        cap = int(capacity) if capacity is not None else max(1, data.size // 1000 + 16)
        while True:
            off, ln = np.empty(cap, np.uint64), np.empty(cap, np.uint64)
            ls = np.empty(cap, np.float64)
            counts = np.empty((cap, 136), np.uint32)
            tnf = np.empty((cap, 136), np.float32)
            st = FastaStats()
            rc = self.lib.mdet_tnf_count_fasta(self.h, P(data.ctypes.data), data.size, int(min_contig), cap,
                                               P(off.ctypes.data), P(ln.ctypes.data), None, P(ls.ctypes.data),
                                               None, None, P(counts.ctypes.data), P(tnf.ctypes.data),
                                               ctypes.byref(st))
            if rc == ERR_CAPACITY and capacity is None and st.n_large > cap:
                cap = int(st.n_large)
                continue
            self._check(rc)
            break
        k = int(st.n_large)
        return off[:k], ln[:k], ls[:k], counts[:k], tnf[:k], st.as_dict()

    def fasta_index_dev(self, d_bytes, nbytes, min_contig, capacity, d_seq_off, d_seq_len, d_size=None,
                        d_log_size=None, d_name_off=None, d_name_len=None):
        st = FastaStats()
        self._check(self.lib.mdet_fasta_index_dev(self.h, P(d_bytes), nbytes, int(min_contig), capacity,
                                                  P(d_seq_off), P(d_seq_len), P(d_size), P(d_log_size),
                                                  P(d_name_off), P(d_name_len), ctypes.byref(st)))
        return st.as_dict()

    def set_abundance(self, abd, var):
        """Coverage of the contigs (n x nabd mean depths and variances, the
        reference's ABD / ABD_VAR); None clears it.  While set, tnf_graph /
        tnf_graph_dev drop pairs of two contigs with no depth above 1."""
        if abd is None:
            self._check(self.lib.mdet_ctx_set_abundance(self.h, None, None, 0, 0))
            return
        abd = np.ascontiguousarray(abd, np.float64)
        var = np.ascontiguousarray(var, np.float64)
        if abd.ndim != 2 or var.shape != abd.shape:
            raise ValueError("abd and var must be n x nabd matrices of the same shape")
        self._check(self.lib.mdet_ctx_set_abundance(self.h, P(abd.ctypes.data), P(var.ctypes.data), abd.shape[0],
                                                    abd.shape[1]))

    def recruit(self, abd, small_abd, label, sizes, small_sizes, min_cls_size=200000, small_total=0):
        """Dissolve small bins and recruit leftover and small contigs
        (mdet_recruit).  abd: n x nabd, small_abd: n_small x nabd depths
        (float); label: bin label of each large contig.  Returns (bin of
        each large contig, bin of each small contig, stats); -1 = no bin."""
        abd = np.ascontiguousarray(abd, np.float32)
        n, nabd = abd.shape
        small = np.ascontiguousarray(small_abd, np.float32).reshape(-1, nabd)
        n1 = small.shape[0]
        lab = np.ascontiguousarray(label, np.int64)
        sz = np.ascontiguousarray(sizes, np.uint64)
        ssz = np.ascontiguousarray(small_sizes, np.uint64)
        out = np.zeros(n, np.int64)
        sout = np.zeros(max(n1, 1), np.int64)
        st = RecruitStats()
        self._check(self.lib.mdet_recruit(self.h, _ptr(abd), _ptr(small), n, n1, nabd, _ptr(lab), _ptr(sz), _ptr(ssz),
                                          int(min_cls_size), int(small_total), _ptr(out), _ptr(sout),
                                          ctypes.byref(st)))
        return out, sout[:n1], st.as_dict()

    def label_propagation(self, from_, to, sscr, n, max_p=0.95, min_s=0.60):
        """Bins by label propagation over the scored edges (host arrays;
        mdet_label_propagation): edge e joins to[e] and from[e].  max_p and
        min_s are fractions.  Returns (bin of every contig, stats)."""
        f = np.ascontiguousarray(from_, np.uint64)
        t = np.ascontiguousarray(to, np.uint64)
        sc = np.ascontiguousarray(sscr, np.float64)
        if not (f.size == t.size == sc.size):
            raise ValueError("from, to and sscr must have the same length")
        mem = np.zeros(max(n, 1), np.uint64)
        st = LpStats()
        self._check(self.lib.mdet_label_propagation(self.h, _ptr(f), _ptr(t), _ptr(sc), sc.size, n, max_p, min_s,
                                                    _ptr(mem), ctypes.byref(st)))
        return mem[:n], st.as_dict()

    def label_propagation_dev(self, d_from: int, d_to: int, d_sscr: int, n_edges: int, n: int, d_mem: int,
                              max_p=0.95, min_s=0.60) -> dict:
        """Device-pointer form (uint64 from/to, float64 scores, uint64 bins)."""
        st = LpStats()
        self._check(self.lib.mdet_label_propagation_dev(self.h, P(d_from), P(d_to), P(d_sscr), n_edges, n, max_p,
                                                        min_s, P(d_mem), ctypes.byref(st)))
        return st.as_dict()

    def edges_sscr(self, from_, to, stnf, min_cv=1.0, min_sample=3):
        """sTNF -> sSCR of edges (host arrays) with the context's abundance."""
        f = np.ascontiguousarray(from_, np.uint64)
        t = np.ascontiguousarray(to, np.uint64)
        s = np.ascontiguousarray(stnf, np.float64)
        if not (f.size == t.size == s.size):
            raise ValueError("from, to and stnf must have the same length")
        out = np.empty(s.size, np.float64)
        self._check(self.lib.mdet_edges_sscr(self.h, P(f.ctypes.data), P(t.ctypes.data), P(s.ctypes.data), s.size,
                                             float(min_cv), int(min_sample), P(out.ctypes.data)))
        return out

    def edges_sscr_dev(self, d_from, d_to, d_stnf, n_edges, d_sscr, min_cv=1.0, min_sample=3):
        self._check(self.lib.mdet_edges_sscr_dev(self.h, P(d_from), P(d_to), P(d_stnf), n_edges, float(min_cv),
                                                 int(min_sample), P(d_sscr)))

    def pair_scores_dev(self, d_tnf, d_ls, n, d_pairs, m, d_dist, d_prob):
        self._check(self.lib.mdet_tnf_pair_scores_dev(self.h, P(d_tnf), P(d_ls), n, P(d_pairs), m, P(d_dist),
                                                      P(d_prob)))

    def tnf_graph_batched(self, assemblies, mode="bf16"):
        """Graphs of many assemblies in one pass (device buffers).  Each item:
        dict(d_tnf, d_ls, n, cutoff, max_edges, d_from, d_to, d_stnf,
        capacity).  Returns ([(status, n_edges)], stats); capacity shortfalls
        are reported per assembly, not raised."""
        arr = (Assembly * len(assemblies))()
        for a, d in zip(arr, assemblies):
            a.d_tnf, a.d_log_size, a.n = P(d["d_tnf"]), P(d["d_ls"]), d["n"]
            a.cutoff, a.max_edges = float(d["cutoff"]), int(d["max_edges"])
            a.d_from, a.d_to, a.d_stnf = P(d["d_from"]), P(d["d_to"]), P(d["d_stnf"])
            a.capacity = int(d["capacity"])
        stats = GraphStats()
        rc = self.lib.mdet_tnf_graph_batched(self.h, arr, len(assemblies), MODES[mode], ctypes.byref(stats))
        if rc not in (OK, ERR_CAPACITY):
            self._check(rc)
        return [(a.status, a.n_edges) for a in arr], stats.as_dict()

    gen_tnf_graph_batched = tnf_graph_batched

    def set_graph_capture(self, enable: bool):
        self._check(self.lib.mdet_ctx_set_graph_capture(self.h, 1 if enable else 0))

    def graph_replays(self) -> int:
        return int(self.lib.mdet_ctx_graph_replays(self.h))

    # ---- learned proposal -----------------------------------------------
    def set_learned(self, net: "Network | None", recall_target: float = 0.999, recall_rows: int = 2048,
                    segment: int = 0, order: int = 0, tau_quantile: float = 0.0):
        """Network used by mode="learned" graph calls; returns the report that
        those calls fill (recall estimate, fallback, tiles skipped, tau, phase
        times).  order 0: embedding-major contig order, order 1: size-major."""
        rep = LearnedReport()
        rep.recall_target = recall_target
        rep.recall_rows = recall_rows
        rep.segment = segment
        rep.order = order
        rep.tau_quantile = tau_quantile
        self._learned = (net, rep)  # the context keeps both pointers
        self._check(self.lib.mdet_ctx_set_learned(self.h, net.h if net else None, ctypes.byref(rep)))
        return rep

    # ---- reference-named aliases ----------------------------------------
    calc_tnf = tnf_count
    gen_tnf_graph = tnf_graph
    gen_tnf_graph_sample = ptnf_search
    max_prob_sample = max_prob


class Network:
    """The learned proposal's 136 -> 256 -> 128 -> 64 embedding network
    (mdet_mlp): parameters live on the context's device."""

    def __init__(self, ctx: Context, seed: int = 1):
        self.ctx = ctx
        self.lib = ctx.lib
        h = P()
        ctx._check(self.lib.mdet_mlp_create(ctx.h, seed, ctypes.byref(h)))
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            self.lib.mdet_mlp_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @staticmethod
    def param_count() -> int:
        return int(load_library().mdet_mlp_param_count())

    def get_params(self) -> np.ndarray:
        out = np.zeros(self.param_count(), np.float32)
        self.ctx._check(self.lib.mdet_mlp_get_params(self.ctx.h, self.h, _ptr(out), out.size))
        return out

    def set_params(self, params: np.ndarray):
        p = np.ascontiguousarray(params, dtype=np.float32)
        self.ctx._check(self.lib.mdet_mlp_set_params(self.ctx.h, self.h, _ptr(p), p.size))

    def embed_dev(self, d_tnf: int, n: int, d_out: int):
        self.ctx._check(self.lib.mdet_mlp_embed_dev(self.ctx.h, self.h, P(d_tnf), n, P(d_out)))

    def grad(self, x: np.ndarray, pairs: np.ndarray, labels: np.ndarray, m_pos: float, m_neg: float):
        """(loss, gradient) of the mean contrastive loss; x rows x 136,
        pairs (np x 2) indexing rows of x, labels (np,) in {0, 1}."""
        x = np.ascontiguousarray(x, dtype=np.float32)
        pr = np.ascontiguousarray(pairs, dtype=np.uint32)
        lab = np.ascontiguousarray(labels, dtype=np.float32)
        g = np.zeros(self.param_count(), np.float32)
        loss = D()
        self.ctx._check(self.lib.mdet_mlp_grad(self.ctx.h, self.h, _ptr(x), x.shape[0], _ptr(pr), _ptr(lab),
                                               lab.size, m_pos, m_neg, _ptr(g), ctypes.byref(loss)))
        return loss.value, g

    def train_dev(self, d_tnf: int, d_ls: int, n: int, **kw) -> dict:
        """Trains on a device-resident assembly; keyword arguments set
        TrainParams fields.  Returns the training report."""
        tp = TrainParams(pairs=4_000_000, candidate_fraction=0.5, label_cutoff=0.7, steps=3000, batch_pairs=8192,
                         lr=1e-3, m_pos=0.5, m_neg=3.0, tau_quantile=0.9995, seed=7)
        for k, v in kw.items():
            setattr(tp, k, v)
        rep = TrainReport()
        self.ctx._check(self.lib.mdet_mlp_train(self.ctx.h, self.h, P(d_tnf), P(d_ls), n, ctypes.byref(tp),
                                                ctypes.byref(rep)))
        return rep.as_dict()


def version() -> str:
    return load_library().mdet_version().decode()
