"""FASTA reading with the reference reader's semantics (cuda/Cuda2.cu:1487-1572).

A '>' starts a record wherever it stands, except inside the name line of the
record before it (there it is part of the name): the record starts are the
first '>' of each line.  The name runs to the end of its line and is cut at
the first space.  The sequence view starts after the header's newline and
runs to the next '>' (or end of file), keeping its inner newlines, with one
trailing newline dropped.  The contig size is the view's length minus its
newlines.  Records with size >= min_contig are the "large" contigs that get
TNF rows, in file order; their log size is log10(min(size, 500000))
(cuda/Cuda2.cu:1531-1536).
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np


@dataclass
class Assembly:
    data: np.ndarray          # uint8 view of the whole file
    names: list               # large-contig names, file order
    seq_off: np.ndarray       # uint64 byte offset of each sequence view
    seq_len: np.ndarray       # uint64 view length (newlines included)
    sizes: np.ndarray         # uint64 bases (newlines excluded)
    log_sizes: np.ndarray     # float64 log10(min(size, 500000))


def parse_fasta_bytes(data: np.ndarray, min_contig: int = 2500) -> Assembly:
    data = np.ascontiguousarray(data, dtype=np.uint8)
    gt = np.flatnonzero(data == ord(">"))
    nl_cum = np.concatenate([[0], np.cumsum(data == ord("\n"), dtype=np.int64)])
    fsize = data.size
    names, offs, lens, sizes = [], [], [], []
    nl_pos = np.flatnonzero(data == ord("\n"))
    # keep the first '>' of each line: the previous '>' lies before the line's start
    if gt.size:
        k = np.searchsorted(nl_pos, gt) - 1
        line0 = np.where(k >= 0, nl_pos[np.maximum(k, 0)] if nl_pos.size else -1, -1)
        first = np.ones(gt.size, bool)
        first[1:] = gt[:-1] < line0[1:]
        gt = gt[first]
    for k, g in enumerate(gt):
        h = np.searchsorted(nl_pos, g + 1)
        if h >= nl_pos.size:
            break  # header without a newline: no sequence
        hdr_end = int(nl_pos[h])
        name = bytes(data[g + 1:hdr_end]).split(b" ")[0].decode(errors="replace")
        s0 = hdr_end + 1
        s1 = int(gt[k + 1]) if k + 1 < gt.size else fsize
        n_lines = int(nl_cum[s1] - nl_cum[s0])
        size = (s1 - s0) - n_lines
        view = s1 - s0
        if view > 0 and data[s1 - 1] == ord("\n"):
            view -= 1
        if size >= min_contig:
            names.append(name)
            offs.append(s0)
            lens.append(view)
            sizes.append(size)
    sizes_a = np.asarray(sizes, dtype=np.uint64)
    return Assembly(
        data=data,
        names=names,
        seq_off=np.asarray(offs, dtype=np.uint64),
        seq_len=np.asarray(lens, dtype=np.uint64),
        sizes=sizes_a,
        log_sizes=np.log10(np.minimum(sizes_a, 500000).astype(np.float64)),
    )


def read_fasta(path: str, min_contig: int = 2500) -> Assembly:
    if path.endswith(".gz"):
        import gzip

        with gzip.open(path, "rb") as f:
            raw = f.read()
    else:
        with open(path, "rb") as f:
            raw = f.read()
    return parse_fasta_bytes(np.frombuffer(raw, dtype=np.uint8), min_contig)
