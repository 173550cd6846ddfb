"""Seeded synthetic assemblies (ctypes wrapper of csrc/synth.c).

Stand-in for the real metagenome assemblies the reference is run on: G
order-3 Markov genomes, log-normal contig lengths clamped into
[min_len, max_len], 0.5% N, 60-column FASTA.  Same seed -> same bytes on any
machine and thread count.
"""
from __future__ import annotations

import ctypes
import os
from dataclasses import dataclass

import numpy as np

_LIB = os.path.join(os.path.dirname(os.path.abspath(__file__)), "_lib", "libmdet_synth.so")
_lib = None


def _load():
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB):
            raise OSError(f"{_LIB} not found: run python -m mdet_gb300.build")
        lib = ctypes.CDLL(_LIB)
        P = ctypes.c_void_p
        u64 = ctypes.c_uint64
        lib.mdet_synth_plan.restype = u64
        lib.mdet_synth_plan.argtypes = [u64, u64, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_double,
                                        ctypes.c_double, P, P, P]
        lib.mdet_synth_write.restype = ctypes.c_int
        lib.mdet_synth_write.argtypes = [u64, u64, ctypes.c_uint32, P, P, P, P, P, P, ctypes.c_int]
        _lib = lib
    return _lib


@dataclass
class SynthAssembly:
    data: np.ndarray      # uint8 FASTA bytes
    seq_off: np.ndarray   # uint64 sequence-view offsets
    seq_len: np.ndarray   # uint64 sequence-view lengths (newlines included)
    sizes: np.ndarray     # uint32 bases per contig
    genome: np.ndarray    # uint32 source genome of each contig
    log_sizes: np.ndarray # float64 log10(min(size, 500000))


def plan(seed: int, n: int, genomes: int, min_len=2500, max_len=500000, median=5000.0, sigma=1.0):
    lib = _load()
    L = np.zeros(n, np.uint32)
    g = np.zeros(n, np.uint32)
    ro = np.zeros(n, np.uint64)
    total = lib.mdet_synth_plan(seed, n, genomes, min_len, max_len, median, sigma, L.ctypes.data, g.ctypes.data,
                                ro.ctypes.data)
    return L, g, ro, int(total)


def generate(seed: int, n: int, genomes: int, min_len=2500, max_len=500000, median=5000.0, sigma=1.0,
             threads: int | None = None, out: np.ndarray | None = None) -> SynthAssembly:
    """Generate n contigs.  `out` may be a preallocated (e.g. pinned) uint8
    buffer of at least the planned size plus 16 bytes."""
    lib = _load()
    L, g, ro, total = plan(seed, n, genomes, min_len, max_len, median, sigma)
    if out is None:
        buf = np.zeros(total + 32, np.uint8)
    else:
        if out.size < total + 16:
            raise ValueError("output buffer too small")
        buf = out
    so = np.zeros(n, np.uint64)
    sl = np.zeros(n, np.uint64)
    th = threads or os.cpu_count() or 1
    rc = lib.mdet_synth_write(seed, n, genomes, L.ctypes.data, g.ctypes.data, ro.ctypes.data, buf.ctypes.data,
                              so.ctypes.data, sl.ctypes.data, th)
    if rc != 0:
        raise RuntimeError("synthetic generation failed")
    data = buf[:total]
    ls = np.log10(np.minimum(L, 500000).astype(np.float64))
    return SynthAssembly(data, so, sl, L, g, ls)


def abundance(genome: np.ndarray, nabd: int, seed: int, low_frac: float = 0.03):
    """Seeded coverage for an assembly, shaped like a depth table (mean and
    variance per contig and sample): each genome gets a mean depth per sample
    (log-normal around 10x), each contig that depth times log-normal noise
    (sigma 0.15) as its mean and mean * U(0.5, 2) as its variance.  A fraction
    low_frac of the contigs get depths in [0, 1) in every sample (no depth
    above 1, so a pair of two of them is not an edge).  Returns (abd, var),
    n x nabd float64 holding float32 values."""
    rng = np.random.default_rng(seed)
    genome = np.asarray(genome)
    n = genome.size
    G = int(genome.max()) + 1 if n else 1
    gd = rng.lognormal(np.log(10.0), 1.0, size=(G, nabd))
    abd = gd[genome] * rng.lognormal(0.0, 0.15, size=(n, nabd))
    low = rng.random(n) < low_frac
    abd[low] = rng.uniform(0.0, 1.0, size=(int(low.sum()), nabd))
    var = abd * rng.uniform(0.5, 2.0, size=(n, nabd))
    # the reference keeps depths in float matrices
    return abd.astype(np.float32).astype(np.float64), var.astype(np.float32).astype(np.float64)
