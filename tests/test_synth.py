"""Synthetic assemblies: deterministic, FASTA layout of the reference's
printFasta, sequence views as the reference's reader builds them."""
import numpy as np

from mdet_gb300 import synth
from mdet_gb300.fasta import parse_fasta_bytes


def test_deterministic_across_thread_counts():
    a = synth.generate(seed=5, n=300, genomes=7, threads=1)
    b = synth.generate(seed=5, n=300, genomes=7, threads=7)
    assert np.array_equal(a.data, b.data)
    c = synth.generate(seed=6, n=300, genomes=7, threads=3)
    assert not np.array_equal(a.data[:1000], c.data[:1000])


def test_layout_and_views():
    a = synth.generate(seed=9, n=200, genomes=5, threads=4)
    text = a.data.tobytes().decode()
    lines = text.split("\n")
    assert lines[0] == ">ctg0"
    assert all(len(l) <= 60 for l in lines if not l.startswith(">"))
    p = parse_fasta_bytes(a.data, min_contig=0)
    assert p.names == [f"ctg{k}" for k in range(200)]
    assert np.array_equal(p.seq_off, a.seq_off)
    assert np.array_equal(p.seq_len, a.seq_len)
    assert np.array_equal(p.sizes, a.sizes.astype(np.uint64))


def test_length_and_base_distribution():
    L, g, _, _ = synth.plan(seed=1, n=20000, genomes=50)
    assert L.min() == 2500 and L.max() <= 500000
    frac_min = (L == 2500).mean()
    assert 0.2 < frac_min < 0.3  # clamped left tail of lognormal(ln 5000, 1)
    assert 4500 < np.median(L) < 5600
    assert np.bincount(g, minlength=50).min() > 0
    a = synth.generate(seed=2, n=400, genomes=4, threads=4)
    seq = a.data[a.data != ord("\n")]
    seq = seq[seq != ord(">")]
    n_frac = (seq == ord("N")).mean()
    assert 0.003 < n_frac < 0.007
