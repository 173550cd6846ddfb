"""FASTA reader semantics of the reference (cuda/Cuda2.cu:1507-1544)."""
import numpy as np

from mdet_gb300.fasta import parse_fasta_bytes


def test_reader_rules():
    txt = b">a desc\nACGT\nAC\n>b\n" + b"A" * 10 + b"\n>c\nACG"
    p = parse_fasta_bytes(np.frombuffer(txt, np.uint8), min_contig=0)
    assert p.names == ["a", "b", "c"]
    # view keeps inner newlines and drops one trailing newline
    v0 = txt[p.seq_off[0]:p.seq_off[0] + p.seq_len[0]]
    assert v0 == b"ACGT\nAC"
    assert list(p.sizes) == [6, 10, 3]
    q = parse_fasta_bytes(np.frombuffer(txt, np.uint8), min_contig=7)
    assert q.names == ["b"]
    assert np.isclose(q.log_sizes[0], 1.0)


def test_log_size_clamp():
    txt = b">big\n" + b"A" * 600000 + b"\n"
    p = parse_fasta_bytes(np.frombuffer(txt, np.uint8))
    assert p.log_sizes[0] == np.log10(500000.0)
