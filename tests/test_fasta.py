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


def test_gt_inside_name_lines_and_sequences():
    """'>' inside a name line is part of the name; inside a sequence line it
    starts a record (the first '>' of each line starts one)."""
    txt = b"junk>h1 x\nAAA\n\n>h2>h3\nCC>n4>n5 y\nGG\n>"
    p = parse_fasta_bytes(np.frombuffer(txt, np.uint8), min_contig=0)
    assert p.names == ["h1", "h2>h3", "n4>n5"]
    assert list(p.sizes) == [3, 2, 2]


def test_reader_matches_oracle_restatement():
    import os
    import gzip

    from oracle import oracle

    g = os.path.join(os.path.dirname(__file__), "golden")
    cases = [gzip.open(os.path.join(g, "count_synth.fa.gz")).read(), open(os.path.join(g, "count_edge.fa"), "rb").read(),
             b">a b>c\nACGT>x>y z\nAC\n>q\nGG", b">>>\n>\n", b"xx\nyy>z\nA", b">only", b""]
    for raw in cases:
        d = np.frombuffer(raw, np.uint8)
        so, sl, sz, no, nl = oracle.fasta_index(d)
        p = parse_fasta_bytes(d, min_contig=0)
        assert np.array_equal(p.seq_off, so) and np.array_equal(p.seq_len, sl) and np.array_equal(p.sizes, sz)
        assert p.names == [raw[int(o):int(o) + int(n)].decode(errors="replace") for o, n in zip(no, nl)]
