"""FASTA ingest on the GPU against the oracle's restatement of the reference
reader (every field, in file order) on the golden fixtures, synthetic
assemblies and hand-made edge cases; then counting straight from the
device-side index."""
import os

import numpy as np
import pytest

from mdet_gb300.fasta import parse_fasta_bytes
from oracle import oracle

pytestmark = pytest.mark.gpu
G = os.path.join(os.path.dirname(__file__), "golden")


def _check(ctx, data, min_contig):
    data = np.ascontiguousarray(data, np.uint8)
    off, ln, sz, ls, names, st = ctx.fasta_index(data, min_contig)
    so, sl, ssz, no, nl = oracle.fasta_index(data)
    keep = ssz >= min_contig
    assert st["n_records"] == so.size
    assert st["n_large"] == int(keep.sum())
    assert st["n_small"] == int(((ssz >= 1000) & ~keep).sum())
    assert np.array_equal(off, so[keep]) and np.array_equal(ln, sl[keep]) and np.array_equal(sz, ssz[keep])
    raw = data.tobytes()
    assert names == [raw[int(o):int(o) + int(n)].decode(errors="replace") for o, n in zip(no[keep], nl[keep])]
    # log10 on the device vs the host's libm: within an ulp
    ref_ls = np.log10(np.minimum(sz, 500000).astype(np.float64))
    assert np.allclose(ls, ref_ls, rtol=4e-16, atol=0)
    # the host reader of the package agrees too
    a = parse_fasta_bytes(data, min_contig)
    assert np.array_equal(a.seq_off, off) and np.array_equal(a.seq_len, ln) and a.names == names
    return st


@pytest.mark.parametrize("name", ["count_synth.fa.gz", "count_edge.fa"])
@pytest.mark.parametrize("min_contig", [0, 1500, 2500])
def test_golden_files(gpu_ctx, name, min_contig):
    import gzip

    p = os.path.join(G, name)
    raw = gzip.open(p).read() if name.endswith(".gz") else open(p, "rb").read()
    _check(gpu_ctx, np.frombuffer(raw, np.uint8), min_contig)


def test_synthetic_assembly(gpu_ctx):
    from mdet_gb300 import synth

    a = synth.generate(seed=99, n=30000, genomes=40, threads=8)
    st = _check(gpu_ctx, a.data, 2500)
    assert st["n_large"] == 30000


@pytest.mark.parametrize("case", [
    b"", b">", b">only-a-name", b"no record here\nACGT\n", b">a\n", b">a\n>b\n", b">>>\n>\n",
    b">a b>c\nACGT>x>y z\nAC\n>q\nGG", b"junk>h1\nAAA\n\n>h2>h3\nCC>\n>", b"xx\nyy>z\nA",
    b">a\r\nAC\r\nGT\r\n>b\nAC", b"\n\n>a\n" + b"ACGT" * 1000 + b"\n",
])
def test_edge_cases(gpu_ctx, case):
    _check(gpu_ctx, np.frombuffer(case, np.uint8), 0)


def test_random_layouts(gpu_ctx):
    """Random records: '>' inside sequences and names, long single-line
    sequences, blank lines, records split across every 16-byte offset."""
    rng = np.random.default_rng(3)
    parts = []
    for k in range(2000):
        name = b"c%d" % k + (b" desc" if k % 3 == 0 else b"") + (b">x" if k % 17 == 0 else b"")
        L = int(rng.integers(0, 3000 if k % 50 else 70000))
        s = rng.choice(np.frombuffer(b"ACGTN\n", np.uint8), L, p=[.24, .24, .24, .24, .02, .02]).tobytes()
        if k % 29 == 0:
            s = s[:L // 2] + b">" + s[L // 2:]  # a record starting inside a line
        parts.append(b">" + name + b"\n" + s + (b"\n" if k % 5 else b""))
        parts.append(b"\n" * int(rng.integers(0, 2)))
    data = np.frombuffer(b"".join(parts), np.uint8)
    for shift in (0, 5):  # the buffer's first byte at another offset of its 16-byte chunk
        _check(gpu_ctx, np.concatenate([np.frombuffer(b"\n" * shift, np.uint8), data]), 500)


def test_capacity_and_device_path(gpu_ctx):
    torch = pytest.importorskip("torch")
    from mdet_gb300 import MdetError

    raw = open(os.path.join(G, "count_edge.fa"), "rb").read()
    data = np.frombuffer(raw, np.uint8)
    _, _, sz, _, _, st = gpu_ctx.fasta_index(data, 0)
    with pytest.raises(MdetError):
        gpu_ctx.fasta_index(data, 0, capacity=max(1, st["n_large"] - 1))
    # device form, then counting from the device-side views
    dev = torch.device("cuda:0")
    buf = torch.zeros(data.size + 64, dtype=torch.uint8, device=dev)
    buf[:data.size] = torch.from_numpy(data.copy()).to(dev)
    n = st["n_large"]
    d_off = torch.empty(n, dtype=torch.int64, device=dev)
    d_len = torch.empty(n, dtype=torch.int64, device=dev)
    st2 = gpu_ctx.fasta_index_dev(buf.data_ptr(), data.size, 0, n, d_off.data_ptr(), d_len.data_ptr())
    assert st2["n_large"] == n
    d_cnt = torch.empty((n, 136), dtype=torch.int32, device=dev)
    d_tnf = torch.empty((n, 136), dtype=torch.float32, device=dev)
    gpu_ctx.tnf_count_dev(buf.data_ptr(), data.size, d_off.data_ptr(), d_len.data_ptr(), n, d_cnt.data_ptr(),
                          d_tnf.data_ptr())
    a = parse_fasta_bytes(data, 0)
    oc, _ = oracle.tnf_count(data, a.seq_off, a.seq_len)
    assert np.array_equal(d_cnt.cpu().numpy().view(np.uint32), oc)
    with pytest.raises(MdetError):  # unaligned device buffer
        gpu_ctx.fasta_index_dev(buf.data_ptr() + 1, data.size - 1, 0, n, d_off.data_ptr(), d_len.data_ptr())


@pytest.mark.parametrize("name,min_contig", [("count_synth.fa.gz", 2500), ("count_edge.fa", 0)])
def test_count_from_fasta_bytes(gpu_ctx, name, min_contig):
    """Record split + counting in one call equals the oracle's count of the
    reference reader's views."""
    import gzip

    p = os.path.join(G, name)
    raw = gzip.open(p).read() if name.endswith(".gz") else open(p, "rb").read()
    data = np.frombuffer(raw, np.uint8)
    off, ln, ls, counts, tnf, st = gpu_ctx.tnf_count_fasta(data, min_contig)
    a = parse_fasta_bytes(data, min_contig)
    assert np.array_equal(off, a.seq_off) and np.array_equal(ln, a.seq_len)
    assert np.allclose(ls, a.log_sizes, rtol=4e-16, atol=0)
    oc, ot = oracle.tnf_count(data, a.seq_off, a.seq_len)
    assert np.array_equal(counts, oc)
    c2, t2 = gpu_ctx.tnf_count(data, a.seq_off, a.seq_len)
    assert np.array_equal(tnf.view(np.uint32), t2.view(np.uint32))
