"""K1 on the GPU: bit-exact counts against the oracle (itself pinned to
TNF.bin of the reference's TNF.cpp) and normalised TNF within 1e-6."""
import os

import numpy as np
import pytest

from mdet_gb300.fasta import parse_fasta_bytes, read_fasta
from oracle import oracle

pytestmark = pytest.mark.gpu
G = os.path.join(os.path.dirname(__file__), "golden")


def _check(ctx, data, off, ln, ref64=None):
    counts, tnf = ctx.tnf_count(data, off, ln)
    oc, ot = oracle.tnf_count(data, off, ln)
    assert np.array_equal(counts, oc)
    # float(c / rsum): the GPU multiplies by 1/rsum, identical except at
    # double-rounding ties (allow a one-ulp difference on at most 1e-6 of entries)
    same = (tnf.view(np.uint32) == ot.view(np.uint32)) | (np.isnan(tnf) & np.isnan(ot))
    if not same.all():
        d = np.abs(tnf.view(np.int32).astype(np.int64) - ot.view(np.int32).astype(np.int64))[~same]
        assert d.max() <= 1 and (~same).mean() < 1e-6
    if ref64 is not None:
        ok = ~np.isnan(ref64)
        rel = np.abs(tnf[ok].astype(np.float64) - ref64[ok]) / np.where(ref64[ok] == 0, 1, ref64[ok])
        assert rel.max() < 1e-6
    return counts


@pytest.mark.parametrize("name", ["count_synth.fa.gz", "count_edge.fa"])
def test_golden_files(gpu_ctx, name):
    a = read_fasta(os.path.join(G, name))
    ref = np.load(os.path.join(G, name.split(".")[0] + "_tnf.npy"))
    _check(gpu_ctx, a.data, a.seq_off, a.seq_len, ref)


def test_config0_size(gpu_ctx):
    from mdet_gb300 import synth

    a = synth.generate(seed=1000000, n=20000, genomes=50, threads=8)
    _check(gpu_ctx, a.data, a.seq_off, a.seq_len)


def test_random_layouts(gpu_ctx):
    rng = np.random.default_rng(7)
    recs = []
    for k in range(300):
        L = int(rng.integers(0, 40000))
        s = rng.choice(np.frombuffer(b"ACGTacgtNNRY\r", np.uint8), L, p=[.2025, .2025, .2025, .2025, .04, .04, .04, .04, .01, .01,
                                                                        .005, .004, .001])
        w = int(rng.integers(1, 130))
        body = b"\n".join(s[i:i + w].tobytes() for i in range(0, L, w))
        if rng.random() < 0.1:
            body = body.replace(b"\n", b"\n\n", 3)
        recs.append(b">r%d\n" % k + body + (b"\n" if rng.random() < 0.9 else b""))
    data = np.frombuffer(b"".join(recs), np.uint8)
    p = parse_fasta_bytes(data, min_contig=0)
    _check(gpu_ctx, data, p.seq_off, p.seq_len)


def test_newline_runs_and_piece_edges(gpu_ctx):
    """Runs of many newlines (a lane's warm-up must walk back past them),
    contigs made of newlines only, and lengths on either side of the 64 KB
    piece size and of 16-byte chunk and lane-run boundaries."""
    rng = np.random.default_rng(11)
    bases = np.frombuffer(b"ACGTacgtN", np.uint8)
    recs = []
    for k, L in enumerate([3, 4, 5, 511, 512, 513, 515, 516, 16380, 16383, 16384, 16385, 16388, 32767, 32768, 32771,
                           49152, 65535, 65536, 65537, 65540, 131075, 200000]):
        s = bases[rng.integers(0, 9, L)].copy()
        nl = rng.random(L) < 0.05
        s[nl] = ord("\n")
        body = s.tobytes()
        if k % 3 == 0:  # stretches of 2-40 newlines
            parts = body.split(b"\n")
            body = b"".join(q + b"\n" * int(rng.integers(2, 41)) for q in parts)
        recs.append(b">r%d\n" % k + body + b"\n")
    recs.append(b">nl\n" + b"\n" * 40)
    data = np.frombuffer(b"".join(recs), np.uint8)
    p = parse_fasta_bytes(data, min_contig=0)
    _check(gpu_ctx, data, p.seq_off, p.seq_len)
    # the same bytes as one view each, newlines inside (no FASTA parsing)
    raw = np.frombuffer(b"".join(r.split(b"\n", 1)[1] for r in recs), np.uint8)
    lens = np.array([len(r.split(b"\n", 1)[1]) for r in recs], np.uint64)
    offs = np.concatenate([[0], np.cumsum(lens)[:-1]]).astype(np.uint64)
    _check(gpu_ctx, raw, offs, lens)


def test_host_path_chunked_equals_device(gpu_ctx):
    """Host buffers of >= 2 GB in file order take the chunked path (copy and
    count overlapped): its counts and TNF must equal the device-buffer path's."""
    torch = pytest.importorskip("torch")
    from mdet_gb300 import synth

    a = synth.generate(seed=31, n=270000, genomes=300)
    assert a.data.size >= (2 << 30)
    counts, tnf = gpu_ctx.tnf_count(a.data, a.seq_off, a.seq_len)
    dev = torch.device("cuda:0")
    nb = a.data.size
    d_bytes = torch.zeros(nb + 64, dtype=torch.uint8, device=dev)
    d_bytes[:nb].copy_(torch.from_numpy(a.data))
    d_off = torch.from_numpy(a.seq_off.astype(np.int64)).to(dev)
    d_len = torch.from_numpy(a.seq_len.astype(np.int64)).to(dev)
    n = a.seq_off.size
    d_cnt = torch.empty((n, 136), dtype=torch.int32, device=dev)
    d_tnf = torch.empty((n, 136), dtype=torch.float32, device=dev)
    gpu_ctx.tnf_count_dev(d_bytes.data_ptr(), nb, d_off.data_ptr(), d_len.data_ptr(), n, d_cnt.data_ptr(),
                          d_tnf.data_ptr())
    torch.cuda.synchronize()
    assert np.array_equal(counts, d_cnt.cpu().numpy().view(np.uint32))
    assert np.array_equal(tnf.view(np.uint32), d_tnf.cpu().numpy().view(np.uint32))
    # TNF rows only (no counts copied back), chunked path and single-copy path
    t_only = np.zeros_like(tnf)
    c_none, _ = gpu_ctx.tnf_count(a.data, a.seq_off, a.seq_len, out=(None, t_only))
    assert c_none is None and np.array_equal(t_only.view(np.uint32), tnf.view(np.uint32))
    t_small = np.zeros((1000, 136), np.float32)
    gpu_ctx.tnf_count(a.data, a.seq_off[:1000], a.seq_len[:1000], out=(None, t_small))
    assert np.array_equal(t_small.view(np.uint32), tnf[:1000].view(np.uint32))


def test_short_and_empty_contigs(gpu_ctx):
    txt = b">e\n>a\nA\n>b\nACG\n>c\nACGT\n>d\nAC\nGT\n>f\nNNNNNNNN\n"
    data = np.frombuffer(txt, np.uint8)
    p = parse_fasta_bytes(data, min_contig=0)
    counts, tnf = gpu_ctx.tnf_count(data, p.seq_off, p.seq_len)
    assert counts.sum(1).tolist() == [0, 0, 0, 1, 1, 0]
    assert np.isnan(tnf[0]).all() and np.isnan(tnf[5]).all()
    assert np.nansum(tnf[3]) == 1.0


def test_device_api_alignment_check(gpu_ctx):
    torch = pytest.importorskip("torch")
    from mdet_gb300 import MdetError

    a = read_fasta(os.path.join(G, "count_edge.fa"))
    n = a.seq_off.size
    buf = torch.zeros(a.data.size + 64, dtype=torch.uint8, device="cuda")
    buf[:a.data.size] = torch.from_numpy(a.data.copy()).cuda()
    off = torch.from_numpy(a.seq_off.astype(np.int64)).cuda()
    ln = torch.from_numpy(a.seq_len.astype(np.int64)).cuda()
    cnt = torch.zeros((n, 136), dtype=torch.int32, device="cuda")
    tnf = torch.zeros((n, 136), dtype=torch.float32, device="cuda")
    gpu_ctx.tnf_count_dev(buf.data_ptr(), a.data.size, off.data_ptr(), ln.data_ptr(), n, cnt.data_ptr(),
                          tnf.data_ptr())
    oc, _ = oracle.tnf_count(a.data, a.seq_off, a.seq_len)
    assert np.array_equal(cnt.cpu().numpy().view(np.uint32), oc)
    with pytest.raises(MdetError):
        gpu_ctx.tnf_count_dev(buf.data_ptr() + 3, a.data.size, off.data_ptr(), ln.data_ptr(), n, cnt.data_ptr(),
                              tnf.data_ptr())


def test_device_api_rejects_views_outside_buffer(gpu_ctx):
    """mdet_tnf_count_dev checks every view against nbytes on the device (from
    a 64-bit piece total) before it sizes anything from the lengths; garbage
    lengths are an error, and the context counts correctly afterwards."""
    torch = pytest.importorskip("torch")
    from mdet_gb300 import MdetError
    from mdet_gb300 import tnf as T

    a = read_fasta(os.path.join(G, "count_edge.fa"))
    n = a.seq_off.size
    buf = torch.zeros(a.data.size + 64, dtype=torch.uint8, device="cuda")
    buf[:a.data.size] = torch.from_numpy(a.data.copy()).cuda()
    cnt = torch.zeros((n, 136), dtype=torch.int32, device="cuda")
    tnf = torch.zeros((n, 136), dtype=torch.float32, device="cuda")
    for bad_len in (a.data.size + 1, 1 << 40, -3):
        ln_h = a.seq_len.astype(np.int64)
        ln_h[n // 2] = bad_len
        off = torch.from_numpy(a.seq_off.astype(np.int64)).cuda()
        ln = torch.from_numpy(ln_h).cuda()
        with pytest.raises(MdetError) as e:
            gpu_ctx.tnf_count_dev(buf.data_ptr(), a.data.size, off.data_ptr(), ln.data_ptr(), n, cnt.data_ptr(),
                                  tnf.data_ptr())
        assert e.value.code == T.ERR_INVALID
    off = torch.from_numpy(a.seq_off.astype(np.int64)).cuda()
    ln = torch.from_numpy(a.seq_len.astype(np.int64)).cuda()
    gpu_ctx.tnf_count_dev(buf.data_ptr(), a.data.size, off.data_ptr(), ln.data_ptr(), n, cnt.data_ptr(),
                          tnf.data_ptr())
    oc, _ = oracle.tnf_count(a.data, a.seq_off, a.seq_len)
    assert np.array_equal(cnt.cpu().numpy().view(np.uint32), oc)
