"""The allocation-free counting entry point (mdet_tnf_count_noalloc).

It serves callers that cannot allocate device memory (a host application
that owns a fixed device arena, or a pipeline where a cudaMalloc between
stages is not allowed).  This test calls it through the C ABI on device
buffers the test itself owns, twice in a row on different inputs, and checks
both results against the regular entry point (mdet_tnf_count_dev) with the
tolerance the other counting tests use: counts bit-exact, TNF equal bit for
bit (both run the same kernel).  Collected last, so a failure here leaves
every other test already run; it also passes alone in a fresh process.
"""
import os
import sys

import numpy as np
import pytest

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))

pytestmark = pytest.mark.gpu


def _device_inputs(torch, a):
    dev = torch.device("cuda:0")
    buf = torch.zeros(a.data.size + 64, dtype=torch.uint8, device=dev)
    buf[:a.data.size] = torch.from_numpy(a.data.copy()).to(dev)
    off = torch.from_numpy(a.seq_off.astype(np.int64)).to(dev)
    ln = torch.from_numpy(a.seq_len.astype(np.int64)).to(dev)
    return buf, off, ln


def test_noalloc_matches_regular_entry_point():
    torch = pytest.importorskip("torch")
    import mdet_gb300 as m
    from mdet_gb300 import synth
    from mdet_gb300 import tnf as T

    lib = T.load_library()
    ctx = m.Context(0)
    stream = torch.cuda.current_stream()
    # two different inputs: many short contigs, then fewer long multi-piece ones
    sets = [synth.generate(seed=71, n=3000, genomes=20, max_len=60000, threads=8),
            synth.generate(seed=72, n=700, genomes=7, min_len=2500, max_len=400000, median=60000.0, threads=8)]
    for a in sets:
        n = a.seq_off.size
        buf, off, ln = _device_inputs(torch, a)
        dev = buf.device
        c0 = torch.zeros((n, 136), dtype=torch.int32, device=dev)
        t0 = torch.zeros((n, 136), dtype=torch.float32, device=dev)
        ctx.tnf_count_dev(buf.data_ptr(), a.data.size, off.data_ptr(), ln.data_ptr(), n, c0.data_ptr(),
                          t0.data_ptr())
        c1 = torch.full((n, 136), 7, dtype=torch.int32, device=dev)  # garbage the call must overwrite
        t1 = torch.full((n, 136), 3.0, dtype=torch.float32, device=dev)
        rc = lib.mdet_tnf_count_noalloc(buf.data_ptr(), a.data.size, off.data_ptr(), ln.data_ptr(), n, c1.data_ptr(),
                                        t1.data_ptr(), stream.cuda_stream)
        assert rc == T.OK
        torch.cuda.synchronize()
        assert torch.equal(c0, c1)
        assert torch.equal(t0.view(torch.int32), t1.view(torch.int32))
    ctx.close()


def test_noalloc_rejects_oversized_input():
    torch = pytest.importorskip("torch")
    from mdet_gb300 import tnf as T

    lib = T.load_library()
    dev = torch.device("cuda:0")
    x = torch.zeros(64, dtype=torch.uint8, device=dev)
    big = 8193
    rc = lib.mdet_tnf_count_noalloc(x.data_ptr(), 16, x.data_ptr(), x.data_ptr(), big, x.data_ptr(), x.data_ptr(),
                                    None)
    assert rc == T.ERR_CAPACITY
    rc = lib.mdet_tnf_count_noalloc(x.data_ptr() + 1, 16, x.data_ptr(), x.data_ptr(), 1, x.data_ptr(), x.data_ptr(),
                                    None)
    assert rc == T.ERR_INVALID


def test_noalloc_rejects_bad_views_and_piece_overflow():
    """Views outside the byte buffer (a garbage or huge length included) and
    a piece total above the array's limit are rejected from the device-side
    64-bit check, before any piece entry is written into the shared array;
    a valid call afterwards still matches the regular entry point."""
    torch = pytest.importorskip("torch")
    import mdet_gb300 as m
    from mdet_gb300 import synth
    from mdet_gb300 import tnf as T

    lib = T.load_library()
    dev = torch.device("cuda:0")
    stream = torch.cuda.current_stream().cuda_stream
    nb = 1 << 20
    buf = torch.full((nb + 64,), ord("A"), dtype=torch.uint8, device=dev)
    out_c = torch.zeros((8192, 136), dtype=torch.int32, device=dev)
    out_t = torch.zeros((8192, 136), dtype=torch.float32, device=dev)

    def call(off, ln, nbytes=nb):
        o = torch.tensor(off, dtype=torch.int64, device=dev)
        ln_ = torch.tensor(ln, dtype=torch.int64, device=dev)
        return lib.mdet_tnf_count_noalloc(buf.data_ptr(), nbytes, o.data_ptr(), ln_.data_ptr(), len(off),
                                          out_c.data_ptr(), out_t.data_ptr(), stream)

    # 8192 views of the whole 1 MB buffer: 16 pieces each, 131,072 > 65,536
    assert call([0] * 8192, [nb] * 8192) == T.ERR_CAPACITY
    # a view that runs past the buffer, one with a huge length, one starting past it
    assert call([0, 10], [100, nb]) == T.ERR_INVALID
    assert call([0], [1 << 40]) == T.ERR_INVALID
    assert call([nb + 1], [0]) == T.ERR_INVALID
    # lengths that would wrap a 32-bit piece count
    assert call([0, 0, 0], [nb, -3, 2]) == T.ERR_INVALID  # -3: 2^64 - 3 as uint64
    # the shared array is still usable
    a = synth.generate(seed=73, n=500, genomes=5, max_len=200000, threads=8)
    n = a.seq_off.size
    b2, off, ln = _device_inputs(torch, a)
    c0 = torch.zeros((n, 136), dtype=torch.int32, device=dev)
    t0 = torch.zeros((n, 136), dtype=torch.float32, device=dev)
    with m.Context(0) as ctx:
        ctx.tnf_count_dev(b2.data_ptr(), a.data.size, off.data_ptr(), ln.data_ptr(), n, c0.data_ptr(), t0.data_ptr())
    rc = lib.mdet_tnf_count_noalloc(b2.data_ptr(), a.data.size, off.data_ptr(), ln.data_ptr(), n, out_c.data_ptr(),
                                    out_t.data_ptr(), stream)
    assert rc == T.OK
    torch.cuda.synchronize()
    assert torch.equal(c0, out_c[:n])
    assert torch.equal(t0.view(torch.int32), out_t[:n].view(torch.int32))
