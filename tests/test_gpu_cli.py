"""The command-line drop-in on the GPU: the record split and counting of a
FASTA file on the device, the graph at a fixed pTNF, its TSV, TNF.bin and
label-propagation bins against the oracle (reader, TNF.cpp normalisation,
graph, binning)."""
import gzip
import os
import subprocess
import sys

import numpy as np
import pytest

sys.path.insert(0, os.path.dirname(__file__))
from gpu_util import compare_graph  # noqa: E402
from mdet_gb300.fasta import parse_fasta_bytes  # noqa: E402
from oracle import oracle  # noqa: E402

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CLI = os.path.join(ROOT, "mdet_gb300", "_lib", "mdet_tnf")


@pytest.mark.parametrize("mode", ["bf16", "plain"])
def test_cli_graph_and_tnf_bin(tmp_path, mode):
    raw = gzip.open(os.path.join(ROOT, "tests", "golden", "count_synth.fa.gz")).read()
    fa = tmp_path / "in.fa"
    fa.write_bytes(raw)
    out = tmp_path / "out"
    r = subprocess.run([CLI, "-i", str(fa), "-o", str(out), "--pTNF", "95", "--seed", "1", "--mode", mode],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    assert "# elapsed time (TNF_CAL)" in r.stdout or "TNF_CAL" in r.stdout
    data = np.frombuffer(raw, np.uint8)
    a = parse_fasta_bytes(data, 2500)
    counts, tnf = oracle.tnf_count(data, a.seq_off, a.seq_len)
    n = len(a.names)
    # TNF.bin: TNF.cpp's FP64 normalisation of the counts, row by row
    tb = np.fromfile(str(out) + ".TNF.bin", dtype=np.float64).reshape(-1, 136)
    assert tb.shape[0] == n
    assert np.array_equal(tb, oracle.normalize_f64(counts), equal_nan=True)
    # graph: names back to indices, then the parity rule of the library's tests
    idx = {nm: k for k, nm in enumerate(a.names)}
    fr, to, st = [], [], []
    for line in open(str(out) + ".tnf_graph.tsv"):
        i, j, s = line.rstrip("\n").split("\t")
        fr.append(idx[i])
        to.append(idx[j])
        st.append(float(s))
    assert len(fr) > 0
    compare_graph(np.array(fr), np.array(to), np.array(st), tnf, a.log_sizes, 0.95, 200)
    # bins: label propagation over the CLI's own graph (sSCR = sTNF, maxP 95, minS 60)
    want, _ = oracle.label_prop(np.array(fr, np.uint64), np.array(to, np.uint64), np.array(st), n, 0.95, 0.60)
    got = np.zeros(n, np.uint64)
    for line in open(str(out) + ".lp_bins.tsv"):
        name, b = line.rstrip("\n").split("\t")
        got[idx[name]] = int(b)
    assert np.array_equal(got, want)


def test_cli_rejects_duplicate_names(tmp_path):
    fa = tmp_path / "dup.fa"
    fa.write_bytes(b">a\n" + b"ACGT" * 800 + b"\n>a\n" + b"TTGCA" * 700 + b"\n")
    r = subprocess.run([CLI, "-i", str(fa), "-o", str(tmp_path / "o"), "--pTNF", "95"], capture_output=True, text=True,
                       timeout=120)
    assert r.returncode != 0 and "duplicated sequence ids" in r.stderr
