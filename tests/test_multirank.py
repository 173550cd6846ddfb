"""The N>1 host logic of bench.py on CPU: gloo ranks that all hold the same
assembly, timing reduced by max over ranks, and the row-shard partition
with the gather of the shards' edge lists (the one data-path exchange)."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, ws, port, q):
    import torch.distributed as dist

    sys.path.insert(0, ROOT)
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    import bench

    mx = bench.reduce_max(10.0 * (rank + 1), "cpu")
    q.put((rank, mx, bench.assembly_seed(rank)))
    dist.barrier()
    dist.destroy_process_group()


def test_two_ranks_max_and_same_assembly():
    mp = pytest.importorskip("torch.multiprocessing")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = [q.get(timeout=120) for _ in range(2)]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    out.sort()
    assert [o[1] for o in out] == [20.0, 20.0]
    assert out[0][2] == out[1][2] == 2  # every rank holds the workload's own assembly


def _shard_worker(rank, ws, port, q):
    import numpy as np
    import torch
    import torch.distributed as dist

    sys.path.insert(0, ROOT)
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    from mdet_gb300 import shard, synth
    from oracle import oracle

    a = synth.generate(seed=17, n=1300, genomes=20, max_len=80000, threads=2)
    _, tnf = oracle.tnf_count(a.data, a.seq_off, a.seq_len, threads=2)
    rows = shard.shard_rows(a.log_sizes, rank, ws)
    fr, to, st = oracle.graph_rows(tnf, a.log_sizes, 0.9, 30, rows, threads=2)
    (gf, gt, gs), counts = shard.gather_edges(torch.from_numpy(fr.astype(np.int64)),
                                              torch.from_numpy(to.astype(np.int64)), torch.from_numpy(st))
    q.put((rank, rows.tolist(), gf.numpy().tolist(), gt.numpy().tolist(), gs.numpy().tolist(), counts))
    dist.barrier()
    dist.destroy_process_group()


@pytest.mark.parametrize("ws", [2, 3])
def test_row_shards_gather_to_the_whole_graph(ws):
    """Each gloo rank takes its block of size-sorted rows (the library's
    partition), scores them with the oracle against all contigs, and the
    gathered edge lists equal the whole graph on every rank."""
    import numpy as np

    mp = pytest.importorskip("torch.multiprocessing")
    from mdet_gb300 import synth
    from oracle import oracle

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_shard_worker, args=(r, ws, port, q)) for r in range(ws)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=180) for _ in range(ws))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    rows = [r for o in out for r in o[1]]
    assert sorted(rows) == list(range(1300))  # every row in exactly one shard
    a = synth.generate(seed=17, n=1300, genomes=20, max_len=80000, threads=2)
    _, tnf = oracle.tnf_count(a.data, a.seq_off, a.seq_len, threads=2)
    fr, to, st = oracle.graph(tnf, a.log_sizes, 0.9, 30)
    want = dict(zip(zip(fr.tolist(), to.tolist()), st.tolist()))
    for o in out:  # the same gathered list on every rank
        got = dict(zip(zip(o[2], o[3]), o[4]))
        assert len(got) == len(o[2]) == sum(o[5])
        assert got == want
