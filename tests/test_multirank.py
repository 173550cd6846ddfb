"""The N>1 host logic of bench.py on CPU: two gloo ranks, each with its own
assembly seed, timing reduced by max over ranks (no data-path collective)."""
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


def test_two_ranks_max_and_independent_seeds():
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
    assert out[0][2] != out[1][2]
    assert out[0][2] == 2  # rank 0 runs the workload's own assembly
