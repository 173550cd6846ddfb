"""Host side of the row-sharded graph on several GPUs (one process per GPU).

The contigs in ascending log size (stable) are cut into `nshards`
contiguous blocks on 256-row boundaries; shard k emits the edges of its
block's rows (mdet_tnf_graph_shard).  The reference deals its row tiles to
devices the same way (cuda/Cuda2.cu:888-891).  TNF rows and log sizes are
replicated on every rank; the only exchange is the concatenation of the
per-shard edge lists, done here with torch.distributed (NCCL between GPUs,
gloo on the host).
"""
from __future__ import annotations

import numpy as np


def shard_bounds(n: int, shard: int, nshards: int):
    """[s0, s1): the sorted positions of shard `shard` (the library's rule)."""
    blocks = (n + 255) // 256
    return min(n, blocks * shard // nshards * 256), min(n, blocks * (shard + 1) // nshards * 256)


def shard_rows(log_sizes, shard: int, nshards: int) -> np.ndarray:
    """Original indices of the rows of shard `shard` of `nshards`, in size order."""
    ls = np.asarray(log_sizes, np.float64)
    order = np.argsort(ls, kind="stable")
    s0, s1 = shard_bounds(ls.size, shard, nshards)
    return order[s0:s1]


def gather_edges(from_, to, stnf, group=None):
    """Every rank's (from, to, sTNF) edge tensors concatenated in rank order,
    on every rank: the edge counts go first (all_gather), then the edges,
    padded to the largest count.  Works on CUDA tensors (NCCL) and host
    tensors (gloo)."""
    import torch
    import torch.distributed as dist

    ws = dist.get_world_size(group)
    dev = from_.device
    cnt = torch.tensor([from_.numel()], dtype=torch.int64, device=dev)
    counts = [torch.zeros_like(cnt) for _ in range(ws)]
    dist.all_gather(counts, cnt, group=group)
    counts = [int(c.item()) for c in counts]
    m = max(counts) if counts else 0
    out = []
    for t in (from_, to, stnf):
        pad = torch.zeros(m, dtype=t.dtype, device=dev)
        pad[:t.numel()] = t
        parts = [torch.zeros_like(pad) for _ in range(ws)]
        dist.all_gather(parts, pad, group=group)
        out.append(torch.cat([p[:c] for p, c in zip(parts, counts)]))
    return tuple(out), counts
