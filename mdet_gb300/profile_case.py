"""One small invocation of a single stage, for profiler captures.

  python -m mdet_gb300.profile_case count --n 100000     K1 on ~0.85 GB of FASTA
  python -m mdet_gb300.profile_case graph --n 500000     pairwise stage (bf16 or plain)

The graph case frees the FASTA before the pairwise call so that only the
stage's own buffers (~1-2 GB) are resident when it runs.
"""
import argparse
import ctypes
import os
import sys

import numpy as np

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("stage", choices=["count", "graph"])
    ap.add_argument("--n", type=int, default=100000)
    ap.add_argument("--genomes", type=int, default=0)
    ap.add_argument("--mode", default="bf16")
    ap.add_argument("--cutoff", type=float, default=0.95)
    ap.add_argument("--repeat", type=int, default=1)
    args = ap.parse_args()
    import torch

    import mdet_gb300 as m
    from mdet_gb300 import synth

    G = args.genomes or max(10, args.n // 500)
    a = synth.generate(3, args.n, G)
    ctx = m.Context(0)
    dev = torch.device("cuda:0")
    nb = a.data.size
    d_bytes = torch.zeros(nb + 64, dtype=torch.uint8, device=dev)
    d_bytes[:nb].copy_(torch.from_numpy(a.data))
    d_off = torch.from_numpy(a.seq_off.astype(np.int64)).to(dev)
    d_len = torch.from_numpy(a.seq_len.astype(np.int64)).to(dev)
    d_cnt = torch.empty((args.n, 136), dtype=torch.int32, device=dev)
    d_tnf = torch.empty((args.n, 136), dtype=torch.float32, device=dev)
    reps = args.repeat if args.stage == "count" else 1
    for _ in range(reps):
        ctx.tnf_count_dev(d_bytes.data_ptr(), nb, d_off.data_ptr(), d_len.data_ptr(), args.n, d_cnt.data_ptr(),
                          d_tnf.data_ptr())
    torch.cuda.synchronize()
    if args.stage == "graph":
        del d_bytes, d_cnt
        torch.cuda.empty_cache()
        d_ls = torch.from_numpy(a.log_sizes).to(dev)
        cap = args.n * 200
        out = [torch.empty(cap, dtype=t, device=dev) for t in (torch.int64, torch.int64, torch.float64)]
        for _ in range(args.repeat):
            ne, st = ctx.tnf_graph_dev(d_tnf.data_ptr(), d_ls.data_ptr(), args.n, args.cutoff, 200, args.mode,
                                       out[0].data_ptr(), out[1].data_ptr(), out[2].data_ptr(), cap)
        print({"edges": ne, **{k: st[k] for k in ("n_candidates", "ms_filter", "ms_total")}})
    torch.cuda.synchronize()
    ctx.close()


if __name__ == "__main__":
    main()
