"""One small invocation of a single stage, for profiler captures.

  python -m mdet_gb300.profile_case count --n 100000     K1 on ~0.85 GB of FASTA
  python -m mdet_gb300.profile_case graph --n 500000     pairwise stage (bf16 or plain)
  python -m mdet_gb300.profile_case learned --n 500000   network trained on a second
                                                          assembly, then the learned graph
  python -m mdet_gb300.profile_case batch --count 64      many assemblies, n ~ logU(nmin, nmax):
                                                          one call per assembly vs one batched call
  python -m mdet_gb300.profile_case fasta --n 100000     FASTA record split of ~0.85 GB on the device
  python -m mdet_gb300.profile_case abd --n 100000       gated graph, then sTNF -> sSCR of its edges
                                                          with 10 samples of coverage

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
    ap.add_argument("stage", choices=["count", "graph", "learned", "batch", "fasta", "abd"])
    ap.add_argument("--samples", type=int, default=10)
    ap.add_argument("--count", type=int, default=64)
    ap.add_argument("--nmin", type=int, default=5000)
    ap.add_argument("--nmax", type=int, default=300000)
    ap.add_argument("--train-n", type=int, default=200000)
    ap.add_argument("--train-steps", type=int, default=3000)
    ap.add_argument("--segs", default="1024", help="comma-separated size-sorted run lengths to try")
    ap.add_argument("--n", type=int, default=100000)
    ap.add_argument("--genomes", type=int, default=0)
    ap.add_argument("--mode", default="bf16")
    ap.add_argument("--cutoff", type=float, default=0.95)
    ap.add_argument("--repeat", type=int, default=1)
    args = ap.parse_args()
    import torch

    import mdet_gb300 as m
    from mdet_gb300 import synth

    ctx = m.Context(0)
    dev = torch.device("cuda:0")
    if args.stage == "batch":
        return batch_case(args, m, synth, ctx, dev, torch)
    G = args.genomes or max(10, args.n // 500)
    a = synth.generate(3, args.n, G)
    nb = a.data.size
    d_bytes = torch.zeros(nb + 64, dtype=torch.uint8, device=dev)
    d_bytes[:nb].copy_(torch.from_numpy(a.data))
    d_off = torch.from_numpy(a.seq_off.astype(np.int64)).to(dev)
    d_len = torch.from_numpy(a.seq_len.astype(np.int64)).to(dev)
    d_cnt = torch.empty((args.n, 136), dtype=torch.int32, device=dev)
    d_tnf = torch.empty((args.n, 136), dtype=torch.float32, device=dev)
    if args.stage == "fasta":
        off = torch.empty(args.n, dtype=torch.int64, device=dev)
        ln = torch.empty(args.n, dtype=torch.int64, device=dev)
        for _ in range(args.repeat):
            st = ctx.fasta_index_dev(d_bytes.data_ptr(), nb, 2500, args.n, off.data_ptr(), ln.data_ptr())
        print(st)
        torch.cuda.synchronize()
        ctx.close()
        return
    reps = args.repeat if args.stage == "count" else 1
    for _ in range(reps):
        ctx.tnf_count_dev(d_bytes.data_ptr(), nb, d_off.data_ptr(), d_len.data_ptr(), args.n, d_cnt.data_ptr(),
                          d_tnf.data_ptr())
    torch.cuda.synchronize()
    if args.stage == "learned":
        import time

        del d_bytes, d_cnt
        torch.cuda.empty_cache()
        d_ls = torch.from_numpy(a.log_sizes).to(dev)
        # training assembly: other genomes (another seed)
        b = synth.generate(4, args.train_n, max(10, args.train_n // 500))
        tb = torch.zeros(b.data.size + 64, dtype=torch.uint8, device=dev)
        tb[:b.data.size].copy_(torch.from_numpy(b.data))
        t_off = torch.from_numpy(b.seq_off.astype(np.int64)).to(dev)
        t_len = torch.from_numpy(b.seq_len.astype(np.int64)).to(dev)
        t_cnt = torch.empty((args.train_n, 136), dtype=torch.int32, device=dev)
        t_tnf = torch.empty((args.train_n, 136), dtype=torch.float32, device=dev)
        ctx.tnf_count_dev(tb.data_ptr(), b.data.size, t_off.data_ptr(), t_len.data_ptr(), args.train_n,
                          t_cnt.data_ptr(), t_tnf.data_ptr())
        t_ls = torch.from_numpy(b.log_sizes).to(dev)
        torch.cuda.synchronize()
        del tb, t_cnt
        net = m.Network(ctx, seed=5)
        t0 = time.time()
        rep = net.train_dev(t_tnf.data_ptr(), t_ls.data_ptr(), args.train_n, steps=args.train_steps)
        print({"train_s": round(time.time() - t0, 2), **rep})
        cap = args.n * 200
        out = [torch.empty(cap, dtype=t, device=dev) for t in (torch.int64, torch.int64, torch.float64)]
        runs = [("bf16", 0)] + [("learned", int(x)) for x in args.segs.split(",") for _ in range(2)] + [("bf16", 0)]
        for mode, seg in runs:
            lr = ctx.set_learned(net, segment=seg)
            ne, st = ctx.tnf_graph_dev(d_tnf.data_ptr(), d_ls.data_ptr(), args.n, args.cutoff, 200, mode,
                                       out[0].data_ptr(), out[1].data_ptr(), out[2].data_ptr(), cap)
            extra = lr.as_dict() if mode == "learned" else {}
            print({"mode": mode, "edges": ne, **{k: round(v, 3) if isinstance(v, float) else v
                                                 for k, v in st.items()}, **extra})
    if args.stage == "abd":
        del d_bytes, d_cnt
        torch.cuda.empty_cache()
        d_ls = torch.from_numpy(a.log_sizes).to(dev)
        abd, var = synth.abundance(a.genome, args.samples, 7)
        ctx.set_abundance(abd, var)
        cap = args.n * 200
        out = [torch.empty(cap, dtype=t, device=dev) for t in (torch.int64, torch.int64, torch.float64)]
        ne, st = ctx.tnf_graph_dev(d_tnf.data_ptr(), d_ls.data_ptr(), args.n, args.cutoff, 200, args.mode,
                                   out[0].data_ptr(), out[1].data_ptr(), out[2].data_ptr(), cap)
        sscr = torch.empty(max(ne, 1), dtype=torch.float64, device=dev)
        for _ in range(args.repeat):
            ctx.edges_sscr_dev(out[0].data_ptr(), out[1].data_ptr(), out[2].data_ptr(), ne, sscr.data_ptr())
        print({"edges": ne, "graph_ms": st["ms_total"]})
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


def batch_case(args, m, synth, ctx, dev, torch):
    """Assemblies of n ~ logU(nmin, nmax) contigs, 20-800 genomes each (each
    one's TNF counted on the GPU, its FASTA freed), then the graphs: one call
    per assembly, and the batched call (sized run + recording, then replays)."""
    import time

    rng = np.random.default_rng(44)
    sizes = np.exp(rng.uniform(np.log(args.nmin), np.log(args.nmax), args.count)).astype(np.int64)
    genomes = np.clip((sizes / 400).astype(np.int64), 20, 800)
    tnfs, lss = [], []
    t0 = time.time()
    for k, (n, G) in enumerate(zip(sizes, genomes)):
        a = synth.generate(1000 + k, int(n), int(G))
        nb = a.data.size
        d_bytes = torch.zeros(nb + 64, dtype=torch.uint8, device=dev)
        d_bytes[:nb].copy_(torch.from_numpy(a.data))
        d_off = torch.from_numpy(a.seq_off.astype(np.int64)).to(dev)
        d_len = torch.from_numpy(a.seq_len.astype(np.int64)).to(dev)
        d_cnt = torch.empty((int(n), 136), dtype=torch.int32, device=dev)
        d_tnf = torch.empty((int(n), 136), dtype=torch.float32, device=dev)
        ctx.tnf_count_dev(d_bytes.data_ptr(), nb, d_off.data_ptr(), d_len.data_ptr(), int(n), d_cnt.data_ptr(),
                          d_tnf.data_ptr())
        tnfs.append(d_tnf)
        lss.append(torch.from_numpy(a.log_sizes).to(dev))
        del d_bytes, d_cnt
    torch.cuda.synchronize()
    print({"assemblies": args.count, "contigs": int(sizes.sum()), "sum_n2": float((sizes.astype(np.float64) ** 2).sum()),
           "prep_s": round(time.time() - t0, 1)})
    K, cut = 200, 0.9
    outs = [[torch.empty(int(n) * K, dtype=t, device=dev) for t in (torch.int64, torch.int64, torch.float64)]
            for n in sizes]
    items = [dict(d_tnf=t.data_ptr(), d_ls=l.data_ptr(), n=int(n), cutoff=cut, max_edges=K, d_from=o[0].data_ptr(),
                  d_to=o[1].data_ptr(), d_stnf=o[2].data_ptr(), capacity=int(n) * K)
             for t, l, n, o in zip(tnfs, lss, sizes, outs)]
    for rep in range(2):
        torch.cuda.synchronize()
        t0 = time.time()
        tot = cands = 0
        for t, l, n, o in zip(tnfs, lss, sizes, outs):
            ne, st = ctx.tnf_graph_dev(t.data_ptr(), l.data_ptr(), int(n), cut, K, "bf16", o[0].data_ptr(),
                                       o[1].data_ptr(), o[2].data_ptr(), int(n) * K)
            tot += ne
            cands += st["n_candidates"]
        torch.cuda.synchronize()
        print({"per_assembly_calls_s": round(time.time() - t0, 4), "edges": tot, "candidates": cands})
    for rep in range(5):
        torch.cuda.synchronize()
        t0 = time.time()
        res, st = ctx.tnf_graph_batched(items, mode="bf16")
        torch.cuda.synchronize()
        print({"batched_call_s": round(time.time() - t0, 4), "edges": sum(r[1] for r in res),
               "replays": ctx.graph_replays(), "gpu_launches": st["gpu_launches"], "tile": st["tile_m_n"],
               "candidates": st["n_candidates"]})
    ctx.close()


if __name__ == "__main__":
    main()
