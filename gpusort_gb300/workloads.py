"""Profiling helper (not part of the sort API): single runs of each sort path
on synthetic uniform keys, so that a profiler sees only the kernels one path
launches. The ncu summaries of the kernels are made with it:

    python -m gpusort_gb300.workloads {radix,pairs,hyk,sample,segmented,gather,host}
        [--log2n N] [--runs R] [--shape S]

* radix      - gs_sort_keys, onesweep radix (upsweep, plan, passes)
* pairs      - gs_sort_pairs, uint64 Zipf(1.1) keys with a uint32 index
               payload, stable (8 key-and-value passes)
* hyk        - GS_ALGO_HYK, p=4, k=4 (partition sorts, merge-path merges)
* sample     - GS_ALGO_SAMPLE, p=64, oversample 32 (sample, bucket
               histogram, bucket scatter pass, per-bucket batched sort)
* segmented  - a planned batched sort of segments with log-uniform lengths
               (group sort, per-segment histograms, segmented passes)
* gather     - gs_gather of 8-byte elements by a random permutation
* host       - gs_sort_keys with pinned host buffers (GS_FLAG_HOST): the
               upsweep reads across the CPU-GPU link; from 2^25 keys the
               sort runs in bucket groups copied out while the next sorts,
               from 2^28 keys the input is split chunk by chunk as it
               arrives

Each run is synchronous and checked for GS_OK; `--runs` (default 2) lets a
profiler skip the first run's launches. `--shape` selects the pass kernel's
tile shape (gs_pass_shape_info) instead of the default by size.
"""
from __future__ import annotations

import argparse

import numpy as np

from . import capi, datagen


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("path", choices=["radix", "pairs", "hyk", "sample", "segmented", "gather",
                                     "host"])
    ap.add_argument("--log2n", type=int, default=26)
    ap.add_argument("--runs", type=int, default=2)
    ap.add_argument("--shape", type=int, default=-1)
    args = ap.parse_args(argv)
    import torch
    ctx = capi.Context(0)
    ctx.set_stream(torch.cuda.current_stream().cuda_stream)
    if args.shape >= 0:
        ctx.debug_set(capi.DEBUG_PASS_SHAPE, args.shape)
    n = 1 << args.log2n
    a = datagen.device("uniform", n, np.uint32, seed=1)
    o = torch.empty_like(a)

    def ok(st):
        if st != capi.GS_OK:
            raise capi.GsError(st, ctx.last_error())

    sync = capi.FLAG_SYNC
    if args.path == "pairs":
        k = datagen.device("zipf", n, np.uint64, seed=3)
        v = torch.arange(n, dtype=torch.int32, device=k.device)
        ko, vo = torch.empty_like(k), torch.empty_like(v)
        torch.cuda.synchronize()
        for _ in range(args.runs):
            ok(ctx.sort_pairs(k, v, ko, vo, key_dtype=np.uint64, val_dtype=np.uint32, stable=True,
                              flags=sync))
    for _ in range(args.runs):
        if args.path == "radix":
            ok(ctx.sort_keys(a, o, dtype=np.uint32, flags=sync))
        elif args.path == "hyk":
            ok(ctx.sort_keys(a, o, dtype=np.uint32, algo=capi.ALGO_HYK, partitions=4, k_way=4,
                             flags=sync))
        elif args.path == "sample":
            ok(ctx.sort_keys(a, o, dtype=np.uint32, algo=capi.ALGO_SAMPLE, partitions=64,
                             oversample=32, flags=sync))
    if args.path == "segmented":
        off = datagen.segment_offsets(max(1, n // 11000), 16, 1 << 22, total=n, seed=8)
        m = int(off[-1])
        s = datagen.device("uniform", m, np.uint32, seed=8)
        so = torch.empty_like(s)
        plan = ctx.segmented_plan(np.uint32, m, off)
        try:
            for _ in range(args.runs):
                ok(ctx.segmented_run(plan, s, so))
            ok(ctx.status_synchronize())
        finally:
            ctx.segmented_destroy(plan)
    elif args.path == "gather":
        perm = torch.randperm(n, device="cuda", dtype=torch.int64)
        src = torch.empty(n, dtype=torch.int64, device="cuda").random_()
        dst = torch.empty_like(src)
        torch.cuda.synchronize()
        for _ in range(args.runs):
            ok(ctx.gather(src, dst, perm, 8, flags=sync))
    elif args.path == "host":
        h = torch.empty(n, dtype=torch.int32, pin_memory=True)
        h.copy_(a.cpu())
        ho = torch.empty(n, dtype=torch.int32, pin_memory=True)  # empty_like would not pin
        for _ in range(args.runs):
            ok(ctx.sort_keys(h, ho, dtype=np.uint32, flags=capi.FLAG_HOST))
    torch.cuda.synchronize()
    print(args.path, "ok", flush=True)


if __name__ == "__main__":
    main()
