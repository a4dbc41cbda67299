"""Autotuner: measure the engine's tunable choices on this GPU and cache them
in a JSON file that the engine reads (gs_ctx_load_tuning).

What is tuned, per key type, payload width and size:
* the pass kernel's tile shape (threads per CTA x items per thread; the
  engine has a fixed 8-bit digit, so digit width is not a free choice);
* the SampleSort bucket count (keys only), used when a call leaves
  gs_opts.partitions at 0.

The reference hard-codes its parameters (include/helpers/hyksort_helper.h:
343-344, include/helpers/samplesort_helper.h:429, src/cuda_utils.cu:515).

    python -m gpusort_gb300.autotune --out tuning.json [--quick]

Every candidate is timed with CUDA events on the context's stream over
uniform keys (the inputs are generated on the device), after warm-up; the
fastest wins. Each size measured covers the log2 sizes up to halfway to its
neighbours in the table.
"""
from __future__ import annotations

import argparse
import json
import os
import time
from pathlib import Path

import numpy as np

from . import capi, datagen

CASES = [("u32", None), ("i32", None), ("f32", None), ("u64", None), ("i64", None),
         ("f64", None), ("u32", "u32"), ("u64", "u32"), ("i64", "u32"), ("u64", "u64")]
NP = {"u32": np.uint32, "i32": np.int32, "f32": np.float32, "u64": np.uint64,
      "i64": np.int64, "f64": np.float64}
SAMPLE_PARTITIONS = (16, 32, 64, 128, 256)


def default_path() -> Path:
    env = os.environ.get("GPUSORT_GB300_TUNING")
    if env:
        return Path(env)
    return Path.home() / ".cache" / "gpusort_gb300" / "tuning.json"


def _time(fn, stream, reps: int) -> float:
    import torch
    fn()
    fn()
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(reps):
        fn()
    e1.record(stream)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / reps


def _ranges(log2ns: list[int]) -> list[tuple[int, int]]:
    """Cover 0..63 with one range per measured size, split halfway."""
    out = []
    for i, lg in enumerate(log2ns):
        lo = 0 if i == 0 else (log2ns[i - 1] + lg) // 2 + 1
        hi = 63 if i == len(log2ns) - 1 else (lg + log2ns[i + 1]) // 2
        out.append((lo, hi))
    return out


def tune(ctx: "capi.Context", cases=CASES, log2ns=(16, 20, 24, 27), reps: int = 5,
         partitions=SAMPLE_PARTITIONS) -> dict:
    """Measure every pass shape (and SampleSort bucket count for keys) for
    each case and size; returns the JSON document (not yet applied)."""
    import torch
    stream = torch.cuda.current_stream()
    ctx.set_stream(stream.cuda_stream)
    log2ns = sorted(log2ns)
    nshapes = capi.load().gs_pass_shape_count()
    entries, measured = [], []
    t_start = time.time()
    for kname, vname in cases:
        kdt = NP[kname]
        vb = 0 if vname is None else np.dtype(NP[vname]).itemsize
        shapes = capi.pass_shapes(np.dtype(kdt).itemsize, vb)
        for (lo, hi), lg in zip(_ranges(list(log2ns)), log2ns):
            n = 1 << lg
            dist = "normal" if np.dtype(kdt).kind == "f" else "uniform"
            keys = datagen.device(dist, n, kdt, seed=lg)
            kout = torch.empty_like(keys)
            vals = vout = None
            if vname is not None:
                tv = torch.int32 if vb == 4 else torch.int64
                vals = torch.arange(n, dtype=tv, device=keys.device)
                vout = torch.empty_like(vals)
            times = []
            for s in range(nshapes):
                ctx.debug_set(capi.DEBUG_PASS_SHAPE, s)
                if vname is None:
                    fn = lambda: ctx.sort_keys(keys, kout, dtype=kdt)  # noqa: E731
                else:
                    fn = lambda: ctx.sort_pairs(keys, vals, kout, vout, key_dtype=kdt,  # noqa: E731
                                                val_dtype=NP[vname], stable=True)
                times.append(_time(fn, stream, reps))
            ctx.debug_set(capi.DEBUG_PASS_SHAPE, 2**64 - 1)
            best = int(np.argmin(times))
            rec = {"key_dtype": kname, "val_bytes": vb, "log2n": lg,
                   "shape_ms": [round(t, 4) for t in times],
                   "shapes": [list(x) for x in shapes]}
            best_p = 0
            if vname is None and lg >= 12 and partitions:
                ptimes = []
                for p in partitions:
                    ptimes.append(_time(lambda: ctx.sort_keys(keys, kout, dtype=kdt,
                                                              algo=capi.ALGO_SAMPLE, partitions=p),
                                        stream, reps))
                best_p = int(partitions[int(np.argmin(ptimes))])
                rec["samplesort_partitions"] = list(partitions)
                rec["samplesort_ms"] = [round(t, 4) for t in ptimes]
            st = ctx.status_synchronize()
            if st != capi.GS_OK:
                raise capi.GsError(st, ctx.last_error())
            measured.append(rec)
            entries.append({"key_dtype": kname, "val_bytes": vb, "log2n_min": lo,
                            "log2n_max": hi, "pass_shape": best, "partitions": best_p,
                            "threads": shapes[best][0], "items_per_thread": shapes[best][1]})
            del keys, kout, vals, vout
        torch.cuda.empty_cache()
    props = torch.cuda.get_device_properties(ctx.device)
    return {"device": props.name, "sms": props.multi_processor_count,
            "digit_bits": 8, "seconds": round(time.time() - t_start, 1),
            "entries": entries, "measured": measured}


def save(doc: dict, path: str | Path) -> Path:
    path = Path(path)
    path.parent.mkdir(parents=True, exist_ok=True)
    path.write_text(json.dumps(doc, indent=1))
    return path


def apply(ctx: "capi.Context", path: str | Path | None = None):
    """Load a tuning file into a context (default: default_path())."""
    ctx.load_tuning(path or default_path())


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("--out", default=None)
    ap.add_argument("--device", type=int, default=0)
    ap.add_argument("--quick", action="store_true", help="u32/u64/pairs at 2^20 and 2^24 only")
    args = ap.parse_args(argv)
    import torch
    torch.cuda.set_device(args.device)
    ctx = capi.Context(args.device)
    if args.quick:
        doc = tune(ctx, cases=[("u32", None), ("u64", None), ("u64", "u32")], log2ns=(20, 24),
                   reps=3)
    else:
        doc = tune(ctx)
    path = save(doc, args.out or default_path())
    ctx.load_tuning(path)  # the engine accepts what was written
    print(json.dumps({"path": str(path), "entries": len(doc["entries"]),
                      "seconds": doc["seconds"]}))


if __name__ == "__main__":
    main()
