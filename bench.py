#!/usr/bin/env python3
"""Benchmark of the GB300 sort engine (one JSON line on stdout).

Workload (the single-array sort the reference's HykSort/SampleSort entry
points perform): 2^30 uint32 keys, i.i.d. uniform over [0, 2^32), sorted
ascending, inputs resident in HBM. A step is one full sort of the array.

  value        Gkeys/s of the device-resident sort (CUDA events, K steps)
  e2e          Gkeys/s through the C ABI with pinned HOST buffers
               (gs_sort_keys + GS_FLAG_HOST: the input is read across the
               CPU-GPU link and split chunk by chunk as it arrives, and the
               sort runs in bucket groups copied out while the next sorts);
               the whole output is compared with the device sort's
  roofline     dominant kernel (one onesweep pass): algorithmic bytes of one
               launch (8 B per key: read + write of a 4-byte key) over its
               average duration measured live with CUDA events on the
               launching stream, against the measured HBM copy bandwidth
  sort_roofline  whole sort under the fixed byte model 36 B/key
               (histogram read + 4 passes of read+write) over the step time
  cpu_baseline the reference's CPU HykSort (k=4 over 4 thread-ranks, merge
               sort local sort) restated in oracle/, timed on a bounded
               sample of the same workload on the host cores
  secondary    the other single-GPU workloads, device-resident, CUDA events:
               2^29 float32 N(0,1) (radix, and the SampleSort shape with
               p=64, oversampling 32); 2^29 uint32 in the HykSort shape
               (p=4 partition sorts, merge-path merge tree); 2^29 uint64
               Zipf(1.1) keys with a
               uint32 index payload, stable; 100,000 uint32 segments of
               log-uniform length in [16, 2^22] scaled to ~2^30 keys, one
               planned batched sort replayed from a CUDA graph
  serving      Poisson arrivals of the serving mix (sizes log-uniform in
               [2^10, 2^26]; 40% u32, 30% u64, 20% f32, 10% i64+u32 pairs),
               120 GB admission budget: the server (gs_server_*) against one
               plain synchronous sort call per request. Both arms are warmed
               up over the whole request set; closed-loop capacity is the
               median of three runs; the Poisson sweep is anchored on the
               plain arm's capacity and runs past its saturation;
               `equal_p99` compares the two arms' throughput at the plain
               arm's p99 before saturation
  reference_gpu  the reference's GPU local sort (thrust::sort over the
               chunk, src/cuda_utils.cu:424, i.e. CUB's radix sort) on the
               same 2^30 keys, from the comparison-only baseline/ library
  checks       every full-size output is compared byte for byte with the
               CPU oracle on the host cores, outside the timed regions
               (--no-check skips that)

`--impl reference` runs only the reference's own CPU sort (its HykSort,
k=4 over 4 thread-ranks, built from its sources into oracle/_ref; the
oracle's restatement when that build is absent) and prints its own line.
With torchrun and N>1 every rank sorts its own array (replicas).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

B_ALG_PER_KEY_U32 = 36          # 4 * (2 * 4 + 1): histogram read + 4 passes
PASS_BYTES_PER_KEY_U32 = 8      # one pass reads and writes each 4-byte key
# DRAM bytes per key of one pass launch, from the ncu capture of a 2^26-key
# sort (dram__bytes_read.sum + dram__bytes_write.sum = 493.6 MB per launch,
# the mean of its four passes, profiles/pass_kernel_u32_2e26_full.md); traffic is per key
# (streaming reads and writes), so it scales to 2^30 by the key count.
PASS_TRAFFIC_PER_KEY_U32 = 493.6e6 / (1 << 26)
METRIC = "sort throughput (Gkeys/s)"
WORKLOAD = "single-array sort, 2^{} uint32 keys uniform over [0, 2^32), ascending"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gpusort", choices=["gpusort", "reference"])
    ap.add_argument("--log2n", type=int, default=30)
    ap.add_argument("--cpu-seconds", type=float, default=10.0,
                    help="bound on the CPU baseline's sampled work")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-secondary", action="store_true")
    ap.add_argument("--no-serving", action="store_true")
    ap.add_argument("--no-check", action="store_true",
                    help="skip the byte-exact oracle comparisons of full-size outputs")
    ap.add_argument("--no-ref-gpu", action="store_true",
                    help="skip the reference GPU (Thrust/CUB) comparison line")
    ap.add_argument("--serve-requests", type=int, default=400)
    ap.add_argument("--serve-slots", type=int, default=8)
    return ap.parse_args()


def peaks() -> dict:
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return {"hbm_gbs": float(d["hbm_gbs"]), "source": "measured"}
    return {"hbm_gbs": 6800.0, "source": "fallback"}


class ClockSampler:
    """nvidia-smi clocks and throttle reasons during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.path = Path(os.environ.get("TMPDIR", "/tmp")) / f"gs_clocks_{os.getpid()}.csv"

    def __enter__(self):
        try:
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "50"],
                stdout=self.fh, stderr=subprocess.DEVNULL)
            # nvidia-smi takes a while to start: wait (up to 1.5 s) for its
            # first sample, so that the timed region is sampled throughout.
            t_end = time.perf_counter() + 1.5
            while time.perf_counter() < t_end and self.proc.poll() is None:
                if self.path.stat().st_size > 0:
                    break
                time.sleep(0.01)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.fh.close()

    def summary(self) -> dict:
        if self.proc is None or not self.path.exists():
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sms, maxs, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.path.read_text().splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sms.append(float(f[1]))
                maxs.append(float(f[2]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        self.path.unlink(missing_ok=True)
        if not sms:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        return {"sm_mhz": statistics.median(sms), "sm_max_mhz": max(maxs),
                "samples": len(sms), "reasons": sorted(reasons)}


REF_DRIVER = ROOT / "oracle" / "_ref" / "ref_driver"


def _write_keys_file(path: Path, keys: np.ndarray):
    """The reference's per-rank file layout: int64 count, then the keys."""
    with open(path, "wb") as f:
        f.write(np.int64(keys.size).tobytes())
        keys.tofile(f)


def ref_driver_times(keys: np.ndarray, runs: int, threads_per_rank: int) -> list[float]:
    """Seconds of `runs` sorts of `keys` by the reference's OWN CPU HykSort
    (k=4 over 4 thread-ranks, OpenMP merge-sort local sort), built from its
    sources into oracle/_ref/ref_driver; each run sorts a fresh copy, timed
    between the ranks' barriers around the sort (I/O excluded)."""
    import tempfile
    with tempfile.TemporaryDirectory() as td:
        fin, fout = Path(td) / "in.dat", Path(td) / "out.dat"
        _write_keys_file(fin, keys)
        env = dict(os.environ, GS_REF_REPEAT=str(runs), OMP_NUM_THREADS=str(threads_per_rank))
        r = subprocess.run([str(REF_DRIVER), "hyk", "u32", "4", "4", str(threads_per_rank), "0",
                            str(fin), str(fout)], capture_output=True, text=True, env=env)
        if r.returncode != 0:
            raise RuntimeError(f"ref_driver failed: {r.stderr[-2000:]}")
        out = np.fromfile(fout, dtype=np.uint32, offset=8)
    if out.size != keys.size or not bool(np.all(out[1:] >= out[:-1])):
        raise RuntimeError("ref_driver output is not a sorted permutation")
    return [float(ln.split()[1]) for ln in r.stderr.splitlines() if ln.startswith("seconds ")]


def cpu_baseline(keys_sample: np.ndarray, budget_s: float, threads_total: int | None = None):
    """Time the reference's own CPU HykSort (k=4, 4 thread-ranks) on a
    sample: the oracle/_ref build when present ("reference"), else the
    oracle's restatement of it ("port")."""
    cores = os.cpu_count() or 1
    if threads_total is None:
        threads_total = cores
    per_rank = max(1, threads_total // 4)
    if REF_DRIVER.exists():
        first = ref_driver_times(keys_sample, 1, per_rank)[0]
        runs = int(max(1, min(30, budget_s / max(first, 1e-3))))
        times = ref_driver_times(keys_sample, runs, per_rank)
        t = statistics.median(times)
        return {"value": keys_sample.size / t / 1e9, "unit": "Gkeys/s", "cores": per_rank * 4,
                "kind": "reference", "sample": f"{keys_sample.size} uint32 uniform keys "
                f"(the reference's HykSort, k=4 over 4 thread-ranks x {per_rank} OpenMP "
                f"threads, built from its sources; median of {len(times)})",
                "seconds": t, "sorted": True}
    from oracle import oracle
    times = []
    t_end = time.perf_counter() + budget_s
    while True:
        t0 = time.perf_counter()
        out = oracle.hyksort_cpu(keys_sample, p=4, k=4, threads=per_rank, seed=1)
        times.append(time.perf_counter() - t0)
        if time.perf_counter() > t_end or len(times) >= 30:
            break
    t = statistics.median(times)
    ok = bool(np.all(out[1:] >= out[:-1]))
    return {"value": keys_sample.size / t / 1e9, "unit": "Gkeys/s", "cores": per_rank * 4,
            "kind": "port", "sample": f"{keys_sample.size} uint32 uniform keys "
            f"(k=4 HykSort over 4 thread-ranks x {per_rank} threads, median of {len(times)})",
            "seconds": t, "sorted": ok}


def max_over_ranks(t_ms: float, world: int, device=None) -> float:
    """The slowest rank's time (replicas are timed together; one rank: t_ms)."""
    if world <= 1:
        return t_ms
    import torch
    import torch.distributed as dist
    tt = torch.tensor([t_ms], dtype=torch.float64, device=device)
    dist.all_reduce(tt, op=dist.ReduceOp.MAX)
    return float(tt.item())


def whole_job_gkeys(n_per_rank: int, world: int, t_ms: float) -> float:
    """Keys sorted by all replicas per second (Gkeys/s) over the slowest rank's time."""
    return world * n_per_rank / (t_ms * 1e-3) / 1e9


def time_steps(fn, stream, steps: int, warmup: int) -> float:
    """Average ms of fn() over `steps` runs after `warmup`, CUDA events on
    `stream` (the stream the engine launches on)."""
    import torch
    for _ in range(warmup):
        fn()
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(steps):
        fn()
    e1.record(stream)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / steps


def _unsigned_sorted(t, wide: bool) -> bool:
    import torch
    sign = torch.tensor(-2**63 if wide else -2**31, dtype=t.dtype, device=t.device)
    s = t ^ sign
    return bool((s[1:] >= s[:-1]).all())


def _host(t, dtype) -> np.ndarray:
    return t.cpu().numpy().view(np.dtype(dtype))


def _same_bytes(a: np.ndarray, b: np.ndarray) -> bool:
    return a.shape == b.shape and bool(np.array_equal(a.view(np.uint8), b.view(np.uint8)))


def secondary(ctx, stream, pk: dict, steps: int, warmup: int, check: bool) -> dict:
    """The other single-GPU workloads; with `check`, every output is compared
    byte for byte with the CPU oracle (outside the timed loops)."""
    import torch
    from gpusort_gb300 import capi, datagen
    oracle = None
    if check:
        from oracle import oracle
    out = {}
    hbm = pk["hbm_gbs"]

    def ok(st):
        if st != capi.GS_OK:
            raise RuntimeError(ctx.last_error())

    # float32 N(0,1), 2^29 keys: radix, and the SampleSort shape (p=64, x32)
    n = 1 << 29
    f = datagen.device("normal", n, np.float32, seed=2)
    fo = torch.empty_like(f)
    want = oracle.sort_keys(_host(f, np.float32)) if check else None
    for name, kw in (("radix", {}),
                     ("samplesort_p64_os32", {"algo": capi.ALGO_SAMPLE, "partitions": 64,
                                              "oversample": 32})):
        ms = time_steps(lambda: ok(ctx.sort_keys(f, fo, dtype=np.float32, **kw)), stream,
                        steps, warmup)
        ctx.synchronize()
        rec = {"gkeys_s": n / ms / 1e6, "ms": ms, "frac_36B": 36 * n / ms / 1e6 / hbm,
               "sorted": bool((fo[1:] >= fo[:-1]).all()),
               "sum_preserved": bool(torch.isclose(fo.double().sum(), f.double().sum()))}
        if check:
            rec["bit_exact"] = _same_bytes(_host(fo, np.float32), want)
        out[f"f32_normal_2^29_{name}"] = rec
    del f, fo, want

    # uint32 uniform, 2^29 keys: the HykSort shape (p=4 partition sorts,
    # then a tree of merge-path merges)
    u = datagen.device("uniform", n, np.uint32, seed=4)
    uo = torch.empty_like(u)
    ms = time_steps(lambda: ok(ctx.sort_keys(u, uo, dtype=np.uint32, algo=capi.ALGO_HYK,
                                             partitions=4, k_way=4)), stream, steps, warmup)
    ctx.synchronize()
    rec = {"gkeys_s": n / ms / 1e6, "ms": ms, "frac_36B": 36 * n / ms / 1e6 / hbm,
           "sorted": _unsigned_sorted(uo, False),
           "sum_preserved": int(uo.to(torch.int64).sum()) == int(u.to(torch.int64).sum())}
    if check:
        rec["bit_exact"] = _same_bytes(_host(uo, np.uint32), oracle.sort_keys(_host(u, np.uint32)))
    out["u32_uniform_2^29_hyksort_p4_k4"] = rec
    del u, uo

    # uint64 Zipf(1.1) keys + uint32 index, stable, 2^29 pairs
    k = datagen.device("zipf", n, np.uint64, seed=3)
    v = torch.arange(n, dtype=torch.int32, device=k.device)
    ko, vo = torch.empty_like(k), torch.empty_like(v)
    ms = time_steps(lambda: ok(ctx.sort_pairs(k, v, ko, vo, key_dtype=np.uint64,
                                              val_dtype=np.uint32, stable=True)),
                    stream, steps, warmup)
    ctx.synchronize()
    ties = ko[1:] == ko[:-1]
    rec = {"gkeys_s": n / ms / 1e6, "ms": ms, "frac_200B": 200 * n / ms / 1e6 / hbm,
           "sorted": _unsigned_sorted(ko, True),
           "ties_in_input_order": bool((vo[1:][ties] > vo[:-1][ties]).all()),
           "payload_permutation": int(vo.to(torch.int64).sum()) == n * (n - 1) // 2}
    del ties
    if check:
        wk, wv = oracle.sort_pairs(_host(k, np.uint64), _host(v, np.uint32), stable=True)
        rec["bit_exact"] = (_same_bytes(_host(ko, np.uint64), wk) and
                            _same_bytes(_host(vo, np.uint32), wv))
        del wk, wv
    out["u64_zipf_2^29_pairs_u32_stable"] = rec
    del k, v, ko, vo

    # batched segmented sort: 100,000 segments, ~2^30 keys, CUDA graph
    off = datagen.segment_offsets(100000, 16, 1 << 22, total=1 << 30, seed=8)
    ns = int(off[-1])
    a = datagen.device("uniform", ns, np.uint32, seed=8)
    ao = torch.empty_like(a)
    plan = ctx.segmented_plan(np.uint32, ns, off)
    side = torch.cuda.Stream()
    try:
        ctx.set_stream(side.cuda_stream)
        ok(ctx.segmented_run(plan, a, ao))  # eager run before capture
        torch.cuda.synchronize()
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g, stream=side):
            ok(ctx.segmented_run(plan, a, ao))
        with torch.cuda.stream(side):  # replay() launches on the current stream
            ms = time_steps(g.replay, side, steps, warmup)
        ok(ctx.status_synchronize())
    finally:
        ctx.set_stream(stream.cuda_stream)
        ctx.segmented_destroy(plan)
    s32 = ao ^ torch.tensor(-2**31, dtype=torch.int32, device=ao.device)
    inner = torch.ones(ns - 1, dtype=torch.bool, device=ao.device)
    bounds = torch.from_numpy(off[1:-1].astype(np.int64) - 1).to(ao.device)
    inner[bounds[(bounds >= 0) & (bounds < ns - 1)]] = False
    rec = {"keys": ns, "segments": 100000, "gkeys_s": ns / ms / 1e6, "ms": ms,
           "frac_36B": 36 * ns / ms / 1e6 / hbm, "graph": True,
           "segments_sorted": bool((s32[1:] >= s32[:-1])[inner].all()),
           "sum_preserved": int(ao.to(torch.int64).sum()) == int(a.to(torch.int64).sum())}
    del s32, inner
    if check:
        rec["bit_exact"] = _same_bytes(_host(ao, np.uint32),
                                       oracle.segmented_sort_keys(_host(a, np.uint32), off))
    out["segmented_100k_u32"] = rec
    del a, ao, g
    torch.cuda.empty_cache()
    return out


def reference_gpu(keys, stream, steps: int, warmup: int, check_against=None) -> dict:
    """The reference's GPU local sort on the same device-resident keys:
    thrust::sort under thrust::less, in place on a fresh copy each step (as
    src/cuda_utils.cu:424 calls it; Thrust allocates its temporary storage
    per call), and CUB's DeviceRadixSort::SortKeys with preallocated
    temporary storage (the same kernels without that allocation). Only the
    sort calls are inside the CUDA-event pairs."""
    import ctypes as C
    import torch
    from baseline import build as baseline_build
    lib = C.CDLL(str(baseline_build.build()))
    lib.ref_thrust_sort_u32.argtypes = [C.c_void_p, C.c_uint64, C.c_void_p]
    lib.ref_thrust_sort_u32.restype = C.c_int
    lib.ref_cub_temp_bytes_u32.argtypes = [C.c_uint64]
    lib.ref_cub_temp_bytes_u32.restype = C.c_size_t
    lib.ref_cub_sort_u32.argtypes = [C.c_void_p, C.c_void_p, C.c_uint64, C.c_void_p, C.c_size_t,
                                     C.c_void_p]
    lib.ref_cub_sort_u32.restype = C.c_int
    n = keys.numel()
    sh = stream.cuda_stream
    buf = torch.empty_like(keys)
    res = {}

    def timed(fn, before=None):
        ts = []
        for i in range(warmup + steps):
            if before is not None:
                before()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            rc = fn()
            e1.record(stream)
            if rc != 0:
                raise RuntimeError(f"reference GPU sort failed: {rc}")
            torch.cuda.synchronize()
            if i >= warmup:
                ts.append(e0.elapsed_time(e1))
        return sum(ts) / len(ts)

    ms = timed(lambda: lib.ref_thrust_sort_u32(buf.data_ptr(), n, sh),
               before=lambda: buf.copy_(keys))
    res["thrust_sort"] = {"ms": ms, "gkeys_s": n / ms / 1e6,
                          "call": "thrust::sort(thrust::cuda::par.on(stream), k, k + n, "
                                  "thrust::less<uint32_t>()), in place"}
    if check_against is not None:
        res["thrust_sort"]["same_as_engine"] = bool(torch.equal(buf, check_against))
    tb = int(lib.ref_cub_temp_bytes_u32(n))
    temp = torch.empty(tb, dtype=torch.uint8, device=keys.device)
    ms = timed(lambda: lib.ref_cub_sort_u32(keys.data_ptr(), buf.data_ptr(), n, temp.data_ptr(),
                                            tb, sh))
    res["cub_radix_sort"] = {"ms": ms, "gkeys_s": n / ms / 1e6, "temp_bytes": tb,
                             "call": "cub::DeviceRadixSort::SortKeys, preallocated temporary "
                                     "storage"}
    if check_against is not None:
        res["cub_radix_sort"]["same_as_engine"] = bool(torch.equal(buf, check_against))
    del buf, temp
    torch.cuda.empty_cache()
    return res


SERVE_LOADS = (0.3, 0.6, 0.9, 1.0, 1.1, 1.25, 1.5, 2.0, 3.0, 4.0)


def equal_p99(sweep: list[dict]) -> dict:
    """Both arms' throughput at the plain arm's p99 before it saturates.

    The latency bound L is the plain arm's p99 at the highest offered load
    it still delivers (achieved >= 95% of offered, and every lower load
    too); the plain arm's throughput there is compared with the most the
    served arm delivered at any load with p99 <= L."""
    plain_ok = None
    for pt in sweep:
        if pt["plain"]["gkeys_s"] >= 0.95 * pt["offered_gkeys_s"]:
            plain_ok = pt
        else:
            break
    if plain_ok is None:
        return {"bound_p99_ms": None}
    bound = plain_ok["plain"]["p99_ms"]
    best = None
    for pt in sweep:
        if pt["served"]["p99_ms"] <= bound and (best is None or
                                                pt["served"]["gkeys_s"] > best["served"]["gkeys_s"]):
            best = pt
    rec = {"bound_p99_ms": bound, "plain_load": plain_ok["load"],
           "plain_gkeys_s": plain_ok["plain"]["gkeys_s"],
           "plain_p99_ms": plain_ok["plain"]["p99_ms"]}
    if best is not None:
        rec.update({"served_load": best["load"], "served_gkeys_s": best["served"]["gkeys_s"],
                    "served_p99_ms": best["served"]["p99_ms"],
                    "throughput_ratio": best["served"]["gkeys_s"] / plain_ok["plain"]["gkeys_s"]})
    return rec


def serving_bench(ctx, count: int, slots: int) -> dict:
    import torch
    from gpusort_gb300 import capi, serving
    specs = serving.request_mix(count, seed=5)
    reqs = [serving.DeviceRequest(s) for s in specs]
    keys = sum(s.n for s in specs)
    res = {"requests": count, "keys": keys, "slots": slots,
           "hbm_budget_gb": 120, "latency": "scheduled arrival -> completion, ms"}
    with capi.Server(0, hbm_budget=120 << 30, max_request_keys=1 << 26, slots=slots) as srv:
        # Warm-up over the whole request set on both arms: the plain arm's
        # context scratch grows to the largest request, and every kernel
        # shape of the mix is loaded, before anything is timed.
        serving.run_plain(ctx, reqs, None)
        serving.run_served(srv, reqs, None)
        plain_runs = [serving.run_plain(ctx, reqs, None) for _ in range(3)]
        served_runs = [serving.run_served(srv, reqs, None) for _ in range(3)]
        plain = sorted(plain_runs, key=lambda r: r["gkeys_s"])[1]
        served = sorted(served_runs, key=lambda r: r["gkeys_s"])[1]
        res["closed_loop"] = {
            "plain": plain, "served": served,
            "plain_gkeys_s_runs": [r["gkeys_s"] for r in plain_runs],
            "served_gkeys_s_runs": [r["gkeys_s"] for r in served_runs],
            "throughput_ratio": served["gkeys_s"] / plain["gkeys_s"]}
        # Poisson sweep anchored on the plain arm's steady-state capacity
        # (median closed-loop run), past its saturation.
        rate = count / plain["wall_s"]
        sweep = []
        for m in SERVE_LOADS:
            arr = serving.poisson_arrivals(count, m * rate, seed=6)
            p = serving.run_plain(ctx, reqs, arr)
            q = serving.run_served(srv, reqs, arr)
            sweep.append({"load": m, "rate_req_s": m * rate,
                          "offered_gkeys_s": m * plain["gkeys_s"],
                          "plain": {k: p[k] for k in ("p50_ms", "p99_ms", "gkeys_s")},
                          "served": {k: q[k] for k in ("p50_ms", "p99_ms", "gkeys_s")}})
        res["poisson"] = sweep
        res["equal_p99"] = equal_p99(sweep)
        res["arena_peak_gb"] = srv.stats()["arena_peak"] / 1e9
    # served outputs equal the plain ones (last writer was the served arm)
    same = True
    for r in reqs[: min(count, 40)]:
        ko = r.keys_out.clone()
        vo = r.vals_out.clone() if r.vals is not None else None
        r.sort_plain(ctx)
        same &= bool(torch.equal(ko, r.keys_out))
        if vo is not None:
            same &= bool(torch.equal(vo, r.vals_out))
    res["served_equals_plain_first40"] = same
    del reqs
    torch.cuda.empty_cache()
    return res


REF_ARM_BUDGET_S = 150.0  # bound on the reference arm's whole --warmup + --steps run


def run_reference(args):
    """The reference's own CPU sort path on the host cores: its HykSort, k=4
    over 4 thread-ranks x cores/4 OpenMP threads, built from its sources
    (oracle/_ref/ref_driver); each step sorts a fresh copy of the sample.
    The sample is the whole 2^log2n workload unless the run would exceed
    REF_ARM_BUDGET_S, then the largest power of two that fits. Without
    that build, the oracle's restatement of the same algorithm is timed."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    cores = os.cpu_count() or 1
    per_rank = max(1, cores // 4)
    runs = args.warmup + args.steps
    full = 1 << args.log2n
    rng = np.random.default_rng(1)
    if REF_DRIVER.exists():
        kind = "reference"
        n = min(full, 1 << 26)
        keys = rng.integers(0, 1 << 32, size=full, dtype=np.uint32)
        est = ref_driver_times(keys[:n], 1, per_rank)[0]  # seconds per sort of n keys
        while n < full and est * 2.1 * runs <= REF_ARM_BUDGET_S:  # n log n growth
            n *= 2
            est *= 2.1
        times = ref_driver_times(np.ascontiguousarray(keys[:n]), runs, per_rank)[args.warmup:]
        what = ("the reference's own HykSort (include/hyksort.h entry, OpenMP merge-sort local "
                "sort), built from its sources against a thread-rank MPI shim")
    else:
        kind = "port"
        from oracle import oracle
        oracle.build()
        n = 1 << min(args.log2n, 26)
        keys = rng.integers(0, 1 << 32, size=n, dtype=np.uint32)
        times = []
        for i in range(runs):
            t0 = time.perf_counter()
            oracle.hyksort_cpu(keys, p=4, k=4, threads=per_rank, seed=1)
            if i >= args.warmup:
                times.append(time.perf_counter() - t0)
        what = "the reference's CPU HykSort restated in oracle/ (its own build is absent)"
    t = sum(times) / len(times)
    v = n / t / 1e9
    sample = (f"{n} uint32 uniform keys per step ({'the whole workload' if n == full else f'1/{full // n} of the 2^{args.log2n}-key workload'}); "
              f"{what}; k=4 over 4 thread-ranks x {per_rank} threads")
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": "Gkeys/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": t * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "u32", "data": "synthetic",
        "config": {"workload": WORKLOAD.format(args.log2n), "sample_keys": n,
                   "same_config": n == full, "ranks": 4, "k_way": 4,
                   "threads_per_rank": per_rank},
        "cpu_baseline": {"value": v, "unit": "Gkeys/s", "cores": per_rank * 4, "kind": kind,
                         "sample": sample},
        "e2e": {"value": v, "unit": "Gkeys/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
        return

    import torch
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")

    from gpusort_gb300 import _build, capi, datagen
    _build.build()
    ctx = capi.Context(local)
    stream = torch.cuda.current_stream()
    ctx.set_stream(stream.cuda_stream)

    n = 1 << args.log2n
    keys = datagen.device("uniform", n, np.uint32, seed=1 + rank)
    out = torch.empty_like(keys)

    def step():
        st = ctx.sort_keys(keys, out, dtype=np.uint32, n=n)
        if st != capi.GS_OK:
            raise RuntimeError(ctx.last_error())

    for _ in range(max(args.warmup, 3)):
        step()
    ctx.synchronize()
    # correctness of the measured configuration (size-independent checks)
    o = out
    sorted_ok = bool(((o.view(torch.int32).to(torch.int64) & 0xFFFFFFFF)[1:] >=
                      (o.view(torch.int32).to(torch.int64) & 0xFFFFFFFF)[:-1]).all())
    ksum = int((keys.view(torch.int32).to(torch.int64) & 0xFFFFFFFF).sum())
    osum = int((o.view(torch.int32).to(torch.int64) & 0xFFFFFFFF).sum())
    checks = {"sorted": sorted_ok, "sum_preserved": ksum == osum}
    if not args.no_check:
        # the whole output against the CPU oracle, byte for byte (untimed)
        from oracle import oracle
        checks["bit_exact"] = _same_bytes(_host(out, np.uint32),
                                          oracle.sort_keys(_host(keys, np.uint32)))

    def barrier():
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        barrier()
        ev0.record(stream)
        for _ in range(args.steps):
            step()
        ev1.record(stream)
        barrier()
    st = ctx.status_synchronize()
    if st != capi.GS_OK:
        raise RuntimeError(ctx.last_error())
    t_ms = max_over_ranks(ev0.elapsed_time(ev1) / args.steps, world, device="cuda")
    value = whole_job_gkeys(n, world, t_ms)

    # per-kernel times of the pipeline (events recorded by the engine on the
    # launching stream), a separate short loop
    ctx.set_timing(True)
    kt = []
    for _ in range(3):
        step()
        ctx.synchronize()
        kt.append(ctx.kernel_times())
    ctx.set_timing(False)
    ups = statistics.median(k[0] for k in kt)
    passes = [statistics.median(k[2 + q] for k in kt) for q in range(4)]
    pass_avg = sum(passes) / len(passes)
    pk = peaks()
    pass_alg = PASS_BYTES_PER_KEY_U32 * n
    achieved = pass_alg / (pass_avg * 1e-3) / 1e9
    sort_alg = B_ALG_PER_KEY_U32 * n
    sort_achieved = sort_alg / (t_ms * 1e-3) / 1e9

    # end to end through the C ABI with pinned host buffers
    e2e = None
    if not args.no_e2e:
        h_in = torch.empty(n, dtype=torch.int32, pin_memory=True)
        h_in.copy_(keys.cpu())
        h_out = torch.empty(n, dtype=torch.int32, pin_memory=True)
        es = []
        for i in range(2 + args.steps):
            t0 = time.perf_counter()
            stt = ctx.sort_keys(h_in, h_out, dtype=np.uint32, n=n, flags=capi.FLAG_HOST)
            dt = time.perf_counter() - t0
            if stt != capi.GS_OK:
                raise RuntimeError(ctx.last_error())
            if i >= 2:
                es.append(dt)
        e_t = statistics.median(es)
        e2e_ok = bool(torch.equal(h_out.cuda(), out))
        e2e = {"value": n / e_t / 1e9, "unit": "Gkeys/s", "h2d_bytes_per_step": 4 * n,
               "d2h_bytes_per_step": 4 * n, "ms_per_step": e_t * 1e3,
               "api": "gs_sort_keys(GS_FLAG_HOST), pinned host buffers", "matches_device": e2e_ok}
        del h_in, h_out

    ref_gpu = None
    if not args.no_ref_gpu:
        ref_gpu = reference_gpu(keys, stream, steps=5, warmup=2, check_against=out)

    cpu = None
    if rank == 0 and not args.no_cpu:
        sample = keys[: 1 << 26].cpu().numpy().view(np.uint32).copy()
        cpu = cpu_baseline(sample, args.cpu_seconds)
    del keys, out
    torch.cuda.empty_cache()
    sec = None
    if not args.no_secondary:
        sec = secondary(ctx, stream, pk, steps=5, warmup=3, check=not args.no_check)
    srv = None
    if not args.no_serving:
        srv = serving_bench(ctx, args.serve_requests, args.serve_slots)

    line = {
        "metric": METRIC, "value": value, "unit": "Gkeys/s", "n_gpus": world,
        "steps": args.steps, "warmup": max(args.warmup, 3), "ms_per_step": t_ms,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u32",
        "data": "synthetic",
        "config": {"workload": WORKLOAD.format(args.log2n), "n": n, "key": "uint32", "algo": "radix (onesweep LSD)",
                   "l2": "inputs 4 GiB > 129 MB L2, no flush needed",
                   "parallelism": f"replicas x{world}" if world > 1 else "single GPU"},
        "roofline": {"bound": "hbm", "kernel": "pass_kernel (one onesweep digit pass)",
                     "achieved": achieved, "peak": pk["hbm_gbs"], "unit": "GB/s",
                     "frac": achieved / pk["hbm_gbs"],
                     "traffic": PASS_TRAFFIC_PER_KEY_U32 * n,
                     "traffic_source": "ncu dram bytes of a 2^26-key pass, scaled by keys",
                     "peak_source": pk["source"], "bytes_per_launch": pass_alg,
                     "launch_ms": pass_avg},
        "sort_roofline": {"achieved": sort_achieved, "peak": pk["hbm_gbs"], "unit": "GB/s",
                          "frac": sort_achieved / pk["hbm_gbs"], "bytes_per_key": 36},
        "kernel_ms": {"upsweep": ups, "passes": passes},
        "e2e": e2e,
        "cpu_baseline": cpu,
        "clocks": clk.summary(),
        "gpu_launches": args.steps * 6,
        "checks": checks,
        "reference_gpu": ref_gpu,
        "secondary": sec,
        "serving": srv,
    }
    if rank == 0:
        print(json.dumps(line), flush=True)
    ctx.close()
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
