"""Serving workload: Poisson arrivals of sort requests of mixed sizes and key
types, driven through the server (gs_server_*) or through one plain sort
call per request, with submit -> completion latency per request.

The mix: sizes log-uniform in [2^10, 2^26] keys; key types 40% uint32,
30% uint64, 20% float32 (N(0,1), NaN-free), 10% (int64 key, uint32 value =
input index). Every request has its own seed. Inputs and outputs are
device-resident before the clock starts, as for a server that keeps its
clients' buffers in HBM.

Both arms see the same schedule. Latency is completion minus the scheduled
arrival, so a request that waits behind others (plain arm) or for a slot
(served arm) is charged for the wait.
"""
from __future__ import annotations

import threading
import time
from dataclasses import dataclass

import numpy as np

from . import capi, datagen

# (key dtype, value dtype or None, share)
MIX = [(np.uint32, None, 0.4), (np.uint64, None, 0.3), (np.float32, None, 0.2),
       (np.int64, np.uint32, 0.1)]


@dataclass
class RequestSpec:
    n: int
    key_dtype: type
    val_dtype: type | None
    seed: int


def request_mix(count: int, lo_log2: int = 10, hi_log2: int = 26, seed: int = 5) -> list[RequestSpec]:
    rng = np.random.default_rng(seed)
    sizes = np.exp2(rng.uniform(lo_log2, hi_log2, size=count)).astype(np.int64)
    shares = np.array([m[2] for m in MIX])
    kinds = rng.choice(len(MIX), size=count, p=shares / shares.sum())
    return [RequestSpec(int(max(1, s)), MIX[k][0], MIX[k][1], int(seed * 100003 + i))
            for i, (s, k) in enumerate(zip(sizes, kinds))]


def poisson_arrivals(count: int, rate_per_s: float, seed: int = 6) -> np.ndarray:
    """Arrival offsets (seconds from the start) of a Poisson process."""
    rng = np.random.default_rng(seed)
    return np.cumsum(rng.exponential(1.0 / rate_per_s, size=count))


def bytes_alg(spec: RequestSpec) -> int:
    """Algorithmic bytes of one radix-8 onesweep sort of the request: a
    histogram read plus P = key bits / 8 passes reading and writing keys
    (and values)."""
    k = np.dtype(spec.key_dtype).itemsize
    v = np.dtype(spec.val_dtype).itemsize if spec.val_dtype is not None else 0
    p = k
    return spec.n * (k * (2 * p + 1) + v * 2 * p)


class DeviceRequest:
    """A request's device buffers: input, output (and values)."""

    def __init__(self, spec: RequestSpec, device_index: int = 0):
        import torch
        self.spec = spec
        dist = "normal" if np.dtype(spec.key_dtype).kind == "f" else "uniform"
        self.keys = datagen.device(dist, spec.n, spec.key_dtype, seed=spec.seed,
                                   device_index=device_index)
        self.keys_out = torch.empty_like(self.keys)
        if spec.val_dtype is not None:
            self.vals = torch.arange(spec.n, dtype=torch.int32, device=self.keys.device)
            self.vals_out = torch.empty_like(self.vals)
        else:
            self.vals = self.vals_out = None
        # the server's streams do not wait for torch's stream
        torch.cuda.synchronize(self.keys.device)

    def submit(self, server: "capi.Server") -> int:
        return server.submit(self.keys, self.keys_out, self.vals, self.vals_out,
                             key_dtype=self.spec.key_dtype, val_dtype=self.spec.val_dtype)

    def sort_plain(self, ctx: "capi.Context") -> int:
        if self.vals is None:
            return ctx.sort_keys(self.keys, self.keys_out, dtype=self.spec.key_dtype,
                                 flags=capi.FLAG_SYNC)
        return ctx.sort_pairs(self.keys, self.vals, self.keys_out, self.vals_out,
                              key_dtype=self.spec.key_dtype, val_dtype=self.spec.val_dtype,
                              flags=capi.FLAG_SYNC)


def _wait_until(t_abs: float):
    while True:
        d = t_abs - time.perf_counter()
        if d <= 0:
            return
        time.sleep(d if d > 2e-4 else 0)


def _summary(lat_ms: list[float], keys: int, bytes_: int, wall_s: float) -> dict:
    a = np.sort(np.asarray(lat_ms))

    def pct(q):
        return float(a[min(len(a) - 1, max(0, int(np.ceil(q * len(a))) - 1))])

    return {"requests": len(a), "p50_ms": pct(0.50), "p99_ms": pct(0.99),
            "mean_ms": float(a.mean()), "max_ms": float(a[-1]),
            "gkeys_s": keys / wall_s / 1e9, "gbs_alg": bytes_ / wall_s / 1e9,
            "wall_s": wall_s}


def run_served(server: "capi.Server", reqs: list[DeviceRequest],
               arrivals: np.ndarray | None) -> dict:
    """Submit each request at its arrival (None: all at once) and wait for
    all. Latency = (submit call - scheduled arrival) + server's submit ->
    completion time."""
    ids = [0] * len(reqs)
    late = [0.0] * len(reqs)
    ready = threading.Semaphore(0)
    errors: list[BaseException] = []
    t0 = time.perf_counter() + 0.002

    def submitter():
        try:
            for i, r in enumerate(reqs):
                t_sched = t0 + (arrivals[i] if arrivals is not None else 0.0)
                _wait_until(t_sched)
                late[i] = time.perf_counter() - t_sched
                ids[i] = r.submit(server)
                ready.release()
        except BaseException as e:  # surfaced below
            errors.append(e)
            ready.release()

    th = threading.Thread(target=submitter)
    th.start()
    lat = []
    t_last = t0
    for i in range(len(reqs)):
        ready.acquire()
        if errors:
            break
        st, ms = server.poll(ids[i], wait=True)
        if st != capi.GS_OK:
            raise capi.GsError(st, f"served request {i} failed")
        lat.append(late[i] * 1e3 + ms)
        t_last = max(t_last, t0 + (arrivals[i] if arrivals is not None else 0.0) + lat[-1] / 1e3)
    th.join()
    if errors:
        raise errors[0]
    keys = sum(r.spec.n for r in reqs)
    return _summary(lat, keys, sum(bytes_alg(r.spec) for r in reqs), t_last - t0)


def run_plain(ctx: "capi.Context", reqs: list[DeviceRequest], arrivals: np.ndarray | None) -> dict:
    """One synchronous sort call per request in arrival order (the plain
    per-request form). Latency = completion - scheduled arrival."""
    t0 = time.perf_counter() + 0.002
    lat = []
    t_end = t0
    for i, r in enumerate(reqs):
        t_sched = t0 + (arrivals[i] if arrivals is not None else 0.0)
        _wait_until(t_sched)
        st = r.sort_plain(ctx)
        if st != capi.GS_OK:
            raise capi.GsError(st, ctx.last_error())
        t_end = time.perf_counter()
        lat.append((t_end - t_sched) * 1e3)
    keys = sum(r.spec.n for r in reqs)
    return _summary(lat, keys, sum(bytes_alg(r.spec) for r in reqs), t_end - t0)
