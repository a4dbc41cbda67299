"""Seeded synthetic inputs for the sort workloads.

The reference generates per-rank data with non-reproducible shared-RNG
generators over [0, 2^31) (src/test/utils.h:425-608); the workloads here use
fixed seeds and the full key range instead:

* ``uniform``   - i.i.d. uniform bits of the key type (u32: [0, 2^32));
* ``normal``    - N(0, 1) floats, NaN-free, -0.0 replaced by +0.0;
* ``zipf``      - Zipf(s=1.1) over 2^20 distinct ranks, each rank mapped to a
                  64-bit value by an odd-multiplier bijection, so the
                  distinct keys spread over the whole range;
* ``sorted`` / ``reverse`` - uniform keys already in (reverse) order;
* ``equal``     - one value repeated;
* ``distinct8`` - 8 distinct values.

``host(...)`` returns a numpy array (small sizes, tests);
``device(...)`` returns a torch CUDA tensor holding the same kind of data
(large sizes, benchmarks; its bytes are not the host generator's).
"""
from __future__ import annotations

import numpy as np

ZIPF_S = 1.1
ZIPF_DISTINCT = 1 << 20
_MUL = 0x9E3779B97F4A7C15
_ADD = 0x632BE59BD9B4E019

INT_DTYPES = (np.uint32, np.int32, np.uint64, np.int64)
FLOAT_DTYPES = (np.float32, np.float64)


def _zipf_cdf() -> np.ndarray:
    r = np.arange(1, ZIPF_DISTINCT + 1, dtype=np.float64)
    w = r ** (-ZIPF_S)
    c = np.cumsum(w)
    return c / c[-1]


def _spread(rank_u64: np.ndarray) -> np.ndarray:
    with np.errstate(over="ignore"):
        return rank_u64 * np.uint64(_MUL) + np.uint64(_ADD)


def host(dist: str, n: int, dtype=np.uint32, seed: int = 0) -> np.ndarray:
    dtype = np.dtype(dtype)
    rng = np.random.default_rng(seed)
    if dist == "uniform" or dist in ("sorted", "reverse"):
        if dtype.kind == "f":
            a = rng.standard_normal(n).astype(dtype)
            a[a == 0] = 0
        else:
            bits = rng.integers(0, 2**64, size=n, dtype=np.uint64, endpoint=False)
            a = bits.view(np.int64).astype(np.int64).view(np.uint64)
            a = a.astype(np.dtype(f"u{dtype.itemsize}"), copy=False).view(dtype)
        if dist == "sorted":
            a = np.sort(a)
        elif dist == "reverse":
            a = np.sort(a)[::-1].copy()
        return a
    if dist == "normal":
        a = rng.standard_normal(n).astype(dtype)
        a[a == 0] = 0
        return a
    if dist == "zipf":
        u = rng.random(n)
        ranks = np.searchsorted(_zipf_cdf(), u, side="right").astype(np.uint64)
        v = _spread(ranks)
        if dtype.kind == "f":
            return (ranks.astype(np.float64) * 0.5 - 1000.0).astype(dtype)
        return v.astype(np.dtype(f"u{dtype.itemsize}"), copy=False).view(dtype)
    if dist == "equal":
        return np.full(n, host("uniform", 1, dtype, seed)[0], dtype=dtype)
    if dist == "distinct8":
        vals = host("uniform", 8, dtype, seed + 7919)
        return vals[rng.integers(0, 8, size=n)]
    raise ValueError(f"unknown distribution {dist}")


def device(dist: str, n: int, dtype=np.uint32, seed: int = 0, device_index: int = 0):
    """Same families as ``host`` generated on the GPU with torch. Returns a
    torch tensor whose storage dtype is int32/int64/float32/float64; the
    logical dtype is ``dtype`` (unsigned types are bit views)."""
    import torch

    dtype = np.dtype(dtype)
    dev = torch.device("cuda", device_index)
    g = torch.Generator(device=dev)
    g.manual_seed(seed)
    if dtype.kind == "f":
        tdt = torch.float32 if dtype.itemsize == 4 else torch.float64
        if dist in ("uniform", "normal", "sorted", "reverse"):
            a = torch.randn(n, generator=g, device=dev, dtype=torch.float64).to(tdt)
            a = torch.where(a == 0, torch.zeros_like(a), a)
        elif dist == "equal":
            a = torch.full((n,), 0.25, device=dev, dtype=tdt)
        elif dist == "distinct8":
            vals = torch.randn(8, generator=g, device=dev, dtype=tdt)
            a = vals[torch.randint(0, 8, (n,), generator=g, device=dev)]
        elif dist == "zipf":
            cdf = torch.from_numpy(_zipf_cdf()).to(dev)
            r = torch.searchsorted(cdf, torch.rand(n, generator=g, device=dev, dtype=torch.float64),
                                   right=True)
            a = (r.to(torch.float64) * 0.5 - 1000.0).to(tdt)
        else:
            raise ValueError(dist)
    else:
        wide = dtype.itemsize == 8
        tdt = torch.int64 if wide else torch.int32
        if dist in ("uniform", "sorted", "reverse"):
            lo = torch.empty(n, dtype=torch.int32, device=dev).random_(-2**31, 2**31, generator=g)
            if wide:
                hi = torch.empty(n, dtype=torch.int32, device=dev).random_(-2**31, 2**31,
                                                                           generator=g)
                a = (hi.to(torch.int64) << 32) | (lo.to(torch.int64) & 0xFFFFFFFF)
            else:
                a = lo
        elif dist == "equal":
            a = torch.full((n,), 123456789, device=dev, dtype=tdt)
        elif dist == "distinct8":
            vals = torch.empty(8, dtype=tdt, device=dev).random_(generator=g)
            a = vals[torch.randint(0, 8, (n,), generator=g, device=dev)]
        elif dist == "zipf":
            cdf = torch.from_numpy(_zipf_cdf()).to(dev)
            r = torch.searchsorted(cdf, torch.rand(n, generator=g, device=dev, dtype=torch.float64),
                                   right=True).to(torch.int64)
            mul = _MUL - (1 << 64)  # same bits as a signed int64
            add = _ADD
            a = r * mul + add  # wraps modulo 2^64
            if not wide:
                a = a.to(torch.int32)
        else:
            raise ValueError(dist)
        if dist in ("sorted", "reverse"):
            # sort by the logical (possibly unsigned) order: flip the sign bit
            # for unsigned types, sort as signed, flip back
            if dtype.kind == "u":
                sign = torch.tensor(-2**63 if wide else -2**31, dtype=tdt, device=dev)
                a = torch.sort(a ^ sign).values ^ sign
            else:
                a = torch.sort(a).values
            if dist == "reverse":
                a = torch.flip(a, dims=[0])
    return a.contiguous()


def segment_offsets(nseg: int, lo: int = 16, hi: int = 1 << 22, total: int | None = None,
                    seed: int = 8) -> np.ndarray:
    """Offsets (nseg + 1, uint64) of segments with lengths log-uniform in
    [lo, hi]. With `total`, lengths are scaled so they sum to about `total`
    and clamped to at least `lo` (the batched workload's normalisation: the
    unscaled mean on [16, 2^22] would give ~3.4e10 keys for 1e5 segments)."""
    rng = np.random.default_rng(seed)
    lens = np.exp(rng.uniform(np.log(lo), np.log(hi), size=nseg))
    if total is not None:
        lens = lens * (total / lens.sum())
    lens = np.maximum(np.rint(lens), lo).astype(np.uint64)
    off = np.zeros(nseg + 1, np.uint64)
    np.cumsum(lens, out=off[1:])
    return off
