"""Parity of the onesweep radix sort with the CPU oracle, through the C ABI.

Bit-exact comparison for every key type of the reference's instantiation
set (src/cuda_utils.cu:257-262), ascending (std::less) and descending
(std::greater), over the reference's test distributions (src/test/utils.h:
425-608) plus the adversarial ones of the sort workloads.
"""
import numpy as np
import pytest

from gpusort_gb300 import capi, datagen
from oracle import oracle
from tests._util import empty_dev, from_dev, same_bits, to_dev

pytestmark = pytest.mark.gpu

DTYPES = [np.uint32, np.int32, np.float32, np.uint64, np.int64, np.float64]
SMALL = [1, 2, 3, 31, 32, 33, 255, 256, 257, 1000, 4095, 4096, 4097, 6143, 6144, 6145, 8191, 8192, 8193,
         16383, 16384, 16385, 40000]
DISTS = ["uniform", "sorted", "reverse", "equal", "distinct8", "zipf"]


def _sort(ctx, a, descending=False, in_place=False):
    d_in = to_dev(a)
    d_out = d_in if in_place else empty_dev(a.size, a.dtype)
    st = ctx.sort_keys(d_in, d_out, dtype=a.dtype, descending=descending, flags=capi.FLAG_SYNC)
    assert st == capi.GS_OK, ctx.last_error()
    return from_dev(d_out, a.dtype)


@pytest.mark.parametrize("dtype", DTYPES)
@pytest.mark.parametrize("dist", DISTS)
def test_keys_small_sizes(ctx, dtype, dist):
    for i, n in enumerate(SMALL):
        a = datagen.host(dist, n, dtype, seed=100 + i)
        for desc in (False, True):
            got = _sort(ctx, a, desc)
            want = oracle.sort_keys(a, desc)
            assert same_bits(got, want), (dtype, dist, n, desc)


@pytest.mark.parametrize("dtype", DTYPES)
@pytest.mark.parametrize("n", [1 << 20, (1 << 22) + 12345])
def test_keys_large_uniform(ctx, dtype, n):
    a = datagen.host("uniform", n, dtype, seed=7)
    for desc in (False, True):
        assert same_bits(_sort(ctx, a, desc), oracle.sort_keys(a, desc)), (dtype, n, desc)


@pytest.mark.parametrize("dtype", [np.uint32, np.uint64, np.float32])
@pytest.mark.parametrize("dist", ["zipf", "distinct8", "equal", "sorted", "reverse"])
def test_keys_large_adversarial(ctx, dtype, dist):
    a = datagen.host(dist, (1 << 21) + 77, dtype, seed=11)
    for desc in (False, True):
        assert same_bits(_sort(ctx, a, desc), oracle.sort_keys(a, desc)), (dtype, dist, desc)


@pytest.mark.parametrize("dtype", [np.uint32, np.int32, np.uint64])
@pytest.mark.parametrize("mask_kind", ["low8", "low16", "mid8", "low24"])
def test_keys_constant_digits(ctx, dtype, mask_kind):
    """Digits shared by every key are skipped, so the first pass that runs is
    a higher digit's (the lowest digit's own kernel does not run) or a
    later pass follows a skipped one: keys with the low byte(s) or a middle
    byte cleared, over several tiles, both orders."""
    bits = np.dtype(dtype).itemsize * 8
    u = np.dtype(f"u{bits // 8}")
    keep = {"low8": ~np.uint64(0xFF), "low16": ~np.uint64(0xFFFF), "mid8": ~np.uint64(0xFF00),
            "low24": ~np.uint64(0xFFFFFF)}[mask_kind]
    for i, n in enumerate([4097, (1 << 21) + 333]):
        r = datagen.host("uniform", n, u, seed=60 + i).astype(np.uint64)
        a = (r & keep).astype(u).view(dtype)
        for desc in (False, True):
            assert same_bits(_sort(ctx, a, desc), oracle.sort_keys(a, desc)), (dtype, mask_kind, n, desc)


@pytest.mark.parametrize("dtype", [np.uint32, np.float64, np.int32])
@pytest.mark.parametrize("dist", ["uniform", "equal", "distinct8"])
def test_keys_in_place(ctx, dtype, dist):
    for n in (1, 100, 8193, 300001):
        a = datagen.host(dist, n, dtype, seed=5)
        for desc in (False, True):
            assert same_bits(_sort(ctx, a, desc, in_place=True), oracle.sort_keys(a, desc))


def test_keys_float_specials(ctx):
    a = np.array([np.inf, -np.inf, 0.0, 1e-45, -1e-45, 3.4e38, -3.4e38, 1.0, -1.0, 2.5] * 1000,
                 dtype=np.float32)
    for desc in (False, True):
        assert same_bits(_sort(ctx, a, desc), oracle.sort_keys(a, desc))


def test_keys_host_pointers(ctx):
    a = datagen.host("uniform", 123457, np.uint32, seed=9)
    out = np.empty_like(a)
    st = ctx.sort_keys(a, out, flags=capi.FLAG_HOST)
    assert st == capi.GS_OK, ctx.last_error()
    assert same_bits(out, oracle.sort_keys(a))
    b = a.copy()
    st = ctx.sort_keys(b, b, flags=capi.FLAG_HOST, descending=True)
    assert st == capi.GS_OK
    assert same_bits(b, oracle.sort_keys(a, True))


def test_empty_input_reports_empty(ctx):
    a = np.empty(0, np.uint32)
    st = ctx.sort_keys(a, a, flags=capi.FLAG_HOST)
    assert st == capi.GS_ERR_EMPTY
    assert ctx.last_error() == "No data to sort."


PAIR_TYPES = [(np.uint32, np.uint32), (np.uint64, np.uint32), (np.float32, np.uint64),
              (np.int64, np.uint32), (np.float64, np.float64), (np.int32, np.int64),
              (np.uint32, np.float32), (np.uint64, np.uint64)]


def _pairs(ctx, k, v, descending, stable, in_place=False):
    dk, dv = to_dev(k), to_dev(v)
    ok = dk if in_place else empty_dev(k.size, k.dtype)
    ov = dv if in_place else empty_dev(v.size, v.dtype)
    st = ctx.sort_pairs(dk, dv, ok, ov, key_dtype=k.dtype, val_dtype=v.dtype,
                        descending=descending, stable=stable, flags=capi.FLAG_SYNC)
    assert st == capi.GS_OK, ctx.last_error()
    return from_dev(ok, k.dtype), from_dev(ov, v.dtype)


@pytest.mark.parametrize("kt,vt", PAIR_TYPES)
@pytest.mark.parametrize("stable", [False, True])
def test_pairs(ctx, kt, vt, stable):
    for i, n in enumerate([1, 33, 5000, 6145, 100003]):
        for dist in ("distinct8", "uniform", "zipf"):
            k = datagen.host(dist, n, kt, seed=i)
            v = (np.arange(n, dtype=np.uint64).astype(vt) if stable
                 else datagen.host("distinct8" if i % 2 else "uniform", n, vt, seed=i + 50))
            for desc in (False, True):
                gk, gv = _pairs(ctx, k, v, desc, stable, in_place=(i == 3))
                wk, wv = oracle.sort_pairs(k, v, desc, stable)
                assert same_bits(gk, wk) and same_bits(gv, wv), (kt, vt, n, dist, desc, stable)


@pytest.mark.parametrize("kt,vt", [(np.uint32, np.uint32), (np.uint64, np.uint32)])
@pytest.mark.parametrize("stable", [False, True])
def test_pairs_constant_low_key_digit(ctx, kt, vt, stable):
    """Keys with the low byte cleared: the key's lowest digit is skipped,
    after the value digits (ties by value) or first (index payload)."""
    n = (1 << 20) + 4097
    u = np.dtype(f"u{np.dtype(kt).itemsize}")
    k = (datagen.host("uniform", n, u, seed=71).astype(np.uint64) & ~np.uint64(0xFF)).astype(u).view(kt)
    v = (np.arange(n, dtype=np.uint64).astype(vt) if stable
         else datagen.host("distinct8", n, vt, seed=72))
    for desc in (False, True):
        gk, gv = _pairs(ctx, k, v, desc, stable)
        wk, wv = oracle.sort_pairs(k, v, desc, stable)
        assert same_bits(gk, wk) and same_bits(gv, wv), (kt, vt, desc, stable)


@pytest.mark.parametrize("kt,vt", [(np.uint32, np.uint32), (np.int64, np.uint32),
                                   (np.float32, np.uint64), (np.uint64, np.int64)])
def test_pairs_values_in_order(ctx, kt, vt):
    """Ties ordered by value when the values already run in order (an index
    payload): the engine drops the value digits and keeps ties in input
    order (reversed when descending). Few distinct keys make every tie
    visible; a single out-of-order value (at a warp boundary, at a
    4096-element chunk boundary, at the end) must switch the shortcut off."""
    for n in (1000, 100003, (1 << 21) + 7):
        k = datagen.host("distinct8", n, kt, seed=n)
        base = np.arange(n, dtype=np.uint64) // 3  # non-decreasing, with runs
        cases = [base.astype(vt)]
        for pos in sorted({31, min(4095, n - 2), n - 2}):
            v = base.copy()
            v[pos], v[pos + 1] = base[pos + 1] + 1, base[pos]
            cases.append(v.astype(vt))
        for v in cases:
            for desc in (False, True):
                for in_place in (False, True):
                    gk, gv = _pairs(ctx, k, v, desc, False, in_place=in_place)
                    wk, wv = oracle.sort_pairs(k, v, desc, False)
                    assert same_bits(gk, wk) and same_bits(gv, wv), (n, desc, in_place)


@pytest.mark.parametrize("kt", [np.float32, np.float64])
def test_signed_zero_keys(ctx, kt):
    """std::less treats -0.0 and +0.0 as equal keys: pair sorts tie them by
    value (or by input order when stable), as the oracle's std::pair and
    std::stable_sort orders do; keys keep their bits. Keys-only sorts put
    -0.0 first (an order std::less allows)."""
    ubits = np.uint32 if kt is np.float32 else np.uint64
    sign = ubits(1) << ubits(8 * np.dtype(kt).itemsize - 1)
    for n in (1000, 100003):
        rng = np.random.default_rng(n)
        k = rng.choice(np.array([-0.0, 0.0, -1.5, 2.0, -np.inf], dtype=kt), size=n)
        for desc in (False, True):
            for stable in (False, True):
                # Ties by value need distinct values: (-0.0, v) and (+0.0, v)
                # would be equal elements with different bits.
                v = (rng.integers(0, 64, size=n, dtype=np.uint32) if stable
                     else rng.permutation(n).astype(np.uint32))
                gk, gv = _pairs(ctx, k, v, desc, stable)
                wk, wv = oracle.sort_pairs(k, v, desc, stable)
                assert same_bits(gk, wk) and same_bits(gv, wv), (n, desc, stable)
            got = _sort(ctx, k, desc)
            b = got.view(ubits)
            key = np.where(b & sign, ~b, b | sign)  # total order, -0.0 < +0.0
            key = ~key if desc else key
            assert np.all(key[1:] >= key[:-1])
            assert same_bits(np.sort(got.view(ubits)), np.sort(k.view(ubits)))


def test_pairs_stable_index_payload_large(ctx):
    """(uint64 key, uint32 original index) pairs, Zipf keys: stable order."""
    n = (1 << 21) + 3
    k = datagen.host("zipf", n, np.uint64, seed=3)
    v = np.arange(n, dtype=np.uint32)
    for desc in (False, True):
        gk, gv = _pairs(ctx, k, v, desc, True)
        wk, wv = oracle.sort_pairs(k, v, desc, True)
        assert same_bits(gk, wk) and same_bits(gv, wv)


def test_lookback_wait_runs_out_and_context_recovers(ctx):
    """A tile waits on a predecessor flag that is never set: the bounded
    wait ends, the call reports GS_ERR_TIMEOUT, and the next sort is right."""
    a = datagen.host("uniform", 200000, np.uint32, seed=1)
    d_in, d_out = to_dev(a), empty_dev(a.size, np.uint32)
    ctx.debug_set(capi.DEBUG_SPIN_LIMIT, 2000)
    ctx.debug_set(capi.DEBUG_INJECT_STALL, 1)
    st = ctx.sort_keys(d_in, d_out, dtype=np.uint32, flags=capi.FLAG_SYNC)
    ctx.debug_set(capi.DEBUG_SPIN_LIMIT, 1 << 20)
    assert st == capi.GS_ERR_TIMEOUT
    assert "ran out" in ctx.last_error()
    assert same_bits(_sort(ctx, a), oracle.sort_keys(a))


def test_budget_exhausted_reports_oom(built_lib):
    import torch
    from gpusort_gb300 import Context
    c = Context(0, hbm_budget_bytes=1 << 20)
    try:
        a = datagen.host("uniform", 1 << 20, np.uint32, seed=2)
        d = to_dev(a)
        st = c.sort_keys(d, d, dtype=np.uint32, flags=capi.FLAG_SYNC)
        assert st == capi.GS_ERR_OOM
        assert "budget" in c.last_error()
        torch.cuda.synchronize()
    finally:
        c.close()


@pytest.mark.parametrize("shape", [0, 1, 2])
@pytest.mark.parametrize("kt,vt", [(np.uint32, None), (np.uint64, None), (np.float32, np.uint32),
                                   (np.int64, np.uint64)])
def test_every_tile_shape(ctx, shape, kt, vt):
    """Each pass-kernel tile shape the autotuner may pick gives the same bytes."""
    ctx.debug_set(capi.DEBUG_PASS_SHAPE, shape)
    try:
        for n in (1, 777, 8193, 100003, 1 << 20):
            k = datagen.host("uniform" if n % 2 else "distinct8", n, kt, seed=n + shape)
            if vt is None:
                for desc in (False, True):
                    assert same_bits(_sort(ctx, k, desc), oracle.sort_keys(k, desc))
            else:
                v = datagen.host("uniform", n, vt, seed=n + 1)
                for stable in (False, True):
                    gk, gv = _pairs(ctx, k, v, True, stable)
                    wk, wv = oracle.sort_pairs(k, v, True, stable)
                    assert same_bits(gk, wk) and same_bits(gv, wv)
    finally:
        ctx.debug_set(capi.DEBUG_PASS_SHAPE, (1 << 64) - 1)


@pytest.mark.parametrize("n", [1, 3, 1001, 65537, (1 << 20) + 5])
@pytest.mark.parametrize("dist", ["uniform", "equal"])
def test_pinned_host_buffers(ctx, n, dist):
    """GS_FLAG_HOST with pinned host memory. On the radix path the upsweep
    reads the input across the CPU-GPU link and keeps the device copy the
    passes sort (all-equal keys: every digit trivial); the SampleSort shape
    moves the buffers with copy kernels. Outputs go back by copy kernel (an
    unaligned view falls back to the copy engine)."""
    import torch
    a = datagen.host(dist, n, np.uint32, seed=n)
    v = np.arange(n, dtype=np.uint32)
    for off in (0, 1):  # off 1: 4-byte offset, not 16-byte aligned
        hk = torch.empty(n + off, dtype=torch.int32, pin_memory=True)
        hv = torch.empty(n + off, dtype=torch.int32, pin_memory=True)
        ko = torch.empty(n + off, dtype=torch.int32, pin_memory=True)
        vo = torch.empty(n + off, dtype=torch.int32, pin_memory=True)
        hk[off:].copy_(torch.from_numpy(a.view(np.int32)))
        hv[off:].copy_(torch.from_numpy(v.view(np.int32)))
        for algo in (capi.ALGO_AUTO, capi.ALGO_SAMPLE):
            ko.zero_()
            st = ctx.sort_keys(hk[off:], ko[off:], dtype=np.uint32, flags=capi.FLAG_HOST,
                               algo=algo)
            assert st == capi.GS_OK, ctx.last_error()
            assert same_bits(ko[off:].numpy().view(np.uint32), oracle.sort_keys(a))
        for desc, stable in ((True, True), (False, False)):
            ko.zero_()
            vo.zero_()
            st = ctx.sort_pairs(hk[off:], hv[off:], ko[off:], vo[off:], key_dtype=np.uint32,
                                val_dtype=np.uint32, descending=desc, stable=stable,
                                flags=capi.FLAG_HOST)
            assert st == capi.GS_OK, ctx.last_error()
            wk, wv = oracle.sort_pairs(a, v, desc, stable)
            assert same_bits(ko[off:].numpy().view(np.uint32), wk)
            assert same_bits(vo[off:].numpy().view(np.uint32), wv)
        assert same_bits(hk[off:].numpy().view(np.uint32), a)  # input untouched


def test_random_sizes_across_dispatch_boundaries(ctx):
    """Seeded random sizes from 1 to ~2^21 cross every size-dependent choice
    (one-CTA sort up to 4096 keys, 256-thread tiles up to 2^18 keys, the
    narrow upsweep below 2^20), for every key type, both orders, keys and
    pairs in both tie orders."""
    rng = np.random.default_rng(20261203)
    sizes = sorted(set(int(x) for x in np.exp2(rng.uniform(0, 21, size=36)).astype(np.int64)) |
                   {4096, 4097, (1 << 18), (1 << 18) + 1, (1 << 20) - 1, 1 << 20})
    for j, n in enumerate(sizes):
        kt = DTYPES[j % len(DTYPES)]
        dist = ("uniform", "zipf", "distinct8", "reverse")[j % 4]
        a = datagen.host(dist, n, kt, seed=j)
        desc = bool(j & 1)
        assert same_bits(_sort(ctx, a, desc), oracle.sort_keys(a, desc)), (n, kt, dist, desc)
        if n <= (1 << 20):
            v = np.arange(n, dtype=np.uint32)[::-1].copy()
            stable = bool(j & 2)
            gk, gv = _pairs(ctx, a, v, desc, stable)
            wk, wv = oracle.sort_pairs(a, v, desc, stable)
            assert same_bits(gk, wk) and same_bits(gv, wv), (n, kt, dist, desc, stable)
