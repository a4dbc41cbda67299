"""GS_FLAG_HOST sorts of pinned buffers in bucket groups.

The upsweep reads the input across the CPU-GPU link; one pass on the most
significant digit that varies splits it into buckets; runs of buckets are
sorted on the digits below, and each run is copied to the host while the
next one sorts. The results must be bit-identical to the oracle and to the
same call with grouping off (GS_DEBUG_HOST_GROUPS 0), for key ranges that
move the split digit (odd and even digit positions, all keys equal), every
key width, pairs in both tie orders, and group counts from 2 to 256.
"""
import numpy as np
import pytest

from gpusort_gb300 import capi, datagen
from oracle import oracle
from tests._util import same_bits

pytestmark = pytest.mark.gpu

N = (1 << 22) + 5  # ragged; grouping is set explicitly (by size it starts at 2^25)


def _pinned(a: np.ndarray):
    """Pinned host tensor holding the bytes of `a`, and a numpy view of it."""
    import torch
    t = torch.empty(a.nbytes, dtype=torch.uint8, pin_memory=True)
    v = t.numpy().view(a.dtype)
    v[:] = a
    return t, v


def _keys(dtype, bits, seed):
    a = datagen.host("uniform", N, dtype, seed=seed)
    if bits is None:
        return a
    if bits == 0:
        return np.full(N, a[0], dtype=dtype)
    u = a.view(np.uint64 if a.itemsize == 8 else np.uint32)
    return (u & ((1 << bits) - 1)).astype(u.dtype).view(dtype)


def _sort_keys(ctx, a, desc, groups):
    ctx.debug_set(capi.DEBUG_HOST_GROUPS, groups)
    hin, vin = _pinned(a)
    hout, vout = _pinned(np.zeros_like(a))
    st = ctx.sort_keys(hin, hout, n=a.size, dtype=a.dtype, descending=desc, flags=capi.FLAG_HOST)
    assert st == capi.GS_OK, ctx.last_error()
    assert same_bits(vin, a)  # input untouched
    return vout.copy()


@pytest.fixture()
def gctx(ctx):
    yield ctx
    ctx.debug_set(capi.DEBUG_HOST_GROUPS, (1 << 64) - 1)


# bits: keys masked to that many low bits (split digit 3, 2, 1, 1, 0), or
# None (full range), or 0 (every key equal). 8 groups are runs of several
# buckets, sorted up to the split digit; 256 groups are mostly single
# buckets, sorted below it (with 8-bit keys: already in order after the
# split).
@pytest.mark.parametrize("bits", [None, 24, 16, 9, 8, 0])
def test_u32_split_digit_positions(gctx, bits):
    a = _keys(np.uint32, bits, seed=11)
    for desc in (False, True):
        want = oracle.sort_keys(a, desc)
        for groups in (8, 256, 0):
            got = _sort_keys(gctx, a, desc, groups)
            assert same_bits(got, want), (bits, desc, groups)


@pytest.mark.parametrize("dtype", [np.int32, np.float32, np.uint64, np.int64, np.float64])
def test_key_types(gctx, dtype):
    if dtype is np.float32:
        a = datagen.host("normal", N, dtype, seed=3)
    else:
        a = _keys(dtype, 40 if dtype is np.uint64 else None, seed=3)
    for desc in (False, True):
        assert same_bits(_sort_keys(gctx, a, desc, 8), oracle.sort_keys(a, desc)), (dtype, desc)


@pytest.mark.parametrize("groups", [2, 3, 16, 256])
def test_group_counts(gctx, groups):
    a = datagen.host("zipf", N, np.uint32, seed=5)
    want = oracle.sort_keys(a)
    assert same_bits(_sort_keys(gctx, a, False, groups), want)


@pytest.mark.parametrize("kdt,vdt", [(np.uint32, np.uint32), (np.uint64, np.uint32),
                                     (np.float32, np.uint64)])
def test_pairs(gctx, kdt, vdt):
    # Many equal keys, so both tie orders are exercised (the rounded normal
    # keys include -0.0 and +0.0, equal under std::less; values are
    # distinct).
    k = _keys(kdt, 12, seed=7) if kdt is not np.float32 else \
        datagen.host("normal", N, kdt, seed=7).round(2)
    v = np.arange(N, dtype=vdt)[::-1].copy()
    for desc, stable in ((False, False), (True, False), (False, True), (True, True)):
        want_k, want_v = oracle.sort_pairs(k, v, desc, stable)
        for groups in (8, 256, 0):
            gctx.debug_set(capi.DEBUG_HOST_GROUPS, groups)
            hk, _ = _pinned(k)
            hv, _ = _pinned(v)
            ok_, vk = _pinned(np.zeros_like(k))
            ov_, vv = _pinned(np.zeros_like(v))
            st = gctx.sort_pairs(hk, hv, ok_, ov_, n=N, key_dtype=kdt, val_dtype=vdt,
                                 descending=desc, stable=stable, flags=capi.FLAG_HOST)
            assert st == capi.GS_OK, gctx.last_error()
            assert same_bits(vk, want_k), (kdt, vdt, desc, stable, groups)
            assert same_bits(vv, want_v), (kdt, vdt, desc, stable, groups)


def test_repeated_calls_and_stall(gctx):
    """Back-to-back grouped sorts reuse the context's buffers and copy
    stream; an injected look-back stall in the split pass is reported and
    the next call succeeds."""
    a = datagen.host("uniform", N, np.uint32, seed=9)
    want = oracle.sort_keys(a)
    for _ in range(3):
        assert same_bits(_sort_keys(gctx, a, False, 8), want)
    gctx.debug_set(capi.DEBUG_SPIN_LIMIT, 2000)
    gctx.debug_set(capi.DEBUG_INJECT_STALL, 1)
    hin, _ = _pinned(a)
    hout, _ = _pinned(np.zeros_like(a))
    st = gctx.sort_keys(hin, hout, n=N, dtype=np.uint32, flags=capi.FLAG_HOST)
    gctx.debug_set(capi.DEBUG_SPIN_LIMIT, 1 << 20)
    assert st == capi.GS_ERR_TIMEOUT
    assert "ran out" in gctx.last_error()
    assert same_bits(_sort_keys(gctx, a, False, 8), want)


def test_default_grouping_by_size_and_phases(gctx):
    """With the default choice a 2^25-element host sort is grouped; the
    phase timer reports the three stages with positive times."""
    n = (1 << 25) + 3
    a = datagen.host("uniform", n, np.uint32, seed=13)
    hin, _ = _pinned(a)
    hout, vout = _pinned(np.zeros_like(a))
    gctx.set_timing(True)
    try:
        st = gctx.sort_keys(hin, hout, n=n, dtype=np.uint32, flags=capi.FLAG_HOST)
        assert st == capi.GS_OK, gctx.last_error()
        ph = gctx.phase_times()
    finally:
        gctx.set_timing(False)
    assert list(ph) == ["Transfer in", "Split", "Sort and transfer out"]
    assert all(t > 0 for t in ph.values())
    assert same_bits(vout, oracle.sort_keys(a))


@pytest.fixture()
def chunked(gctx):
    """Chunk-by-chunk splitting from 4096 keys, so 2^22-key cases take it."""
    gctx.debug_set(capi.DEBUG_HOST_CHUNKED, 4096)
    yield gctx
    gctx.debug_set(capi.DEBUG_HOST_CHUNKED, 1 << 28)


# Key ranges: the top digit varies (chunked split) or is constant (the
# single split on the digit below, after the chunks are in).
@pytest.mark.parametrize("bits", [None, 24, 8, 0])
@pytest.mark.parametrize("dtype", [np.uint32, np.float32, np.int64])
def test_chunked_split(chunked, bits, dtype):
    if dtype is np.float32:
        a = datagen.host("normal", N, dtype, seed=17) if bits is None else _keys(dtype, bits, 17)
    else:
        a = _keys(dtype, bits, seed=17)
    for desc in (False, True):
        want = oracle.sort_keys(a, desc)
        for groups in (8, 256, 2):
            got = _sort_keys(chunked, a, desc, groups)
            assert same_bits(got, want), (bits, desc, groups)


def test_chunked_ragged_and_repeated(chunked):
    """Chunk lengths are multiples of 4096 keys: sizes just around that,
    zipf keys, back-to-back calls reusing the chunk work areas."""
    for n in (4096 * 4 + 1, 4096 * 3 + 4095, (1 << 20) + 17):
        a = datagen.host("zipf", n, np.uint32, seed=n)
        want = oracle.sort_keys(a)
        for _ in range(2):
            assert same_bits(_sort_keys(chunked, a, False, 8), want), n


@pytest.mark.parametrize("chunk_min", [0, 4096])
def test_in_place(gctx, chunk_min):
    """Output buffer = input buffer: every read of the input (upsweeps across
    the link) completes before the first run is copied out."""
    gctx.debug_set(capi.DEBUG_HOST_CHUNKED, chunk_min)
    try:
        for dtype, dist in ((np.uint32, "uniform"), (np.int64, "zipf")):
            a = datagen.host(dist, N, dtype, seed=21)
            for desc in (False, True):
                for groups in (8, 0):
                    gctx.debug_set(capi.DEBUG_HOST_GROUPS, groups)
                    h, v = _pinned(a)
                    st = gctx.sort_keys(h, h, n=N, dtype=dtype, descending=desc,
                                        flags=capi.FLAG_HOST)
                    assert st == capi.GS_OK, gctx.last_error()
                    assert same_bits(v, oracle.sort_keys(a, desc)), (dtype, desc, groups)
    finally:
        gctx.debug_set(capi.DEBUG_HOST_CHUNKED, 1 << 28)
