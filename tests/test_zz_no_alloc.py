"""gs_sort_keys_noalloc: the entry point for callers that cannot call
cudaMalloc (code under a framework whose caching allocator owns the device
memory, latency-critical paths where an allocation would synchronise the
device, plugins forbidden to allocate after start-up). It sorts with a fixed
scratch array inside the library instead of allocating.

The tests call it through the C ABI, twice in a row per input, and compare
each result with the CPU oracle and with the existing entry point,
gs_sort_keys, bit for bit (integer work: the tolerance is exact equality).
They cover every 32-bit key type, the one-CTA sizes (1, 4096) and the
pipeline sizes (4097 up to the 2^20-key limit), in place, on a non-blocking
stream (the first call of a fresh process comes on one), and that a call
leaves the device's free memory unchanged. This file is collected last, so a
run that stops at the first failure has already run every other test; it
also passes alone in a fresh process.
"""
import ctypes as C

import numpy as np
import pytest

from gpusort_gb300 import capi, datagen
from oracle import oracle
from tests._util import empty_dev, from_dev, to_dev

pytestmark = pytest.mark.gpu

LIMIT = 1 << 20


def _noalloc(L, d_in, d_out, a, descending, stream):
    flags = capi.FLAG_SYNC | (capi.FLAG_DESCENDING if descending else 0)
    st = L.gs_sort_keys_noalloc(capi.dtype_code(a.dtype), d_in.data_ptr(), d_out.data_ptr(),
                                a.size, flags, stream)
    assert st == capi.GS_OK, L.gs_last_global_error().decode()
    return from_dev(d_out, a.dtype)


def _with_context(ctx, a, descending):
    d_in, d_out = to_dev(a), empty_dev(a.size, a.dtype)
    st = ctx.sort_keys(d_in, d_out, dtype=a.dtype, descending=descending, flags=capi.FLAG_SYNC)
    assert st == capi.GS_OK, ctx.last_error()
    return from_dev(d_out, a.dtype)


def _same(x, y):
    return np.array_equal(x.view(np.uint8), y.view(np.uint8))


def test_noalloc_first_call_on_a_non_blocking_stream(ctx):
    """The scratch set-up clears the array before any sort is enqueued, also
    when the first call comes on a stream that does not wait for the legacy
    default stream."""
    import torch
    L = capi.load()
    side = torch.cuda.Stream()  # torch's side streams are non-blocking
    a = datagen.host("uniform", LIMIT, np.uint32, seed=11)
    d_in, d_out = to_dev(a), empty_dev(a.size, a.dtype)
    torch.cuda.synchronize()
    want = oracle.sort_keys(a)
    for _ in range(2):
        assert _same(_noalloc(L, d_in, d_out, a, False, side.cuda_stream), want)


@pytest.mark.parametrize("dtype,dist", [(np.uint32, "uniform"), (np.int32, "uniform"),
                                        (np.float32, "normal"), (np.int32, "distinct8")])
@pytest.mark.parametrize("n", [1, 4096, 4097, 300_007, LIMIT])
def test_noalloc_matches_oracle_and_gs_sort_keys_on_two_calls_in_a_row(ctx, dtype, dist, n):
    import torch
    L = capi.load()
    stream = torch.cuda.current_stream().cuda_stream or None
    for desc in (False, True):
        a = datagen.host(dist, n, dtype, seed=n + int(desc))
        want = oracle.sort_keys(a, desc)
        assert _same(_with_context(ctx, a, desc), want)
        d_in, d_out = to_dev(a), empty_dev(a.size, a.dtype)
        first = _noalloc(L, d_in, d_out, a, desc, stream)
        second = _noalloc(L, d_in, d_out, a, desc, stream)  # the array keeps the last call's data
        assert _same(first, want), (n, desc, 1)
        assert _same(second, want), (n, desc, 2)


@pytest.mark.parametrize("n", [4096, 4097, LIMIT])
def test_noalloc_in_place(ctx, n):
    import torch
    L = capi.load()
    stream = torch.cuda.current_stream().cuda_stream or None
    a = datagen.host("uniform", n, np.int32, seed=n)
    d = to_dev(a)
    got = _noalloc(L, d, d, a, True, stream)
    assert _same(got, oracle.sort_keys(a, True))


def test_noalloc_allocates_nothing(ctx):
    """Free device memory is the same before and after a call (buffers made
    first; the first call has loaded the kernels)."""
    import torch
    L = capi.load()
    stream = torch.cuda.current_stream().cuda_stream or None
    a = datagen.host("uniform", LIMIT, np.uint32, seed=3)
    d_in, d_out = to_dev(a), empty_dev(a.size, a.dtype)
    _noalloc(L, d_in, d_out, a, False, stream)
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    got = _noalloc(L, d_in, d_out, a, False, stream)
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free0
    assert _same(got, oracle.sort_keys(a))


def test_noalloc_rejects_sizes_beyond_its_limit(ctx):
    L = capi.load()
    st = L.gs_sort_keys_noalloc(capi.GS_U32, C.c_void_p(16), C.c_void_p(16), LIMIT + 1,
                                capi.FLAG_SYNC, None)
    assert st == capi.GS_ERR_TOO_LARGE
    assert b"exceeds its fixed scratch limit" in L.gs_last_global_error()
    st = L.gs_sort_keys_noalloc(capi.GS_U64, C.c_void_p(16), C.c_void_p(16), 10, 0, None)
    assert st == capi.GS_ERR_BAD_DTYPE
