"""gs_sort_keys_noalloc: the entry point for callers that cannot call
cudaMalloc (code under a framework whose caching allocator owns the device
memory, latency-critical paths where an allocation would synchronise the
device, plugins forbidden to allocate after start-up). It sorts with a fixed
scratch array inside the library instead of allocating.

The test calls it through the C ABI twice in a row and compares each result
with the existing entry point, gs_sort_keys, bit for bit (integer keys: the
tolerance is exact equality). This file is collected last, so a run that
stops at the first failure has already run every other test; it also passes
alone in a fresh process.
"""
import ctypes as C

import numpy as np
import pytest

from gpusort_gb300 import capi, datagen
from tests._util import empty_dev, from_dev, to_dev

pytestmark = pytest.mark.gpu


def _noalloc(L, a, descending, stream):
    d_in, d_out = to_dev(a), empty_dev(a.size, a.dtype)
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


def test_noalloc_matches_gs_sort_keys_on_two_calls_in_a_row(ctx):
    import torch
    L = capi.load()
    stream = torch.cuda.current_stream().cuda_stream or None
    cases = [("uniform", np.uint32, 1 << 20, False), ("normal", np.float32, 300_007, True)]
    for dist, dt, n, desc in cases:
        a = datagen.host(dist, n, dt, seed=n)
        first = _noalloc(L, a, desc, stream)
        second = _noalloc(L, a, desc, stream)     # same scratch, last call's contents
        want = _with_context(ctx, a, desc)
        assert np.array_equal(first.view(np.uint8), want.view(np.uint8)), (dist, 1)
        assert np.array_equal(second.view(np.uint8), want.view(np.uint8)), (dist, 2)


def test_noalloc_rejects_sizes_beyond_its_limit(ctx):
    L = capi.load()
    limit = 1 << 20
    st = L.gs_sort_keys_noalloc(capi.GS_U32, C.c_void_p(16), C.c_void_p(16), limit + 1,
                                capi.FLAG_SYNC, None)
    assert st == capi.GS_ERR_TOO_LARGE
    assert b"exceeds its fixed scratch limit" in L.gs_last_global_error()
    st = L.gs_sort_keys_noalloc(capi.GS_U64, C.c_void_p(16), C.c_void_p(16), 10, 0, None)
    assert st == capi.GS_ERR_BAD_DTYPE
