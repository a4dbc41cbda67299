"""Byte-exact parity at the full sizes of the measured workloads.

Every case sorts the same seeded input that bench.py sorts, on the GPU
through the C ABI, and compares the whole output byte for byte with the
CPU oracle (the reference's sort semantics: include/helpers/
hyksort_helper.h:224-297 for pairs, the globally sorted multiset for keys),
run on every host core. Sizes:

* 2^30 uint32 uniform keys (seed 1), the single-array drop-in;
* 2^29 float32 N(0,1) keys (seed 2), radix and the SampleSort shape with
  p = 64 partitions and oversampling 32;
* 2^29 uint32 uniform keys (seed 4) in the HykSort shape, p = 4, k = 4;
* 2^29 uint64 Zipf(1.1) keys with a uint32 index payload (seed 3), stable,
  both orders; and the already-sorted, reverse-sorted, all-equal and
  8-distinct variants of the same pairs;
* 100,000 uint32 segments with lengths log-uniform in [16, 2^22] scaled to
  ~2^30 keys (seed 8), one planned batched sort.
"""
from __future__ import annotations

import numpy as np
import pytest

from gpusort_gb300 import capi, datagen
from oracle import oracle

pytestmark = pytest.mark.gpu


def _host(t, dtype) -> np.ndarray:
    return t.cpu().numpy().view(np.dtype(dtype))


def _sort_keys(ctx, d, dtype, **kw):
    import torch
    o = torch.empty_like(d)
    st = ctx.sort_keys(d, o, dtype=dtype, flags=capi.FLAG_SYNC, **kw)
    assert st == capi.GS_OK, ctx.last_error()
    got = _host(o, dtype)
    del o
    return got


def _same(got: np.ndarray, want: np.ndarray) -> bool:
    return got.shape == want.shape and bool(np.array_equal(got.view(np.uint8),
                                                           want.view(np.uint8)))


def test_u32_uniform_2e30(ctx):
    d = datagen.device("uniform", 1 << 30, np.uint32, seed=1)
    got = _sort_keys(ctx, d, np.uint32)
    want = oracle.sort_keys(_host(d, np.uint32))
    assert _same(got, want)


def test_f32_normal_2e29_radix_and_samplesort(ctx):
    d = datagen.device("normal", 1 << 29, np.float32, seed=2)
    want = oracle.sort_keys(_host(d, np.float32))
    assert _same(_sort_keys(ctx, d, np.float32), want)
    got = _sort_keys(ctx, d, np.float32, algo=capi.ALGO_SAMPLE, partitions=64, oversample=32)
    assert _same(got, want)


def test_u32_uniform_2e29_hyksort_shape(ctx):
    d = datagen.device("uniform", 1 << 29, np.uint32, seed=4)
    got = _sort_keys(ctx, d, np.uint32, algo=capi.ALGO_HYK, partitions=4, k_way=4)
    assert _same(got, oracle.sort_keys(_host(d, np.uint32)))


def _pairs_case(ctx, dist, descending):
    import torch
    n = 1 << 29
    k = datagen.device(dist, n, np.uint64, seed=3)
    v = torch.arange(n, dtype=torch.int32, device=k.device)
    ko, vo = torch.empty_like(k), torch.empty_like(v)
    st = ctx.sort_pairs(k, v, ko, vo, key_dtype=np.uint64, val_dtype=np.uint32,
                        descending=descending, stable=True, flags=capi.FLAG_SYNC)
    assert st == capi.GS_OK, ctx.last_error()
    gk, gv = _host(ko, np.uint64), _host(vo, np.uint32)
    del ko, vo
    wk, wv = oracle.sort_pairs(_host(k, np.uint64), _host(v, np.uint32), descending=descending,
                               stable=True)
    assert _same(gk, wk)
    assert _same(gv, wv)


@pytest.mark.parametrize("descending", [False, True])
def test_u64_zipf_pairs_2e29_stable(ctx, descending):
    _pairs_case(ctx, "zipf", descending)


@pytest.mark.parametrize("dist", ["sorted", "reverse", "equal", "distinct8"])
def test_u64_adversarial_pairs_2e29_stable(ctx, dist):
    _pairs_case(ctx, dist, False)


def test_segmented_100k_2e30(ctx):
    import torch
    off = datagen.segment_offsets(100000, 16, 1 << 22, total=1 << 30, seed=8)
    n = int(off[-1])
    d = datagen.device("uniform", n, np.uint32, seed=8)
    o = torch.empty_like(d)
    plan = ctx.segmented_plan(np.uint32, n, off)
    try:
        assert ctx.segmented_run(plan, d, o) == capi.GS_OK, ctx.last_error()
        assert ctx.status_synchronize() == capi.GS_OK, ctx.last_error()
    finally:
        ctx.segmented_destroy(plan)
    got = _host(o, np.uint32)
    del o
    assert _same(got, oracle.segmented_sort_keys(_host(d, np.uint32), off))
