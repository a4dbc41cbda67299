"""Serving loop (gs_server_*): every result is the same alone and in the mix.

Requests of the serving mix (uint32 / uint64 / float32 keys, int64 keys with
uint32 values) run concurrently through the server; each output is compared
bit for bit with the same input sorted alone by the plain call
(gs_sort_keys / gs_sort_pairs) and, for the smaller requests, with the CPU
oracle. Admission by HBM budget, host-staged requests, cancellation and the
error statuses are covered too.
"""
import numpy as np
import pytest

from gpusort_gb300 import capi, datagen, serving
from oracle import oracle
from tests._util import empty_dev, from_dev, same_bits, to_dev

pytestmark = pytest.mark.gpu


def _solo(ctx, r: serving.DeviceRequest):
    import torch
    k_out = torch.empty_like(r.keys)
    if r.vals is None:
        st = ctx.sort_keys(r.keys, k_out, dtype=r.spec.key_dtype, flags=capi.FLAG_SYNC)
        assert st == capi.GS_OK, ctx.last_error()
        return k_out, None
    v_out = torch.empty_like(r.vals)
    st = ctx.sort_pairs(r.keys, r.vals, k_out, v_out, key_dtype=r.spec.key_dtype,
                        val_dtype=r.spec.val_dtype, flags=capi.FLAG_SYNC)
    assert st == capi.GS_OK, ctx.last_error()
    return k_out, v_out


def _bits(t, dtype):
    return from_dev(t, dtype)


@pytest.mark.parametrize("slots", [1, 4, 16])
def test_mix_same_alone_and_in_mix(ctx, slots):
    specs = serving.request_mix(48, lo_log2=10, hi_log2=22, seed=11 + slots)
    reqs = [serving.DeviceRequest(s) for s in specs]
    with capi.Server(0, hbm_budget=1 << 30, max_request_keys=1 << 22, slots=slots) as srv:
        ids = [r.submit(srv) for r in reqs]
        for i in ids:
            st, ms = srv.poll(i, wait=True)
            assert st == capi.GS_OK
            assert ms >= 0
        stats = srv.stats()
        assert stats["completed"] == len(reqs)
        assert stats["keys_done"] == sum(s.n for s in specs)
        assert stats["arena_peak"] <= 1 << 30
        assert stats["running"] == 0 and stats["queued"] == 0
    for r in reqs:
        k_solo, v_solo = _solo(ctx, r)
        kd = r.spec.key_dtype
        assert same_bits(_bits(r.keys_out, kd), _bits(k_solo, kd)), r.spec
        if r.vals is not None:
            assert same_bits(_bits(r.vals_out, np.uint32), _bits(v_solo, np.uint32)), r.spec
        if r.spec.n <= 1 << 18:
            a = _bits(r.keys, kd)
            if r.vals is None:
                assert same_bits(_bits(r.keys_out, kd), oracle.sort_keys(a)), r.spec
            else:
                wk, wv = oracle.sort_pairs(a, _bits(r.vals, np.uint32))
                assert same_bits(_bits(r.keys_out, kd), wk), r.spec
                assert same_bits(_bits(r.vals_out, np.uint32), wv), r.spec


def test_admission_by_budget(ctx):
    # 24 requests of 2^20 uint64 keys need 8 MiB of scratch each; a 20 MiB
    # arena admits two at a time whatever the slot count.
    budget = 20 << 20
    n = 1 << 20
    specs = [serving.RequestSpec(n, np.uint64, None, 900 + i) for i in range(24)]
    reqs = [serving.DeviceRequest(s) for s in specs]
    with capi.Server(0, hbm_budget=budget, max_request_keys=n, slots=8) as srv:
        ids = [r.submit(srv) for r in reqs]
        for i in ids:
            assert srv.poll(i, wait=True)[0] == capi.GS_OK
        st = srv.stats()
        assert 8 << 20 <= st["arena_peak"] <= 2 * (8 << 20)
    for r in reqs:
        want = oracle.sort_keys(_bits(r.keys, np.uint64))
        assert same_bits(_bits(r.keys_out, np.uint64), want)


@pytest.mark.parametrize("descending,stable", [(False, False), (True, False), (True, True)])
def test_host_requests(ctx, descending, stable):
    with capi.Server(0, hbm_budget=256 << 20, max_request_keys=1 << 20, slots=4) as srv:
        jobs = []
        for i, n in enumerate([1, 1000, 65537, 300000]):
            k = datagen.host("zipf", n, np.uint64, seed=40 + i)
            v = np.arange(n, dtype=np.uint32)
            ko = np.empty_like(k)
            vo = np.empty_like(v)
            rid = srv.submit(k, ko, v, vo, descending=descending, stable=stable,
                             flags=capi.FLAG_HOST)
            jobs.append((rid, k, v, ko, vo))
        for rid, k, v, ko, vo in jobs:
            assert srv.poll(rid, wait=True)[0] == capi.GS_OK
            wk, wv = oracle.sort_pairs(k, v, descending, stable)
            assert same_bits(ko, wk) and same_bits(vo, wv)


def test_in_place_device_request(ctx):
    a = datagen.host("uniform", 123457, np.float32, seed=3)
    d = to_dev(a)
    with capi.Server(0, hbm_budget=64 << 20, max_request_keys=1 << 20, slots=2) as srv:
        rid = srv.submit(d, d, key_dtype=np.float32, descending=True)
        assert srv.poll(rid, wait=True)[0] == capi.GS_OK
    assert same_bits(from_dev(d, np.float32), oracle.sort_keys(a, True))


def test_cancel_queued_request(ctx):
    n = 1 << 24
    reqs = [serving.DeviceRequest(serving.RequestSpec(n, np.uint64, None, 70 + i))
            for i in range(4)]
    with capi.Server(0, hbm_budget=1 << 30, max_request_keys=n, slots=1) as srv:
        ids = [r.submit(srv) for r in reqs]
        # one slot: the last request is still queued behind three long sorts
        assert srv.cancel(ids[-1]) == capi.GS_OK
        assert srv.poll(ids[-1], wait=True)[0] == capi.GS_ERR_CANCELLED
        assert srv.poll(ids[-1], wait=False)[0] == capi.GS_ERR_INVALID
        for i in ids[:-1]:
            assert srv.poll(i, wait=True)[0] == capi.GS_OK
        assert srv.cancel(ids[0]) == capi.GS_ERR_INVALID
    for r in reqs[:-1]:
        want = oracle.sort_keys(_bits(r.keys, np.uint64))
        assert same_bits(_bits(r.keys_out, np.uint64), want)


def test_queue_bound_and_errors(ctx):
    n = 1 << 25
    big = [serving.DeviceRequest(serving.RequestSpec(n, np.uint64, None, 80 + i))
           for i in range(6)]
    with capi.Server(0, hbm_budget=1 << 30, max_request_keys=n, slots=1, max_queue=2) as srv:
        ids, busy = [], 0
        for r in big:
            try:
                ids.append(r.submit(srv))
            except capi.GsError as e:
                assert e.status == capi.GS_ERR_BUSY
                busy += 1
        assert busy >= 1
        for i in ids:
            assert srv.poll(i, wait=True)[0] == capi.GS_OK
        small = to_dev(np.arange(10, dtype=np.uint32))
        out = empty_dev(10, np.uint32)
        with pytest.raises(capi.GsError) as e:
            srv.submit(small, out, key_dtype=np.uint32, n=0)
        assert e.value.status == capi.GS_ERR_EMPTY
        with pytest.raises(capi.GsError) as e:
            srv.submit(small, out, key_dtype=np.uint32, n=n + 1)
        assert e.value.status == capi.GS_ERR_TOO_LARGE
        host = np.arange(10, dtype=np.uint32)
        with pytest.raises(capi.GsError) as e:  # host memory without FLAG_HOST
            srv.submit(host, np.empty_like(host))
        assert e.value.status == capi.GS_ERR_INVALID
        assert srv.poll(123456789, wait=False)[0] == capi.GS_ERR_INVALID
    with capi.Server(0, hbm_budget=1 << 20, max_request_keys=1 << 20, slots=1) as srv:
        d = empty_dev(1 << 20, np.uint64)
        with pytest.raises(capi.GsError) as e:  # 8 MiB of scratch > 1 MiB arena
            srv.submit(d, d, key_dtype=np.uint64)
        assert e.value.status == capi.GS_ERR_OOM


def test_poisson_load_small(ctx):
    specs = serving.request_mix(60, lo_log2=10, hi_log2=20, seed=21)
    reqs = [serving.DeviceRequest(s) for s in specs]
    arr = serving.poisson_arrivals(len(reqs), rate_per_s=4000.0, seed=22)
    with capi.Server(0, hbm_budget=1 << 30, max_request_keys=1 << 20, slots=8) as srv:
        res = serving.run_served(srv, reqs, arr)
    assert res["requests"] == len(reqs)
    assert 0 < res["p50_ms"] <= res["p99_ms"] <= res["max_ms"]
    plain = serving.run_plain(ctx, reqs[:10], arr[:10])
    assert plain["requests"] == 10
    for r in reqs:
        want = oracle.sort_keys(_bits(r.keys, r.spec.key_dtype)) if r.vals is None else \
            oracle.sort_pairs(_bits(r.keys, r.spec.key_dtype), _bits(r.vals, np.uint32))[0]
        assert same_bits(_bits(r.keys_out, r.spec.key_dtype), want)


def test_small_requests_batched_in_one_launch(ctx):
    """Small device requests (keys only, <= 4096 keys) queued together run
    as one launch, one CTA each; interleaved key widths split the batches.
    Every output equals the oracle's."""
    rng = np.random.default_rng(17)
    kinds = [np.uint32, np.int32, np.float32, np.uint64, np.int64, np.float64]
    jobs = []
    with capi.Server(0, hbm_budget=256 << 20, max_request_keys=1 << 20, slots=2) as srv:
        for i in range(300):
            dt = kinds[int(rng.integers(len(kinds)))]
            n = int(rng.integers(1, 4097)) if i % 25 else 300000  # a few large ones
            a = datagen.host("uniform" if i % 3 else "distinct8", n, dt, seed=500 + i)
            desc = bool(i % 2)
            d_in = to_dev(a)
            d_out = d_in if i % 7 == 0 else empty_dev(n, dt)  # some in place
            rid = srv.submit(d_in, d_out, key_dtype=dt, descending=desc)
            jobs.append((rid, a, d_out, dt, desc))
        for rid, a, d_out, dt, desc in jobs:
            assert srv.poll(rid, wait=True)[0] == capi.GS_OK
        st = srv.stats()
        assert st["completed"] == len(jobs) and st["running"] == 0
    for rid, a, d_out, dt, desc in jobs:
        assert same_bits(from_dev(d_out, dt), oracle.sort_keys(a, desc)), (a.size, dt, desc)
