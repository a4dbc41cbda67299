"""Tuning table on the GPU: the table steers the pass shape and SampleSort
bucket count, explicit choices win, and tuned sorts stay bit-exact."""
import numpy as np
import pytest

from gpusort_gb300 import autotune, capi, datagen
from oracle import oracle
from tests._util import empty_dev, from_dev, same_bits, to_dev

pytestmark = pytest.mark.gpu


def test_table_drives_the_choice(ctx):
    try:
        ctx.set_tuning([
            {"key_dtype": "u32", "val_bytes": 0, "log2n_min": 0, "log2n_max": 19,
             "pass_shape": 1, "partitions": 16},
            {"key_dtype": "u32", "val_bytes": 0, "log2n_min": 20, "log2n_max": 63,
             "pass_shape": 2, "partitions": 128},
            {"key_dtype": "u64", "val_bytes": 4, "log2n_min": 0, "log2n_max": 63,
             "pass_shape": 1},
        ])
        assert ctx.choice(np.uint32, 0, 1000) == (1, 16)
        assert ctx.choice(np.uint32, 0, 1 << 20) == (2, 128)
        assert ctx.choice(np.uint64, 4, 1 << 25)[0] == 1
        # No entry: the defaults (the 256-thread tiles up to 2^18 keys).
        assert ctx.choice(np.int32, 0, 1000) == (1, 64)
        assert ctx.choice(np.int32, 0, 1 << 22) == (0, 64)
        ctx.debug_set(capi.DEBUG_PASS_SHAPE, 0)        # explicit shape wins
        assert ctx.choice(np.uint32, 0, 1000)[0] == 0
        ctx.debug_set(capi.DEBUG_PASS_SHAPE, 2**64 - 1)
        for n in (5000, (1 << 20) + 3):
            a = datagen.host("uniform", n, np.uint32, seed=n)
            d_in, d_out = to_dev(a), empty_dev(n, np.uint32)
            for algo in (capi.ALGO_RADIX, capi.ALGO_SAMPLE):
                st = ctx.sort_keys(d_in, d_out, dtype=np.uint32, algo=algo, flags=capi.FLAG_SYNC)
                assert st == capi.GS_OK, ctx.last_error()
                assert same_bits(from_dev(d_out, np.uint32), oracle.sort_keys(a))
    finally:
        ctx.set_tuning([])
        ctx.debug_set(capi.DEBUG_PASS_SHAPE, 2**64 - 1)
    assert ctx.choice(np.uint32, 0, 1000) == (1, 64)
    assert ctx.choice(np.uint32, 4, 1000) == (0, 64)  # pairs keep the 512-thread tiles


def test_quick_tune_round_trip(ctx, tmp_path):
    import torch
    try:
        doc = autotune.tune(ctx, cases=[("u32", None), ("u64", "u32")], log2ns=(14, 18), reps=1,
                            partitions=(16, 64))
        assert len(doc["entries"]) == 4
        path = autotune.save(doc, tmp_path / "tuning.json")
        autotune.apply(ctx, path)
        for e in doc["entries"]:
            lg = (e["log2n_min"] + e["log2n_max"]) // 2 if e["log2n_max"] < 63 else 20
            shape, parts = ctx.choice(e["key_dtype"] == "u32" and np.uint32 or np.uint64,
                                      e["val_bytes"], 1 << lg)
            assert shape == e["pass_shape"]
        a = datagen.host("zipf", 300001, np.uint64, seed=4)
        v = np.arange(a.size, dtype=np.uint32)
        ko, vo = empty_dev(a.size, np.uint64), empty_dev(a.size, np.uint32)
        st = ctx.sort_pairs(to_dev(a), to_dev(v), ko, vo, key_dtype=np.uint64,
                            val_dtype=np.uint32, stable=True, flags=capi.FLAG_SYNC)
        assert st == capi.GS_OK, ctx.last_error()
        wk, wv = oracle.sort_pairs(a, v, False, True)
        assert same_bits(from_dev(ko, np.uint64), wk) and same_bits(from_dev(vo, np.uint32), wv)
    finally:
        ctx.set_tuning([])
        ctx.set_stream(torch.cuda.current_stream().cuda_stream)
