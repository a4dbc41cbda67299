"""Batched (segmented) sorting through the C ABI: every segment sorted on
its own, compared bit for bit with the oracle's per-segment std::sort."""
import numpy as np
import pytest

from gpusort_gb300 import capi, datagen
from oracle import oracle
from tests._util import empty_dev, from_dev, same_bits, to_dev

pytestmark = pytest.mark.gpu


def _layouts():
    rng = np.random.default_rng(5)
    yield "tiny", np.concatenate([[0], np.cumsum(rng.integers(0, 40, 3000))]).astype(np.uint64)
    yield "mixed", datagen.segment_offsets(400, 1, 60000, seed=2)
    yield "empty+singletons", np.array([0, 0, 1, 1, 2, 2, 5, 5, 100, 100, 5000, 5001],
                                       np.uint64)
    yield "one_large", np.array([0, 300001], np.uint64)
    yield "boundaries", np.cumsum([0, 4095, 4096, 4097, 6143, 6144, 6145, 8192, 1, 12289]
                                  ).astype(np.uint64)
    yield "loguniform", datagen.segment_offsets(2000, 16, 1 << 17, total=1 << 22, seed=9)
    # groups made only of segments of <= 32 keys take the warp bitonic path
    yield "all_tiny", np.concatenate([[0], np.cumsum(rng.integers(1, 33, 5000))]).astype(np.uint64)
    runs = []
    for r in range(60):
        runs += list(rng.integers(1, 33, int(rng.integers(1, 300))))
        runs.append(int(rng.integers(33, 9000)))
    yield "tiny_runs", np.concatenate([[0], np.cumsum(runs)]).astype(np.uint64)


@pytest.mark.parametrize("dtype", [np.uint32, np.int32, np.float32, np.uint64, np.int64,
                                   np.float64])
def test_segmented_matches_oracle(ctx, dtype):
    for name, off in _layouts():
        n = int(off[-1])
        a = datagen.host("uniform" if name != "mixed" else "distinct8", n, dtype, seed=n)
        d_off = to_dev(off.view(np.int64))
        for desc in (False, True):
            d_in, d_out = to_dev(a), empty_dev(n, a.dtype)
            st = ctx.segmented_sort_keys(d_in, d_out, d_off, off.size - 1, dtype=a.dtype,
                                         descending=desc)
            assert st == capi.GS_OK, ctx.last_error()
            want = oracle.segmented_sort_keys(a, off, desc)
            assert same_bits(from_dev(d_out, a.dtype), want), (name, desc)


def test_segmented_in_place_and_host_pointers(ctx):
    off = datagen.segment_offsets(300, 1, 30000, seed=4)
    n = int(off[-1])
    a = datagen.host("uniform", n, np.uint32, seed=1)
    d = to_dev(a)
    st = ctx.segmented_sort_keys(d, d, to_dev(off.view(np.int64)), off.size - 1, dtype=np.uint32)
    assert st == capi.GS_OK, ctx.last_error()
    want = oracle.segmented_sort_keys(a, off)
    assert same_bits(from_dev(d, np.uint32), want)
    h = a.copy()
    st = ctx.segmented_sort_keys(h, h, off, off.size - 1,
                                 flags=capi.FLAG_HOST | capi.FLAG_OFFSETS_HOST)
    assert st == capi.GS_OK, ctx.last_error()
    assert same_bits(h, want)


def test_plan_runs_twice_and_in_a_cuda_graph(ctx):
    import torch
    off = datagen.segment_offsets(1000, 16, 1 << 15, total=1 << 21, seed=3)
    n = int(off[-1])
    a = datagen.host("uniform", n, np.uint32, seed=7)
    want = oracle.segmented_sort_keys(a, off)
    plan = ctx.segmented_plan(np.uint32, n, off)
    try:
        d_in, d_out = to_dev(a), empty_dev(n, np.uint32)
        for _ in range(2):
            d_out.zero_()
            assert ctx.segmented_run(plan, d_in, d_out) == capi.GS_OK, ctx.last_error()
            ctx.synchronize()
            assert same_bits(from_dev(d_out, np.uint32), want)
        s = torch.cuda.Stream()
        ctx.set_stream(s.cuda_stream)
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g, stream=s):
            st = ctx.segmented_run(plan, d_in, d_out)
        assert st == capi.GS_OK, ctx.last_error()
        for _ in range(2):
            d_out.zero_()
            torch.cuda.synchronize()
            g.replay()
            torch.cuda.synchronize()
            assert same_bits(from_dev(d_out, np.uint32), want)
    finally:
        ctx.set_stream(torch.cuda.current_stream().cuda_stream or None)
        ctx.segmented_destroy(plan)
