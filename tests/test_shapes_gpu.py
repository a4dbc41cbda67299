"""The SampleSort and HykSort shapes of the engine (gs_opts.algo) give the
reference's bytes: splitters from an oversampled sample + bucket scatter +
per-bucket sort (include/helpers/samplesort_helper.h:390-565), and local
sorts + merge-path merge tree (include/helpers/hyksort_helper.h:307-633)."""
import numpy as np
import pytest

from gpusort_gb300 import capi, datagen
from oracle import oracle
from tests._util import empty_dev, from_dev, same_bits, to_dev

pytestmark = pytest.mark.gpu


def _run(ctx, a, algo, desc=False, in_place=False, **kw):
    d_in = to_dev(a)
    d_out = d_in if in_place else empty_dev(a.size, a.dtype)
    st = ctx.sort_keys(d_in, d_out, dtype=a.dtype, descending=desc, flags=capi.FLAG_SYNC,
                       algo=algo, **kw)
    assert st == capi.GS_OK, ctx.last_error()
    return from_dev(d_out, a.dtype)


@pytest.mark.parametrize("dtype", [np.uint32, np.float32, np.int64, np.float64])
@pytest.mark.parametrize("dist", ["uniform", "zipf", "distinct8", "equal", "sorted", "reverse"])
def test_sample_sort_shape(ctx, dtype, dist):
    for n, p, os in ((5000, 2, 1), (100003, 64, 32), ((1 << 21) + 9, 64, 32), (300007, 256, 8),
                     (70001, 7, 5)):
        a = datagen.host(dist, n, dtype, seed=n + p)
        for desc in (False, True):
            got = _run(ctx, a, capi.ALGO_SAMPLE, desc, in_place=(n == 70001), partitions=p,
                       oversample=os, seed=n)
            assert same_bits(got, oracle.sort_keys(a, desc)), (n, p, os, desc)


@pytest.mark.parametrize("dtype", [np.uint32, np.int32, np.uint64, np.float64])
@pytest.mark.parametrize("dist", ["uniform", "zipf", "distinct8", "equal", "reverse"])
def test_hyk_sort_shape(ctx, dtype, dist):
    for n, p, k in ((4096, 4, 4), (4 << 20, 4, 4), (100003, 8, 2), (250001, 64, 4),
                    (123457, 6, 4), (99991, 16, 3)):
        a = datagen.host(dist, n, dtype, seed=n + p)
        for desc in (False, True):
            got = _run(ctx, a, capi.ALGO_HYK, desc, in_place=(p == 8), partitions=p, k_way=k)
            assert same_bits(got, oracle.sort_keys(a, desc)), (n, p, k, desc)


@pytest.mark.parametrize("p", [4, 16, 64])
@pytest.mark.parametrize("k", [2, 4, 8])
@pytest.mark.parametrize("dtype", [np.uint32, np.float64])
def test_hyk_rounds_p_by_k(ctx, p, k, dtype):
    """log_k(p) rounds of splitter selection, cuts and one k-way merge each
    (k reduced to the group size in the last round when k does not divide
    the group evenly in powers)."""
    for dist in ("uniform", "zipf", "distinct8", "equal", "sorted"):
        for n in (p * 3 + 1, 200_003):
            a = datagen.host(dist, n, dtype, seed=n + p * 7 + k)
            for desc in (False, True):
                got = _run(ctx, a, capi.ALGO_HYK, desc, in_place=desc, partitions=p,
                           k_way=k, seed=p + k)
                assert same_bits(got, oracle.sort_keys(a, desc)), (dist, n, p, k, desc)


def test_hyk_large_groups(ctx):
    """256 partitions with 16-way rounds, and 512 partitions 2-way."""
    for p, k, n in ((256, 16, 1 << 20), (512, 2, 300_001)):
        a = datagen.host("uniform", n, np.uint64, seed=p)
        got = _run(ctx, a, capi.ALGO_HYK, False, partitions=p, k_way=k)
        assert same_bits(got, oracle.sort_keys(a)), (p, k)


def test_shapes_on_reference_rank_config(ctx):
    """The reference's CPU case: 4 ranks x 2^20 uint32, HykSort k=4."""
    a = np.concatenate([datagen.host("uniform", 1 << 20, np.uint32, seed=0x67707573 + r)
                        for r in range(4)])
    want = oracle.sort_keys(a)
    for algo in (capi.ALGO_HYK, capi.ALGO_SAMPLE, capi.ALGO_RADIX):
        assert same_bits(_run(ctx, a, algo, partitions=4, k_way=4), want)
