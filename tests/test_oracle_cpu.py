"""The CPU oracle against itself and numpy, and the HykSort port against the
oracle: the checker has to be right before the GPU path is checked with it."""
import numpy as np
import pytest

from gpusort_gb300 import datagen
from oracle import oracle

DTYPES = [np.uint32, np.int32, np.float32, np.uint64, np.int64, np.float64]


@pytest.mark.parametrize("dtype", DTYPES)
def test_sort_keys_matches_numpy(dtype):
    for dist in ("uniform", "zipf", "distinct8", "equal", "reverse"):
        a = datagen.host(dist, 50000, dtype, seed=4)
        s = oracle.sort_keys(a)
        assert np.array_equal(s, np.sort(a, kind="stable"))
        assert np.array_equal(oracle.sort_keys(a, True), s[::-1])


def test_pairs_lexicographic_and_stable():
    rng = np.random.default_rng(0)
    k = rng.integers(0, 40, 20000).astype(np.int64)
    v = rng.integers(-50, 50, 20000).astype(np.int32)
    ko, vo = oracle.sort_pairs(k, v)
    idx = np.lexsort((v, k))
    assert np.array_equal(ko, k[idx]) and np.array_equal(vo, v[idx])
    ko, vo = oracle.sort_pairs(k, v, descending=True)
    assert np.array_equal(ko, k[idx][::-1]) and np.array_equal(vo, v[idx][::-1])
    i = np.arange(k.size, dtype=np.uint32)
    st = np.argsort(k, kind="stable")
    assert np.array_equal(oracle.sort_pairs(k, i, stable=True)[1], st)
    assert np.array_equal(oracle.sort_pairs(k, i, descending=True, stable=True)[1], st[::-1])


@pytest.mark.parametrize("p,k", [(4, 4), (8, 2), (16, 4), (2, 2), (1, 4), (8, 8), (6, 4), (4, 3)])
@pytest.mark.parametrize("dtype", [np.uint32, np.float64, np.int64])
def test_hyksort_port_equals_sorted(p, k, dtype):
    for dist in ("uniform", "distinct8", "equal", "zipf"):
        a = datagen.host(dist, 100003, dtype, seed=p * 31 + k)
        for desc in (False, True):
            got = oracle.hyksort_cpu(a, p=p, k=k, threads=2, seed=1, descending=desc)
            assert np.array_equal(got, oracle.sort_keys(a, desc)), (p, k, dist, desc)
