"""The synthetic inputs and the serving mix behave as the workloads state:
seeded and reproducible, NaN-free floats without -0.0, Zipf keys over 2^20
distinct values, segment lengths normalised to the requested total, and
the serving mix's sizes, type shares and arrival rate."""
import numpy as np
import pytest

from gpusort_gb300 import datagen, serving

DISTS = ["uniform", "normal", "zipf", "sorted", "reverse", "equal", "distinct8"]


@pytest.mark.parametrize("dist", DISTS)
@pytest.mark.parametrize("dtype", [np.uint32, np.int32, np.float32, np.uint64, np.int64,
                                   np.float64])
def test_host_inputs_are_seeded(dist, dtype):
    if dist == "normal" and np.dtype(dtype).kind != "f":
        pytest.skip("normal is a float distribution")
    a = datagen.host(dist, 5000, dtype, seed=11)
    b = datagen.host(dist, 5000, dtype, seed=11)
    assert a.dtype == np.dtype(dtype) and a.size == 5000
    assert np.array_equal(a.view(np.uint8), b.view(np.uint8))
    if dist not in ("equal",):
        c = datagen.host(dist, 5000, dtype, seed=12)
        assert not np.array_equal(a.view(np.uint8), c.view(np.uint8))


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_floats_have_no_nan_and_no_negative_zero(dtype):
    for dist in ("uniform", "normal", "zipf", "distinct8"):
        a = datagen.host(dist, 200_000, dtype, seed=3)
        assert not np.isnan(a).any()
        assert not np.any((a == 0) & np.signbit(a)), dist


def test_orders_and_value_counts():
    s = datagen.host("sorted", 10_000, np.uint32, seed=1)
    assert np.all(s[1:] >= s[:-1])
    r = datagen.host("reverse", 10_000, np.int64, seed=1)
    assert np.all(r[1:] <= r[:-1])
    assert np.unique(datagen.host("equal", 1000, np.uint64, seed=1)).size == 1
    assert np.unique(datagen.host("distinct8", 100_000, np.int32, seed=1)).size <= 8


def test_zipf_keys():
    """Zipf(1.1) ranks over 2^20 values: the most frequent key carries about
    1/zeta(1.1) of the mass, and the distinct keys spread over the range."""
    a = datagen.host("zipf", 1_000_000, np.uint64, seed=5)
    vals, counts = np.unique(a, return_counts=True)
    assert vals.size <= datagen.ZIPF_DISTINCT
    top = counts.max() / a.size
    ranks = np.arange(1, datagen.ZIPF_DISTINCT + 1, dtype=np.float64)
    want = 1.0 / np.sum(ranks ** -datagen.ZIPF_S)
    assert abs(top - want) < 0.01
    assert vals.max() > (1 << 62) and vals.min() < (1 << 62)  # spread, not clustered


def test_segment_offsets_normalised():
    off = datagen.segment_offsets(100_000, 16, 1 << 22, total=1 << 30, seed=8)
    lens = np.diff(off.astype(np.int64))
    assert off.size == 100_001 and off[0] == 0
    assert lens.min() >= 16
    assert abs(int(off[-1]) - (1 << 30)) / (1 << 30) < 0.01
    unscaled = datagen.segment_offsets(1000, 16, 1 << 22, seed=8)
    assert np.diff(unscaled.astype(np.int64)).max() <= (1 << 22)


def test_serving_mix_and_arrivals():
    specs = serving.request_mix(4000, seed=5)
    sizes = np.array([s.n for s in specs])
    assert sizes.min() >= 1 << 10 and sizes.max() <= 1 << 26
    # log-uniform: about half the requests below the geometric midpoint 2^18
    assert 0.45 < np.mean(sizes < (1 << 18)) < 0.55
    kinds = [(np.dtype(s.key_dtype).name, s.val_dtype is not None) for s in specs]
    share = {k: kinds.count(k) / len(kinds) for k in set(kinds)}
    assert abs(share[("uint32", False)] - 0.4) < 0.03
    assert abs(share[("uint64", False)] - 0.3) < 0.03
    assert abs(share[("float32", False)] - 0.2) < 0.03
    assert abs(share[("int64", True)] - 0.1) < 0.03
    assert len({s.seed for s in specs}) == len(specs)
    t = serving.poisson_arrivals(20_000, 1000.0, seed=6)
    assert np.all(np.diff(t) >= 0)
    assert abs(np.mean(np.diff(t)) - 1e-3) < 5e-5


def test_algorithmic_bytes_of_a_request():
    """Histogram read plus key-bits/8 passes reading and writing keys (and
    values): 36 B per 32-bit key, 136 per 64-bit key, 200 per 64-bit key
    with a 32-bit value."""
    S = serving.RequestSpec
    assert serving.bytes_alg(S(1, np.uint32, None, 0)) == 36
    assert serving.bytes_alg(S(1, np.uint64, None, 0)) == 136
    assert serving.bytes_alg(S(1, np.int64, np.uint32, 0)) == 200
    assert serving.bytes_alg(S(10, np.float32, None, 0)) == 360
