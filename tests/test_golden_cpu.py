"""Pin the CPU oracle to the reference: every golden fixture in tests/golden
was produced by the reference's own HykSort / SampleSort / HyperQuickSort
(built from its sources by oracle/ref, run on thread-ranks; see
tests/golden/make_golden.py). The oracle must reproduce each one exactly."""
from pathlib import Path

import numpy as np
import pytest

from oracle import oracle

GOLDEN = Path(__file__).resolve().parent / "golden"
KEYS = sorted(GOLDEN.glob("keys_*.npz"))
PAIRS = sorted(GOLDEN.glob("pairs_*.npz"))
KATS = sorted(GOLDEN.glob("kat_*.npz"))


def test_fixture_set_is_complete():
    assert len(KEYS) == 90 and len(PAIRS) == 36 and len(KATS) >= 20


@pytest.mark.parametrize("path", KEYS, ids=lambda p: p.stem)
def test_oracle_matches_reference_keys(path):
    f = np.load(path)
    got = oracle.sort_keys(f["input"], bool(f["desc"]))
    assert np.array_equal(got.view(np.uint8), f["output"].view(np.uint8))
    assert int(f["rank_sizes"].sum()) == f["input"].size


@pytest.mark.parametrize("path", PAIRS, ids=lambda p: p.stem)
def test_oracle_matches_reference_pairs(path):
    f = np.load(path)
    ko, vo = oracle.sort_pairs(f["keys"], f["vals"], bool(f["desc"]))
    assert np.array_equal(ko, f["keys_out"]) and np.array_equal(vo, f["vals_out"])


@pytest.mark.parametrize("path", KATS, ids=lambda p: p.stem)
def test_oracle_known_answers(path):
    f = np.load(path)
    assert np.array_equal(oracle.sort_keys(f["input"], bool(f["desc"])), f["output"])


@pytest.mark.parametrize("path", KEYS[::9], ids=lambda p: p.stem)
def test_hyksort_port_matches_reference(path):
    f = np.load(path)
    got = oracle.hyksort_cpu(f["input"], p=int(f["p"]), k=int(f["k"]), threads=2,
                             descending=bool(f["desc"]))
    assert np.array_equal(got, f["output"])
