"""The GPU engine against the reference's own outputs (tests/golden, made by
tests/golden/make_golden.py from the reference's CPU HykSort / SampleSort /
HyperQuickSort), bit for bit, through the C ABI."""
from pathlib import Path

import numpy as np
import pytest

from gpusort_gb300 import capi
from tests._util import empty_dev, from_dev, same_bits, to_dev

pytestmark = pytest.mark.gpu
GOLDEN = Path(__file__).resolve().parent / "golden"


@pytest.mark.parametrize("path", sorted(GOLDEN.glob("keys_*.npz")) + sorted(GOLDEN.glob("kat_*.npz")),
                         ids=lambda p: p.stem)
def test_engine_matches_reference_keys(ctx, path):
    f = np.load(path)
    a = f["input"]
    d_in, d_out = to_dev(a), empty_dev(a.size, a.dtype)
    st = ctx.sort_keys(d_in, d_out, dtype=a.dtype, descending=bool(f["desc"]),
                       flags=capi.FLAG_SYNC)
    assert st == capi.GS_OK, ctx.last_error()
    assert same_bits(from_dev(d_out, a.dtype), f["output"])


@pytest.mark.parametrize("path", sorted(GOLDEN.glob("pairs_*.npz")), ids=lambda p: p.stem)
def test_engine_matches_reference_pairs(ctx, path):
    f = np.load(path)
    k, v = f["keys"], f["vals"]
    dk, dv = to_dev(k), to_dev(v)
    ok, ov = empty_dev(k.size, k.dtype), empty_dev(v.size, v.dtype)
    st = ctx.sort_pairs(dk, dv, ok, ov, key_dtype=k.dtype, val_dtype=v.dtype,
                        descending=bool(f["desc"]), flags=capi.FLAG_SYNC)
    assert st == capi.GS_OK, ctx.last_error()
    assert same_bits(from_dev(ok, k.dtype), f["keys_out"])
    assert same_bits(from_dev(ov, v.dtype), f["vals_out"])
