"""Tuning table: the engine's JSON reader and the tuner's size ranges (no GPU)."""
import json

import pytest

from gpusort_gb300 import autotune, capi


def test_parse_entries_strings_numbers_and_extra_keys(built_lib):
    doc = {"device": "x", "entries": [
        {"key_dtype": "u32", "val_bytes": 0, "log2n_min": 0, "log2n_max": 22, "pass_shape": 1,
         "partitions": 32, "threads": 256, "items_per_thread": 20},
        {"key_dtype": 3, "val_bytes": 4, "log2n_min": 23, "log2n_max": 63, "pass_shape": -1},
    ], "measured": [{"shape_ms": [1.5, 2.25e-1], "note": 'a } brace " quote'}]}
    got = capi.tuning_parse(json.dumps(doc))
    assert got == [
        {"key_dtype": 0, "val_bytes": 0, "log2n_min": 0, "log2n_max": 22, "pass_shape": 1,
         "partitions": 32},
        {"key_dtype": 3, "val_bytes": 4, "log2n_min": 23, "log2n_max": 63, "pass_shape": -1,
         "partitions": 0},
    ]
    assert capi.tuning_parse("[]") == []
    assert capi.tuning_parse('{"entries": []}') == []


@pytest.mark.parametrize("bad", [
    '{"entries": [{"key_dtype": "u16"}]}',                      # unknown type
    '{"entries": [{"key_dtype": "u32", "pass_shape": 7}]}',    # no such shape
    '{"entries": [{"key_dtype": "u32", "val_bytes": 2}]}',     # payload width
    '{"entries": [{"key_dtype": "u32", "log2n_min": 9, "log2n_max": 3}]}',
    '{"entries": [{"key_dtype": "u32", "partitions": 1}]}',
    '{"entries": [{"key_dtype": "u32", "pass_shape": 0.5}]}',
    '{"entries": [{"key_dtype": "u32"}',                        # truncated
    '{"entries": [{"key_dtype": "u32"}]} trailing',
    '',
])
def test_parse_rejects(built_lib, bad):
    assert capi.tuning_parse(bad) is None


def test_pass_shapes_describe_threads_and_items(built_lib):
    for kb in (4, 8):
        for vb in (0, 4, 8):
            shapes = capi.pass_shapes(kb, vb)
            assert len(shapes) == capi.load().gs_pass_shape_count() >= 2
            for t, it in shapes:
                assert t in (256, 384, 512) and 1 <= it <= 32
    L = capi.load()
    assert L.gs_pass_shape_info(2, 0, 0, None, None) == capi.GS_ERR_INVALID
    assert L.gs_pass_shape_info(4, 0, 99, None, None) == capi.GS_ERR_INVALID


def test_tuner_ranges_cover_all_sizes():
    for sizes in ([20], [16, 20, 24, 27], [10, 30]):
        r = autotune._ranges(sizes)
        assert r[0][0] == 0 and r[-1][1] == 63
        for (a, b), (c, d) in zip(r, r[1:]):
            assert c == b + 1 and a <= b
        for (lo, hi), lg in zip(r, sizes):
            assert lo <= lg <= hi


def test_context_calls_need_a_context(built_lib):
    L = capi.load()
    e = capi.gs_tuning_entry(0, 0, 0, 63, 0, 0)
    assert L.gs_ctx_set_tuning(None, e, 1) == capi.GS_ERR_INVALID
    assert L.gs_ctx_load_tuning(None, b"/nonexistent") == capi.GS_ERR_INVALID
    assert L.gs_ctx_choice(None, 0, 0, 10, None, None) == capi.GS_ERR_INVALID
