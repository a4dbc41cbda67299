"""CPU-only checks of the C ABI library: it builds, loads, and exports every
function include/gpusort_gb300.h declares. No compute call is made."""
import ctypes as C
import re
from pathlib import Path

import pytest

from gpusort_gb300 import capi

ROOT = Path(__file__).resolve().parents[1]


def _declared_functions(header: Path) -> list[str]:
    text = header.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(gs_[a-z_0-9]+)\s*\(", text)))


def test_library_exports_every_declared_symbol(built_lib):
    L = capi.load()
    declared = _declared_functions(ROOT / "include" / "gpusort_gb300.h")
    assert declared, "no declarations parsed"
    missing = [f for f in declared if not hasattr(L, f)]
    assert not missing, missing
    assert sorted(capi.EXPORTED) == declared


def test_version_and_no_device_behaviour(built_lib):
    L = capi.load()
    assert L.gs_version() == 0x000100
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    assert L.gs_device_count() == 0
    assert L.gs_ctx_create(0, 0) is None
    assert b"No CUDA-capable" in L.gs_last_global_error()


def test_null_context_is_rejected(built_lib):
    L = capi.load()
    o = capi.gs_opts()
    assert L.gs_sort_keys(None, capi.GS_U32, None, None, 10, 0, o) == capi.GS_ERR_INVALID
    assert L.gs_ctx_synchronize(None) == capi.GS_ERR_INVALID


def test_server_needs_a_device(built_lib):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    L = capi.load()
    o = capi.gs_server_opts(1 << 20, 0, 2, 0)
    assert L.gs_server_create(0, o) is None
    assert b"no such CUDA device" in L.gs_last_global_error()
    with pytest.raises(capi.GsError):
        capi.Server(0)
    stats = capi.gs_server_stats()
    assert L.gs_server_get_stats(None, stats, 0) == capi.GS_ERR_INVALID
    assert L.gs_server_poll(None, 1, 0, None) == capi.GS_ERR_INVALID
    assert L.gs_server_cancel(None, 1) == capi.GS_ERR_INVALID
    rid = C.c_uint64()
    assert L.gs_server_submit(None, capi.GS_U32, 0, 0, None, None, None, None, 10, 0,
                              rid) == capi.GS_ERR_INVALID
    L.gs_server_destroy(None)


def _header_constants(header: Path) -> dict:
    """Every `NAME = value` enumerator and `#define NAME value` of the
    header, comments removed."""
    text = re.sub(r"/\*.*?\*/", "", header.read_text(), flags=re.S)
    consts = {}
    for name, val in re.findall(r"\b(GS_[A-Z0-9_]+)\s*=\s*(0x[0-9a-fA-F]+|\d+)", text):
        consts[name] = int(val, 0)
    for name, val in re.findall(r"#define\s+(GS_[A-Z0-9_]+)\s+(0x[0-9a-fA-F]+|\d+)u?", text):
        consts[name] = int(val, 0)
    return consts


def test_python_mirror_constants_match_the_header():
    """The ctypes mirror uses the header's status codes, key types, flags,
    strategies and debug keys."""
    h = _header_constants(ROOT / "include" / "gpusort_gb300.h")
    pairs = {
        "GS_OK": capi.GS_OK, "GS_ERR_EMPTY": capi.GS_ERR_EMPTY, "GS_ERR_OOM": capi.GS_ERR_OOM,
        "GS_ERR_BAD_DTYPE": capi.GS_ERR_BAD_DTYPE, "GS_ERR_TIMEOUT": capi.GS_ERR_TIMEOUT,
        "GS_ERR_CUDA": capi.GS_ERR_CUDA, "GS_ERR_INVALID": capi.GS_ERR_INVALID,
        "GS_ERR_NO_DEVICE": capi.GS_ERR_NO_DEVICE, "GS_ERR_TOO_LARGE": capi.GS_ERR_TOO_LARGE,
        "GS_ERR_BUSY": capi.GS_ERR_BUSY, "GS_ERR_CANCELLED": capi.GS_ERR_CANCELLED,
        "GS_U32": capi.GS_U32, "GS_I32": capi.GS_I32, "GS_F32": capi.GS_F32,
        "GS_U64": capi.GS_U64, "GS_I64": capi.GS_I64, "GS_F64": capi.GS_F64,
        "GS_FLAG_DESCENDING": capi.FLAG_DESCENDING, "GS_FLAG_PAIRS_STABLE": capi.FLAG_PAIRS_STABLE,
        "GS_FLAG_HOST": capi.FLAG_HOST, "GS_FLAG_SYNC": capi.FLAG_SYNC,
        "GS_FLAG_OFFSETS_HOST": capi.FLAG_OFFSETS_HOST,
        "GS_ALGO_AUTO": capi.ALGO_AUTO, "GS_ALGO_RADIX": capi.ALGO_RADIX,
        "GS_ALGO_SAMPLE": capi.ALGO_SAMPLE, "GS_ALGO_HYK": capi.ALGO_HYK,
        "GS_DEBUG_SPIN_LIMIT": capi.DEBUG_SPIN_LIMIT,
        "GS_DEBUG_INJECT_STALL": capi.DEBUG_INJECT_STALL, "GS_DEBUG_BUDGET": capi.DEBUG_BUDGET,
        "GS_DEBUG_PASS_SHAPE": capi.DEBUG_PASS_SHAPE,
        "GS_DEBUG_HOST_GROUPS": capi.DEBUG_HOST_GROUPS,
        "GS_DEBUG_HOST_CHUNKED": capi.DEBUG_HOST_CHUNKED,
    }
    missing = [k for k in pairs if k not in h]
    assert not missing, missing
    wrong = {k: (h[k], v) for k, v in pairs.items() if h[k] != v}
    assert not wrong, wrong
