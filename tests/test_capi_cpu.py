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
