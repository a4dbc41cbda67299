"""ctypes binding of the CPU ORACLE (gs_oracle.cc). TEST INFRASTRUCTURE.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline /
reference arm may import this module, and only as the checker or as the
timed CPU baseline. Nothing in the gpusort_gb300 package imports it.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "libgs_oracle.so"

_CODES = {
    np.dtype(np.uint32): 0, np.dtype(np.int32): 1, np.dtype(np.float32): 2,
    np.dtype(np.uint64): 3, np.dtype(np.int64): 4, np.dtype(np.float64): 5,
}
_lib = None


def build() -> Path:
    """Compile the oracle with make (g++, C++20, no other dependency)."""
    r = subprocess.run(["make", "-s", "-C", str(HERE), "libgs_oracle.so"],
                       capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{r.stdout}\n{r.stderr}")
    return LIB


def _load():
    global _lib
    if _lib is None:
        if not LIB.exists():
            build()
        L = C.CDLL(str(LIB))
        vp, u64, i32 = C.c_void_p, C.c_uint64, C.c_int
        L.oracle_sort_keys.argtypes = [i32, vp, vp, u64, i32, i32]
        L.oracle_sort_pairs.argtypes = [i32, i32, vp, vp, vp, vp, u64, i32, i32, i32]
        L.oracle_hyksort_cpu.argtypes = [i32, vp, u64, i32, i32, i32, u64, i32]
        L.oracle_segmented_sort_keys.argtypes = [i32, vp, vp, u64, vp, C.c_uint32, i32, i32]
        for f in ("oracle_sort_keys", "oracle_sort_pairs", "oracle_hyksort_cpu",
                  "oracle_segmented_sort_keys"):
            getattr(L, f).restype = i32
        _lib = L
    return _lib


def _threads(threads: int | None) -> int:
    """Worker threads of one oracle call: every host core unless given."""
    return max(1, int(threads if threads is not None else (os.cpu_count() or 1)))


def sort_keys(keys: np.ndarray, descending: bool = False, threads: int | None = None) -> np.ndarray:
    """Globally sorted copy under std::less / std::greater."""
    a = np.ascontiguousarray(keys)
    out = np.empty_like(a)
    rc = _load().oracle_sort_keys(_CODES[a.dtype], a.ctypes.data, out.ctypes.data, a.size,
                                  int(descending), _threads(threads))
    assert rc == 0
    return out


def sort_pairs(keys: np.ndarray, vals: np.ndarray, descending: bool = False,
               stable: bool = False, threads: int | None = None) -> tuple[np.ndarray, np.ndarray]:
    """(key, value) order of the reference's CPU pair path, or stable-by-key."""
    k = np.ascontiguousarray(keys)
    v = np.ascontiguousarray(vals)
    ko, vo = np.empty_like(k), np.empty_like(v)
    rc = _load().oracle_sort_pairs(_CODES[k.dtype], _CODES[v.dtype], k.ctypes.data,
                                   v.ctypes.data, ko.ctypes.data, vo.ctypes.data, k.size,
                                   int(descending), int(stable), _threads(threads))
    assert rc == 0
    return ko, vo


def segmented_sort_keys(keys: np.ndarray, offsets: np.ndarray,
                        descending: bool = False, threads: int | None = None) -> np.ndarray:
    """Each segment [offsets[s], offsets[s+1]) sorted on its own."""
    a = np.ascontiguousarray(keys)
    off = np.ascontiguousarray(offsets, dtype=np.uint64)
    out = np.empty_like(a)
    rc = _load().oracle_segmented_sort_keys(_CODES[a.dtype], a.ctypes.data, out.ctypes.data,
                                            a.size, off.ctypes.data, off.size - 1, int(descending),
                                            _threads(threads))
    assert rc == 0
    return out


def hyksort_cpu(keys: np.ndarray, p: int = 4, k: int = 4, threads: int | None = None,
                seed: int = 0, descending: bool = False) -> np.ndarray:
    """The reference's CPU HykSort restated on p thread-ranks; returns the
    concatenation of the ranks' outputs (in place on a copy)."""
    a = np.ascontiguousarray(keys).copy()
    if threads is None:
        threads = max(1, (os.cpu_count() or 4) // p)
    rc = _load().oracle_hyksort_cpu(_CODES[a.dtype], a.ctypes.data, a.size, p, k, threads,
                                    seed, int(descending))
    if rc == -2:  # p or k not a power of two: the reference runs SampleSort
        return sort_keys(keys, descending)
    assert rc == 0, rc
    return a
