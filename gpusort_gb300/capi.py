"""ctypes binding of the engine's C ABI (include/gpusort_gb300.h).

The shared library is built in-tree (``gpusort_gb300/_lib``) by
``gpusort_gb300._build``. Loading fails loudly when it is missing: there is
no CPU fallback anywhere in the package.
"""
from __future__ import annotations

import ctypes as C
import threading
from pathlib import Path

import numpy as np

_LIB_PATH = Path(__file__).resolve().parent / "_lib" / "libgpusort_gb300.so"

# gs_status
GS_OK = 0
GS_ERR_EMPTY = 1
GS_ERR_OOM = 2
GS_ERR_BAD_DTYPE = 3
GS_ERR_TIMEOUT = 4
GS_ERR_CUDA = 5
GS_ERR_INVALID = 6
GS_ERR_NO_DEVICE = 7
GS_ERR_TOO_LARGE = 8
GS_ERR_BUSY = 9
GS_ERR_CANCELLED = 10

# gs_dtype
GS_U32, GS_I32, GS_F32, GS_U64, GS_I64, GS_F64 = range(6)

FLAG_DESCENDING = 0x1
FLAG_PAIRS_STABLE = 0x2
FLAG_HOST = 0x4
FLAG_SYNC = 0x8
FLAG_OFFSETS_HOST = 0x10

ALGO_AUTO, ALGO_RADIX, ALGO_SAMPLE, ALGO_HYK = range(4)

DEBUG_SPIN_LIMIT = 1
DEBUG_INJECT_STALL = 2
DEBUG_BUDGET = 3
DEBUG_PASS_SHAPE = 4
DEBUG_HOST_GROUPS = 5
DEBUG_HOST_CHUNKED = 6

# Every symbol include/gpusort_gb300.h declares (checked by the CPU tests).
EXPORTED = [
    "gs_version", "gs_device_count", "gs_ctx_create", "gs_ctx_destroy",
    "gs_ctx_set_stream", "gs_ctx_synchronize", "gs_last_error",
    "gs_last_global_error", "gs_sort_keys", "gs_sort_pairs",
    "gs_segmented_sort_keys", "gs_gather", "gs_phase_times",
    "gs_ctx_set_timing", "gs_kernel_times", "gs_debug_set", "gs_sort_keys_noalloc",
    "gs_segmented_plan_create", "gs_segmented_plan_run", "gs_segmented_plan_destroy",
    "gs_segmented_layout",
    "gs_server_create", "gs_server_destroy", "gs_server_submit", "gs_server_poll",
    "gs_server_cancel", "gs_server_get_stats",
    "gs_pass_shape_count", "gs_pass_shape_info", "gs_ctx_set_tuning", "gs_tuning_parse",
    "gs_ctx_load_tuning", "gs_ctx_choice",
    "gs_file_count", "gs_file_read", "gs_file_write", "gs_partitions_read",
    "gs_partitions_write", "gs_partition_block",
]

_NP_DTYPE = {
    np.dtype(np.uint32): GS_U32, np.dtype(np.int32): GS_I32, np.dtype(np.float32): GS_F32,
    np.dtype(np.uint64): GS_U64, np.dtype(np.int64): GS_I64, np.dtype(np.float64): GS_F64,
}


class gs_opts(C.Structure):
    _fields_ = [("algo", C.c_uint32), ("partitions", C.c_uint32), ("k_way", C.c_uint32),
                ("oversample", C.c_uint32), ("seed", C.c_uint64)]


class gs_tuning_entry(C.Structure):
    _fields_ = [("key_dtype", C.c_int32), ("val_bytes", C.c_int32), ("log2n_min", C.c_uint32),
                ("log2n_max", C.c_uint32), ("pass_shape", C.c_int32), ("partitions", C.c_uint32)]


DTYPE_NAMES = ["u32", "i32", "f32", "u64", "i64", "f64"]


class gs_server_opts(C.Structure):
    _fields_ = [("hbm_budget", C.c_uint64), ("max_request_keys", C.c_uint64),
                ("slots", C.c_uint32), ("max_queue", C.c_uint32)]


class gs_server_stats(C.Structure):
    _fields_ = [("completed", C.c_uint64), ("keys_done", C.c_uint64), ("queued", C.c_uint64),
                ("running", C.c_uint64), ("arena_used", C.c_uint64), ("arena_peak", C.c_uint64),
                ("p50_ms", C.c_double), ("p99_ms", C.c_double), ("mean_ms", C.c_double),
                ("max_ms", C.c_double)]


class GsError(RuntimeError):
    """A non-OK gs_status, with the engine's message."""

    def __init__(self, status: int, message: str):
        super().__init__(f"gs_status {status}: {message}")
        self.status = status
        self.message = message


_lib = None
_lock = threading.Lock()


def lib_path() -> Path:
    return _LIB_PATH


def load() -> C.CDLL:
    """Load the engine library (built in-tree). Raises if it is missing."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not _LIB_PATH.exists():
            raise RuntimeError(
                f"gpusort_gb300 native library not built: {_LIB_PATH} is missing "
                "(run gpusort_gb300._build.build())")
        L = C.CDLL(str(_LIB_PATH))
        vp, u64, u32, i32 = C.c_void_p, C.c_uint64, C.c_uint32, C.c_int
        L.gs_version.restype = u32
        L.gs_device_count.restype = i32
        L.gs_ctx_create.argtypes = [i32, u64]
        L.gs_ctx_create.restype = vp
        L.gs_ctx_destroy.argtypes = [vp]
        L.gs_ctx_destroy.restype = None
        L.gs_ctx_set_stream.argtypes = [vp, vp]
        L.gs_ctx_synchronize.argtypes = [vp]
        L.gs_last_error.argtypes = [vp]
        L.gs_last_error.restype = C.c_char_p
        L.gs_last_global_error.restype = C.c_char_p
        L.gs_sort_keys.argtypes = [vp, i32, vp, vp, u64, u32, C.POINTER(gs_opts)]
        L.gs_sort_pairs.argtypes = [vp, i32, i32, vp, vp, vp, vp, u64, u32, C.POINTER(gs_opts)]
        L.gs_segmented_sort_keys.argtypes = [vp, i32, vp, vp, u64, vp, u32, u32]
        L.gs_gather.argtypes = [vp, vp, vp, u64, u32, vp, u32]
        L.gs_phase_times.argtypes = [vp, C.POINTER(C.c_char_p), C.POINTER(C.c_double), i32]
        L.gs_phase_times.restype = i32
        L.gs_ctx_set_timing.argtypes = [vp, i32]
        L.gs_kernel_times.argtypes = [vp, C.POINTER(C.c_double), i32]
        L.gs_kernel_times.restype = i32
        L.gs_debug_set.argtypes = [vp, i32, u64]
        L.gs_segmented_plan_create.argtypes = [vp, i32, u64, vp, u32, u32, C.POINTER(vp)]
        L.gs_segmented_plan_create.restype = i32
        L.gs_segmented_plan_run.argtypes = [vp, vp, vp, vp]
        L.gs_segmented_plan_run.restype = i32
        L.gs_segmented_plan_destroy.argtypes = [vp]
        L.gs_segmented_plan_destroy.restype = None
        L.gs_segmented_layout.argtypes = [i32, u64, vp, u32, vp, C.POINTER(u64)]
        L.gs_segmented_layout.restype = i32
        L.gs_sort_keys_noalloc.argtypes = [i32, vp, vp, u64, u32, vp]
        L.gs_sort_keys_noalloc.restype = i32
        L.gs_pass_shape_count.restype = i32
        L.gs_pass_shape_info.argtypes = [i32, i32, i32, C.POINTER(u32), C.POINTER(u32)]
        L.gs_pass_shape_info.restype = i32
        L.gs_ctx_set_tuning.argtypes = [vp, C.POINTER(gs_tuning_entry), u32]
        L.gs_ctx_set_tuning.restype = i32
        L.gs_tuning_parse.argtypes = [C.c_char_p, C.POINTER(gs_tuning_entry), u32]
        L.gs_tuning_parse.restype = i32
        L.gs_ctx_load_tuning.argtypes = [vp, C.c_char_p]
        L.gs_ctx_load_tuning.restype = i32
        L.gs_ctx_choice.argtypes = [vp, i32, i32, u64, C.POINTER(C.c_int), C.POINTER(u32)]
        L.gs_ctx_choice.restype = i32
        L.gs_file_count.argtypes = [C.c_char_p]
        L.gs_file_count.restype = C.c_int64
        L.gs_file_read.argtypes = [vp, C.c_char_p, vp, u64, u32, u32, C.POINTER(u64)]
        L.gs_file_read.restype = i32
        L.gs_file_write.argtypes = [vp, C.c_char_p, vp, u64, u32, u32]
        L.gs_file_write.restype = i32
        L.gs_partitions_read.argtypes = [vp, C.c_char_p, C.c_char_p, i32, vp, u64, u32, u32,
                                         C.POINTER(u64)]
        L.gs_partitions_read.restype = i32
        L.gs_partitions_write.argtypes = [vp, C.c_char_p, C.c_char_p, i32, vp, u64, u32, u32]
        L.gs_partitions_write.restype = i32
        L.gs_partition_block.argtypes = [u64, i32]
        L.gs_partition_block.restype = u64
        L.gs_server_create.argtypes = [i32, C.POINTER(gs_server_opts)]
        L.gs_server_create.restype = vp
        L.gs_server_destroy.argtypes = [vp]
        L.gs_server_destroy.restype = None
        L.gs_server_submit.argtypes = [vp, i32, i32, i32, vp, vp, vp, vp, u64, u32,
                                       C.POINTER(u64)]
        L.gs_server_submit.restype = i32
        L.gs_server_poll.argtypes = [vp, u64, i32, C.POINTER(C.c_double)]
        L.gs_server_poll.restype = i32
        L.gs_server_cancel.argtypes = [vp, u64]
        L.gs_server_cancel.restype = i32
        L.gs_server_get_stats.argtypes = [vp, C.POINTER(gs_server_stats), i32]
        L.gs_server_get_stats.restype = i32
        for fn in ("gs_ctx_set_stream", "gs_ctx_synchronize", "gs_sort_keys", "gs_sort_pairs",
                   "gs_segmented_sort_keys", "gs_gather", "gs_ctx_set_timing", "gs_debug_set"):
            getattr(L, fn).restype = i32
        _lib = L
        return L


def _entry(e: dict) -> gs_tuning_entry:
    kd = e["key_dtype"]
    kd = DTYPE_NAMES.index(kd) if isinstance(kd, str) else int(kd)
    return gs_tuning_entry(kd, int(e.get("val_bytes", 0)), int(e.get("log2n_min", 0)),
                           int(e.get("log2n_max", 63)), int(e.get("pass_shape", -1)),
                           int(e.get("partitions", 0)))


def pass_shapes(key_bytes: int, val_bytes: int) -> list[tuple[int, int]]:
    """(threads, items per thread) of every pass shape for a key/payload width."""
    L = load()
    out = []
    for s in range(L.gs_pass_shape_count()):
        t, it = C.c_uint32(), C.c_uint32()
        if L.gs_pass_shape_info(key_bytes, val_bytes, s, C.byref(t), C.byref(it)) != GS_OK:
            raise GsError(GS_ERR_INVALID, "pass shape")
        out.append((t.value, it.value))
    return out


SEG_EMPTY, SEG_WARP, SEG_GROUP, SEG_PASSES = 0, 1, 2, 3  # gs_seg_kind


def segmented_layout(dtype, n: int, offsets) -> tuple[np.ndarray, dict]:
    """gs_segmented_layout: the gs_seg_kind of each segment and the counts of
    groups, warp-sorted segments, pass-sorted segments and pass tiles
    (host only; no device needed)."""
    L = load()
    off = np.ascontiguousarray(offsets, dtype=np.uint64)
    nseg = off.size - 1
    kinds = np.zeros(max(1, nseg), dtype=np.uint8)
    counts = (C.c_uint64 * 4)()
    st = L.gs_segmented_layout(dtype_code(dtype), int(n), off.ctypes.data, nseg,
                               kinds.ctypes.data, counts)
    if st != GS_OK:
        raise GsError(st, L.gs_last_global_error().decode())
    keys = ("groups", "warp_segments", "pass_segments", "tiles")
    return kinds[:nseg], {k: int(counts[i]) for i, k in enumerate(keys)}


def tuning_parse(text: str) -> list[dict] | None:
    """Entries the engine reads from a tuning JSON document (None: rejected)."""
    L = load()
    k = L.gs_tuning_parse(text.encode(), None, 0)
    if k < 0:
        return None
    arr = (gs_tuning_entry * max(1, k))()
    assert L.gs_tuning_parse(text.encode(), arr, k) == k
    return [{f: getattr(arr[i], f) for f, _ in gs_tuning_entry._fields_} for i in range(k)]


def dtype_code(dt) -> int:
    """gs_dtype of a numpy or torch dtype."""
    try:
        import torch
        tmap = {torch.int32: GS_I32, torch.float32: GS_F32, torch.int64: GS_I64,
                torch.float64: GS_F64}
        for name, code in (("uint32", GS_U32), ("uint64", GS_U64)):
            if hasattr(torch, name):
                tmap[getattr(torch, name)] = code
        if dt in tmap:
            return tmap[dt]
    except ImportError:
        pass
    d = np.dtype(dt)
    if d not in _NP_DTYPE:
        raise GsError(GS_ERR_BAD_DTYPE, f"unsupported dtype {dt}")
    return _NP_DTYPE[d]


def _count(x) -> int:
    return int(x.numel()) if hasattr(x, "numel") else int(x.size)


def _ptr(x) -> int:
    if x is None:
        return 0
    if isinstance(x, np.ndarray):
        return x.ctypes.data
    return x.data_ptr()


class Context:
    """One engine context (device, stream, scratch within an HBM budget)."""

    def __init__(self, device: int = 0, hbm_budget_bytes: int = 0):
        self.L = load()
        h = self.L.gs_ctx_create(device, hbm_budget_bytes)
        if not h:
            raise GsError(GS_ERR_NO_DEVICE, self.L.gs_last_global_error().decode())
        self.h = h
        self.device = device

    def close(self):
        if getattr(self, "h", None):
            self.L.gs_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, st: int):
        if st != GS_OK:
            raise GsError(st, self.L.gs_last_error(self.h).decode())

    def set_stream(self, stream_handle: int | None):
        self._check(self.L.gs_ctx_set_stream(self.h, stream_handle or None))

    def synchronize(self):
        self._check(self.L.gs_ctx_synchronize(self.h))

    def status_synchronize(self) -> int:
        return self.L.gs_ctx_synchronize(self.h)

    def last_error(self) -> str:
        return self.L.gs_last_error(self.h).decode()

    @staticmethod
    def _opts(algo=ALGO_AUTO, partitions=0, k_way=0, oversample=0, seed=0):
        return gs_opts(algo, partitions, k_way, oversample, seed)

    def sort_keys(self, keys_in, keys_out, *, descending=False, flags=0, n=None, dtype=None,
                  algo=ALGO_AUTO, partitions=0, k_way=0, oversample=0, seed=0) -> int:
        """Sort device tensors (or host arrays with FLAG_HOST). `dtype` (a numpy
        dtype) overrides the element type, e.g. to sort int32-typed torch
        storage as uint32. Returns gs_status."""
        n = _count(keys_in) if n is None else int(n)
        f = flags | (FLAG_DESCENDING if descending else 0)
        o = self._opts(algo, partitions, k_way, oversample, seed)
        code = dtype_code(dtype if dtype is not None else keys_in.dtype)
        return self.L.gs_sort_keys(self.h, code, _ptr(keys_in), _ptr(keys_out), n, f, C.byref(o))

    def sort_pairs(self, keys_in, vals_in, keys_out, vals_out, *, descending=False,
                   stable=False, flags=0, n=None, key_dtype=None, val_dtype=None,
                   algo=ALGO_AUTO, partitions=0, k_way=0, oversample=0, seed=0) -> int:
        n = _count(keys_in) if n is None else int(n)
        f = flags | (FLAG_DESCENDING if descending else 0) | (FLAG_PAIRS_STABLE if stable else 0)
        o = self._opts(algo, partitions, k_way, oversample, seed)
        kc = dtype_code(key_dtype if key_dtype is not None else keys_in.dtype)
        vc = dtype_code(val_dtype if val_dtype is not None else vals_in.dtype)
        return self.L.gs_sort_pairs(self.h, kc, vc, _ptr(keys_in), _ptr(vals_in), _ptr(keys_out),
                                    _ptr(vals_out), n, f, C.byref(o))

    def segmented_sort_keys(self, keys_in, keys_out, offsets, nseg, *, descending=False,
                            flags=0, n=None, dtype=None) -> int:
        n = _count(keys_in) if n is None else int(n)
        f = flags | (FLAG_DESCENDING if descending else 0)
        code = dtype_code(dtype if dtype is not None else keys_in.dtype)
        return self.L.gs_segmented_sort_keys(self.h, code, _ptr(keys_in), _ptr(keys_out), n,
                                             _ptr(offsets), nseg, f)

    def segmented_plan(self, dtype, n: int, host_offsets: np.ndarray, *, descending=False):
        """Plan a batched sort (host offsets, nseg+1 entries). Returns a handle."""
        off = np.ascontiguousarray(host_offsets, dtype=np.uint64)
        h = C.c_void_p()
        st = self.L.gs_segmented_plan_create(self.h, dtype_code(dtype), n, off.ctypes.data,
                                             off.size - 1,
                                             FLAG_DESCENDING if descending else 0, C.byref(h))
        self._check(st)
        return h

    def segmented_run(self, plan, keys_in, keys_out) -> int:
        return self.L.gs_segmented_plan_run(self.h, plan, _ptr(keys_in), _ptr(keys_out))

    def segmented_destroy(self, plan):
        self.L.gs_segmented_plan_destroy(plan)

    def gather(self, src, dst, perm, elem_bytes, flags=0) -> int:
        n = _count(perm)
        return self.L.gs_gather(self.h, _ptr(src), _ptr(dst), n, elem_bytes, _ptr(perm), flags)

    def set_timing(self, enable: bool):
        self._check(self.L.gs_ctx_set_timing(self.h, int(enable)))

    def phase_times(self) -> dict:
        names = (C.c_char_p * 8)()
        ms = (C.c_double * 8)()
        k = self.L.gs_phase_times(self.h, names, ms, 8)
        return {names[i].decode(): ms[i] for i in range(min(k, 8))}

    def kernel_times(self) -> list[float]:
        """[upsweep, plan, pass 0, pass 1, ...] device ms of the last sort."""
        ms = (C.c_double * 32)()
        k = self.L.gs_kernel_times(self.h, ms, 32)
        return [ms[i] for i in range(min(k, 32))]

    def debug_set(self, key: int, value: int):
        self._check(self.L.gs_debug_set(self.h, key, value))

    def set_tuning(self, entries: list[dict]):
        """Install a tuning table (dicts with the gs_tuning_entry fields)."""
        arr = (gs_tuning_entry * max(1, len(entries)))()
        for i, e in enumerate(entries):
            arr[i] = _entry(e)
        self._check(self.L.gs_ctx_set_tuning(self.h, arr, len(entries)))

    def load_tuning(self, path):
        self._check(self.L.gs_ctx_load_tuning(self.h, str(path).encode()))

    def choice(self, key_dtype, val_bytes: int, n: int) -> tuple[int, int]:
        """(pass shape, SampleSort buckets) the context uses for such a call."""
        shape, parts = C.c_int(), C.c_uint32()
        self._check(self.L.gs_ctx_choice(self.h, dtype_code(key_dtype), val_bytes, n,
                                         C.byref(shape), C.byref(parts)))
        return shape.value, parts.value


class Server:
    """Serving loop on one device (gs_server_*): submit sort requests, poll
    their completion. Device tensors by default; host arrays with FLAG_HOST."""

    def __init__(self, device: int = 0, hbm_budget: int = 0, max_request_keys: int = 0,
                 slots: int = 0, max_queue: int = 0):
        self.L = load()
        o = gs_server_opts(hbm_budget, max_request_keys, slots, max_queue)
        h = self.L.gs_server_create(device, C.byref(o))
        if not h:
            raise GsError(GS_ERR_NO_DEVICE, self.L.gs_last_global_error().decode())
        self.h = h
        self.device = device

    def close(self):
        if getattr(self, "h", None):
            self.L.gs_server_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def submit(self, keys_in, keys_out, vals_in=None, vals_out=None, *, descending=False,
               stable=False, flags=0, n=None, key_dtype=None, val_dtype=None) -> int:
        """Queue one request; returns its id. Raises GsError on refusal."""
        n = _count(keys_in) if n is None else int(n)
        f = flags | (FLAG_DESCENDING if descending else 0) | (FLAG_PAIRS_STABLE if stable else 0)
        kc = dtype_code(key_dtype if key_dtype is not None else keys_in.dtype)
        has_v = vals_in is not None
        vc = dtype_code(val_dtype if val_dtype is not None else vals_in.dtype) if has_v else 0
        rid = C.c_uint64()
        st = self.L.gs_server_submit(self.h, kc, int(has_v), vc, _ptr(keys_in), _ptr(vals_in),
                                     _ptr(keys_out), _ptr(vals_out), n, f, C.byref(rid))
        if st != GS_OK:
            raise GsError(st, self.L.gs_last_global_error().decode())
        return rid.value

    def poll(self, request_id: int, wait: bool = True) -> tuple[int, float]:
        """(status, latency ms); status GS_ERR_BUSY while not finished."""
        ms = C.c_double()
        st = self.L.gs_server_poll(self.h, request_id, int(wait), C.byref(ms))
        return st, ms.value

    def cancel(self, request_id: int) -> int:
        return self.L.gs_server_cancel(self.h, request_id)

    def stats(self, reset: bool = False) -> dict:
        s = gs_server_stats()
        st = self.L.gs_server_get_stats(self.h, C.byref(s), int(reset))
        if st != GS_OK:
            raise GsError(st, "stats")
        return {k: getattr(s, k) for k, _ in gs_server_stats._fields_}


# ---- per-rank binary files (gs_file_* / gs_partitions_*) ----

def _raise_global(st: int):
    if st != GS_OK:
        raise GsError(st, load().gs_last_global_error().decode())


def _elem_bytes(x) -> int:
    return int(x.element_size()) if hasattr(x, "element_size") else int(x.itemsize)


def file_count(path) -> int:
    return int(load().gs_file_count(str(path).encode()))


def read_file(path, out, ctx: "Context | None" = None) -> int:
    """Read one rank file into `out` (a numpy array: host; a CUDA tensor:
    device through `ctx`). Returns the element count read."""
    host = isinstance(out, np.ndarray)
    got = C.c_uint64()
    _raise_global(load().gs_file_read(None if host else ctx.h, str(path).encode(), _ptr(out),
                                      _count(out), _elem_bytes(out), FLAG_HOST if host else 0,
                                      C.byref(got)))
    return got.value


def write_file(path, data, n: int | None = None, ctx: "Context | None" = None):
    host = isinstance(data, np.ndarray)
    n = _count(data) if n is None else int(n)
    _raise_global(load().gs_file_write(None if host else ctx.h, str(path).encode(), _ptr(data), n,
                                       _elem_bytes(data), FLAG_HOST if host else 0))


def read_partitions(directory, nparts: int, out, ext: str = ".dat",
                    ctx: "Context | None" = None) -> int:
    host = isinstance(out, np.ndarray)
    got = C.c_uint64()
    _raise_global(load().gs_partitions_read(None if host else ctx.h, str(directory).encode(),
                                            ext.encode(), nparts, _ptr(out), _count(out),
                                            _elem_bytes(out), FLAG_HOST if host else 0,
                                            C.byref(got)))
    return got.value


def write_partitions(directory, nparts: int, data, ext: str = ".dat", n: int | None = None,
                     ctx: "Context | None" = None):
    host = isinstance(data, np.ndarray)
    n = _count(data) if n is None else int(n)
    _raise_global(load().gs_partitions_write(None if host else ctx.h, str(directory).encode(),
                                             ext.encode(), nparts, _ptr(data), n,
                                             _elem_bytes(data), FLAG_HOST if host else 0))
