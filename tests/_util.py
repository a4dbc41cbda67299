"""Helpers shared by the tests: numpy <-> torch CUDA byte-exact transfers."""
from __future__ import annotations

import numpy as np

_STORAGE = {1: None, 4: np.int32, 8: np.int64}


def storage_dtype(dt):
    dt = np.dtype(dt)
    if dt.kind == "f":
        return dt
    return np.dtype(np.int32 if dt.itemsize == 4 else np.int64)


def to_dev(a: np.ndarray):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a).view(storage_dtype(a.dtype))).cuda()


def from_dev(t, dtype) -> np.ndarray:
    return t.cpu().numpy().view(np.dtype(dtype))


def empty_dev(n: int, dtype):
    import torch
    sd = storage_dtype(dtype)
    tmap = {np.dtype(np.int32): torch.int32, np.dtype(np.int64): torch.int64,
            np.dtype(np.float32): torch.float32, np.dtype(np.float64): torch.float64}
    return torch.empty(n, dtype=tmap[np.dtype(sd)], device="cuda")


def same_bits(a: np.ndarray, b: np.ndarray) -> bool:
    if a.shape != b.shape or a.dtype != b.dtype:
        return False
    return bool(np.array_equal(a.view(np.uint8), b.view(np.uint8)))
