"""When the reference's own CPU path has been built here (oracle/_ref, only
where the reference sources exist), compare it with the oracle on fresh
seeded inputs, for all three entry points and key/value sorts."""
import subprocess
import tempfile
from pathlib import Path

import numpy as np
import pytest

from gpusort_gb300 import datagen
from oracle import oracle

DRIVER = Path(__file__).resolve().parents[1] / "oracle" / "_ref" / "ref_driver"
pytestmark = pytest.mark.skipif(not DRIVER.exists(), reason="reference build not present")
CODES = {np.dtype(np.uint32): "u32", np.dtype(np.int32): "i32", np.dtype(np.float32): "f32",
         np.dtype(np.uint64): "u64", np.dtype(np.int64): "i64", np.dtype(np.float64): "f64"}


def _io(td, name, a=None, dt=None):
    p = Path(td) / name
    if a is not None:
        with open(p, "wb") as f:
            np.array([a.size], np.int64).tofile(f)
            a.tofile(f)
        return str(p)
    with open(p, "rb") as f:
        n = int(np.fromfile(f, np.int64, 1)[0])
        return np.fromfile(f, dt, n)


@pytest.mark.parametrize("algo", ["hyk", "sample", "hquick"])
@pytest.mark.parametrize("dtype", [np.uint32, np.float64, np.int32])
def test_reference_keys_equal_oracle(algo, dtype):
    for dist, p, k, desc in (("uniform", 4, 4, 0), ("zipf", 8, 2, 1), ("distinct8", 2, 2, 0)):
        a = datagen.host(dist, 30011, dtype, seed=p + k)
        with tempfile.TemporaryDirectory() as td:
            r = subprocess.run([str(DRIVER), algo, CODES[np.dtype(dtype)], str(p), str(k), "2",
                                str(desc), _io(td, "i", a), str(Path(td) / "o")],
                               capture_output=True, text=True, timeout=300)
            assert r.returncode == 0, r.stderr
            assert np.array_equal(_io(td, "o", dt=dtype), oracle.sort_keys(a, bool(desc)))


@pytest.mark.parametrize("algo", ["hyk", "sample"])
def test_reference_pairs_equal_oracle(algo):
    k = datagen.host("distinct8", 20000, np.int64, seed=1)
    v = datagen.host("uniform", 20000, np.uint32, seed=2)
    for desc in (0, 1):
        with tempfile.TemporaryDirectory() as td:
            r = subprocess.run([str(DRIVER), algo, "i64", "4", "4", "2", str(desc),
                                _io(td, "k", k), str(Path(td) / "ko"), "u32", _io(td, "v", v),
                                str(Path(td) / "vo")], capture_output=True, text=True, timeout=300)
            assert r.returncode == 0, r.stderr
            wk, wv = oracle.sort_pairs(k, v, bool(desc))
            assert np.array_equal(_io(td, "ko", dt=np.int64), wk)
            assert np.array_equal(_io(td, "vo", dt=np.uint32), wv)
