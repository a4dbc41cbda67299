#!/usr/bin/env python3
"""Generate the golden fixtures of tests/golden/ by running the REFERENCE'S
OWN sort code (HykSort / SampleSort / HyperQuickSort, CPU path, built from
the reference sources by oracle/ref/Makefile into oracle/_ref/ref_driver)
on seeded inputs.

Run in a container where the reference sources are present:
    make -C oracle/ref && python tests/golden/make_golden.py
The fixtures are small .npz files (input, output, parameters) that travel
with the repository; the tests compare the CPU oracle and the GPU engine
with them.

Cases:
* keys: each algorithm x key type x distribution x order, p ranks, k-way;
* pairs: key/value sorts (ties ordered by value, include/helpers/
  hyksort_helper.h:266-280);
* known answers from the reference's own checkers: shuffled arithmetic
  progressions must come out as a1 + i*d (src/test/arithmetic_progression_
  checker.h:49-106), shuffled log10/ln sequences as log(i + start)
  (src/test/log_checker.h:45-87), constant inputs unchanged
  (src/test/zero_checker.h:34-74).
"""
from __future__ import annotations

import subprocess
import sys
import tempfile
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))
from gpusort_gb300 import datagen  # noqa: E402

DRIVER = ROOT / "oracle" / "_ref" / "ref_driver"
OUT = Path(__file__).resolve().parent
CODES = {np.dtype(np.uint32): "u32", np.dtype(np.int32): "i32", np.dtype(np.float32): "f32",
         np.dtype(np.uint64): "u64", np.dtype(np.int64): "i64", np.dtype(np.float64): "f64"}


def _write(path: Path, a: np.ndarray):
    with open(path, "wb") as f:
        np.array([a.size], np.int64).tofile(f)
        a.tofile(f)


def _read(path: Path, dt) -> np.ndarray:
    with open(path, "rb") as f:
        n = int(np.fromfile(f, np.int64, 1)[0])
        return np.fromfile(f, dt, n)


def run_ref(algo, keys, p, k, desc, vals=None):
    with tempfile.TemporaryDirectory() as td:
        td = Path(td)
        _write(td / "k.bin", keys)
        cmd = [str(DRIVER), algo, CODES[keys.dtype], str(p), str(k), "2", str(int(desc)),
               str(td / "k.bin"), str(td / "ko.bin")]
        if vals is not None:
            _write(td / "v.bin", vals)
            cmd += [CODES[vals.dtype], str(td / "v.bin"), str(td / "vo.bin")]
        r = subprocess.run(cmd, capture_output=True, text=True, timeout=600)
        if r.returncode != 0:
            raise RuntimeError(f"reference run failed: {' '.join(cmd)}\n{r.stderr}")
        ko = _read(td / "ko.bin", keys.dtype)
        vo = _read(td / "vo.bin", vals.dtype) if vals is not None else None
        sizes = [int(x) for x in r.stderr.split("sizes", 1)[1].split()]
        return ko, vo, np.array(sizes, np.int64)


def main():
    if not DRIVER.exists():
        sys.exit(f"{DRIVER} missing: build it with make -C oracle/ref")
    n_written = 0
    cases = []
    seed = 1000
    for algo in ("hyk", "sample", "hquick"):
        for dt in (np.uint32, np.int32, np.float32, np.uint64, np.int64, np.float64):
            for dist in ("uniform", "zipf", "distinct8", "equal", "reverse"):
                seed += 1
                desc = bool(seed % 2)
                p, k = ((4, 4), (8, 2), (4, 2), (16, 4), (6, 4))[seed % 5]
                cases.append((algo, dt, dist, desc, p, k, 3000 + (seed % 7) * 517, seed))
    for algo, dt, dist, desc, p, k, n, s in cases:
        a = datagen.host(dist, n, dt, seed=s)
        ko, _, sizes = run_ref(algo, a, p, k, desc)
        name = f"keys_{algo}_{CODES[np.dtype(dt)]}_{dist}_{'desc' if desc else 'asc'}.npz"
        np.savez_compressed(OUT / name, input=a, output=ko, rank_sizes=sizes,
                            algo=algo, p=p, k=k, desc=desc)
        n_written += 1
    # pairs
    pair_types = [(np.uint32, np.uint32), (np.float32, np.int64), (np.uint64, np.float64),
                  (np.int64, np.uint32), (np.int32, np.int32), (np.float64, np.uint64)]
    for algo in ("hyk", "sample", "hquick"):
        for i, (kt, vt) in enumerate(pair_types):
            for desc in (False, True):
                s = 5000 + i * 2 + desc
                kk = datagen.host("distinct8" if i % 2 else "zipf", 4096, kt, seed=s)
                vv = datagen.host("distinct8", 4096, vt, seed=s + 77)
                ko, vo, sizes = run_ref(algo, kk, 4, 4, desc, vv)
                name = (f"pairs_{algo}_{CODES[np.dtype(kt)]}_{CODES[np.dtype(vt)]}_"
                        f"{'desc' if desc else 'asc'}.npz")
                np.savez_compressed(OUT / name, keys=kk, vals=vv, keys_out=ko, vals_out=vo,
                                    rank_sizes=sizes, algo=algo, p=4, k=4, desc=desc)
                n_written += 1
    # known answers of the reference's checkers
    rng = np.random.default_rng(77)
    kat = []
    for dt in (np.float64, np.float32, np.int64, np.int32):
        for d in (0.5, -0.5, 1, -1, 2, -2, 3, -3):
            if np.dtype(dt).kind == "i" and d != int(d):
                continue
            n, a1 = 5000, dt(1)
            ap = (a1 + np.arange(n) * dt(d)).astype(dt)
            shuffled = ap[rng.permutation(n)]
            for desc in (False, True):
                ko, _, _ = run_ref("hyk", shuffled, 4, 4, desc)
                # ArithmeticProgressionChecker: increasing order with d < 0
                # means the reversed progression
                want = np.sort(ap)[::-1] if desc else np.sort(ap)
                assert np.array_equal(ko, want), (dt, d, desc)
                kat.append(dict(kind="ap", input=shuffled, output=ko, desc=desc))
    for fn, start in ((np.log10, 1), (np.log, 7)):
        n = 6000
        seq = fn(np.arange(start, start + n, dtype=np.float64))
        sh = seq[rng.permutation(n)]
        ko, _, _ = run_ref("hyk", sh, 4, 4, False)
        assert np.array_equal(ko, seq)
        kat.append(dict(kind=fn.__name__, input=sh, output=ko, desc=False))
    const = np.full(4000, 123456, np.int64)
    ko, _, _ = run_ref("sample", const, 4, 4, False)
    assert np.array_equal(ko, const)
    kat.append(dict(kind="zero", input=const, output=ko, desc=False))
    for i, c in enumerate(kat):
        np.savez_compressed(OUT / f"kat_{i:02d}_{c['kind']}.npz", input=c["input"],
                            output=c["output"], desc=c["desc"], kind=c["kind"])
        n_written += 1
    print(f"wrote {n_written} fixtures to {OUT}")


if __name__ == "__main__":
    main()
