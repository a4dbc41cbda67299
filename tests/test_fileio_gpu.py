"""Per-rank binary files to and from device memory (pinned staging on the
context's stream), and the reference's file-based workflow: p rank files
read into HBM as p partitions, sorted, written back."""
import numpy as np
import pytest

from gpusort_gb300 import capi, datagen
from oracle import oracle
from tests._util import empty_dev, from_dev, same_bits, to_dev

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("dtype,n", [(np.uint32, 20_000_003), (np.float64, 9_000_001),
                                     (np.int64, 0), (np.uint32, 1)])
def test_device_round_trip(ctx, tmp_path, dtype, n):
    a = datagen.host("uniform", n, dtype, seed=5)
    d = to_dev(a)
    path = tmp_path / "x.dat"
    capi.write_file(path, d, ctx=ctx)
    assert path.read_bytes()[:8] == np.int64(n).tobytes()
    back = empty_dev(n + 3, dtype)
    assert capi.read_file(path, back, ctx=ctx) == n
    assert same_bits(from_dev(back, dtype)[:n], a)


def test_rank_files_sorted_on_the_device(ctx, tmp_path):
    p = 4
    parts = [datagen.host("uniform", 1 << 20, np.uint32, seed=0x67707573 + r) for r in range(p)]
    for r, a in enumerate(parts):
        capi.write_file(tmp_path / f"{r}.dat", a)
    whole = np.concatenate(parts)
    d = empty_dev(whole.size, np.uint32)
    assert capi.read_partitions(tmp_path, p, d, ctx=ctx) == whole.size
    out = empty_dev(whole.size, np.uint32)
    st = ctx.sort_keys(d, out, dtype=np.uint32, algo=capi.ALGO_HYK, partitions=p, k_way=4,
                       flags=capi.FLAG_SYNC)
    assert st == capi.GS_OK, ctx.last_error()
    (tmp_path / "out").mkdir()
    capi.write_partitions(tmp_path / "out", p, out, ext=".sorted", ctx=ctx)
    back = np.empty(whole.size, np.uint32)
    assert capi.read_partitions(tmp_path / "out", p, back, ext=".sorted") == whole.size
    assert same_bits(back, oracle.sort_keys(whole))
