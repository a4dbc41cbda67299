"""Per-rank binary files (int64 count + raw elements, the reference's test
data format, src/test/utils.h:610-661) in host mode: layout, round trips,
the partition split rule (include/common.h:146-155) and errors."""
import numpy as np
import pytest

from gpusort_gb300 import capi, datagen

DTYPES = [np.uint32, np.int32, np.float32, np.uint64, np.int64, np.float64]


def each_block(total: int, p: int) -> int:
    """The reference's CalcNumElemsEachBlock (include/common.h:146-155)."""
    r = total % p
    if r == 0:
        return total // p
    tmp = (total + (p - r)) // p
    return tmp - 1 if tmp * (p - 1) >= total else tmp


@pytest.mark.parametrize("dtype", DTYPES)
def test_layout_and_round_trip(built_lib, tmp_path, dtype):
    for n in (0, 1, 1000, 77777):
        a = datagen.host("uniform", n, dtype, seed=n)
        path = tmp_path / f"{n}.dat"
        capi.write_file(path, a)
        raw = path.read_bytes()
        assert raw == np.int64(n).tobytes() + a.tobytes()
        assert capi.file_count(path) == n
        out = np.empty(n + 5, dtype)
        assert capi.read_file(path, out) == n
        assert np.array_equal(out[:n].view(np.uint8), a.view(np.uint8))


def test_reads_a_file_laid_out_like_the_reference(built_lib, tmp_path):
    # SaveMyData: ofs.Write(int64 nelem); ofs.Write(first, last)
    a = np.arange(10, dtype=np.float64) * 0.5 - 1.0
    (tmp_path / "3.dat").write_bytes(np.int64(10).tobytes() + a.tobytes())
    out = np.empty(10, np.float64)
    assert capi.read_file(tmp_path / "3.dat", out) == 10
    assert np.array_equal(out, a)


@pytest.mark.parametrize("n,p", [(0, 4), (1, 4), (9, 4), (10, 4), (10, 3), (1 << 16, 4),
                                 (1000003, 7), (5, 8)])
def test_partition_split_and_concatenation(built_lib, tmp_path, n, p):
    a = datagen.host("uniform", n, np.uint32, seed=p)
    capi.write_partitions(tmp_path, p, a)
    each = each_block(n, p) if n else 0
    assert capi.load().gs_partition_block(n, p) == each
    sizes = [capi.file_count(tmp_path / f"{r}.dat") for r in range(p)]
    assert sizes[:-1] == [min(each, max(0, n - each * r)) for r in range(p - 1)]
    assert sum(sizes) == n  # the last file holds the remainder
    out = np.empty(n, np.uint32)
    assert capi.read_partitions(tmp_path, p, out) == n
    assert np.array_equal(out, a)


def test_custom_extension(built_lib, tmp_path):
    a = np.arange(100, dtype=np.int64)
    capi.write_partitions(tmp_path, 2, a, ext=".keys")
    assert (tmp_path / "0.keys").exists() and (tmp_path / "1.keys").exists()
    out = np.empty(100, np.int64)
    assert capi.read_partitions(tmp_path, 2, out, ext=".keys") == 100
    assert np.array_equal(out, a)


def test_errors(built_lib, tmp_path):
    with pytest.raises(capi.GsError) as e:
        capi.read_file(tmp_path / "missing.dat", np.empty(4, np.uint32))
    assert e.value.status == capi.GS_ERR_INVALID
    capi.write_file(tmp_path / "a.dat", np.arange(10, dtype=np.uint32))
    with pytest.raises(capi.GsError) as e:
        capi.read_file(tmp_path / "a.dat", np.empty(9, np.uint32))
    assert e.value.status == capi.GS_ERR_TOO_LARGE
    (tmp_path / "short.dat").write_bytes(np.int64(10).tobytes() + b"\0" * 12)
    with pytest.raises(capi.GsError):
        capi.read_file(tmp_path / "short.dat", np.empty(10, np.uint32))
    (tmp_path / "empty.dat").write_bytes(b"")
    assert capi.file_count(tmp_path / "empty.dat") == -1
    L = capi.load()
    # device memory needs a context
    assert L.gs_file_read(None, str(tmp_path / "a.dat").encode(), None, 10, 4, 0,
                          None) == capi.GS_ERR_INVALID
    assert L.gs_partitions_read(None, str(tmp_path).encode(), b".dat", 0, None, 0, 4,
                                capi.FLAG_HOST, None) == capi.GS_ERR_INVALID
