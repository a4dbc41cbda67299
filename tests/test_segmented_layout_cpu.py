"""How a segmented sort treats each segment (gs_segmented_layout), checked on
the host against a restatement of the planning rules:

* segments of at most 4096 keys are packed, in order, into groups of
  consecutive segments holding at most 4096 keys and 256 segments;
* a group made only of segments of at most 32 keys is sorted one warp per
  segment instead of as a group;
* longer segments go through the radix passes, in tiles of the pass shape
  (256 x 20 keys when segments average under 4096 keys, else 384 x 24 for
  32-bit keys).

The layout is what the GPU tests then sort; here it needs no device.
"""
import numpy as np
import pytest

from gpusort_gb300 import capi

GROUP_KEYS, GROUP_SEGS, TINY_KEYS = 4096, 256, 32


def _tile(n, nseg, key_bytes):
    shape = 0 if nseg and n // nseg >= 4096 else 1
    threads, items = capi.pass_shapes(key_bytes, 0)[shape]
    return threads * items


def _model(off, key_bytes):
    off = [int(x) for x in off]
    nseg = len(off) - 1
    n = off[-1]
    tile = _tile(n, nseg, key_bytes)
    kinds = [capi.SEG_EMPTY] * nseg
    counts = {"groups": 0, "warp_segments": 0, "pass_segments": 0, "tiles": 0}
    group = []  # indices of the open group's non-empty segments
    gkeys = 0

    def close():
        nonlocal group, gkeys
        if group:
            lens = [off[t + 1] - off[t] for t in group]
            if max(lens) <= TINY_KEYS:
                for t in group:
                    kinds[t] = capi.SEG_WARP
                counts["warp_segments"] += len(group)
            else:
                for t in group:
                    kinds[t] = capi.SEG_GROUP
                counts["groups"] += 1
        group, gkeys = [], 0

    for s in range(nseg):
        ln = off[s + 1] - off[s]
        if ln == 0:
            continue
        if ln > GROUP_KEYS:
            close()
            kinds[s] = capi.SEG_PASSES
            counts["pass_segments"] += 1
            counts["tiles"] += -(-ln // tile)
            continue
        if group and (gkeys + ln > GROUP_KEYS or len(group) + 1 > GROUP_SEGS):
            close()
        group.append(s)
        gkeys += ln
    close()
    return np.array(kinds, dtype=np.uint8), counts


def _offsets(lengths):
    return np.concatenate([[0], np.cumsum(np.asarray(lengths, dtype=np.uint64))]).astype(np.uint64)


def _check(lengths, dtype=np.uint32):
    off = _offsets(lengths)
    kinds, counts = capi.segmented_layout(dtype, int(off[-1]), off)
    want_kinds, want_counts = _model(off, np.dtype(dtype).itemsize)
    assert counts == want_counts
    assert np.array_equal(kinds, want_kinds)
    return kinds, counts


@pytest.mark.parametrize("lengths", [
    [1],
    [0, 0, 5, 0],
    [32, 32, 33],                     # a 33-key segment makes the group a group sort
    [32] * 300,                       # more than 256 segments: two warp groups
    [4096, 1],                        # a full group, then a new one
    [4097],                           # the smallest segment the passes take
    [4096, 4097, 4096],
    [10, 10, 5000, 10, 30, 15000, 1],
    [2000, 2000, 97, 1, 4096],        # the key limit closes groups
    [0] * 10 + [70000] + [0] * 3,
])
def test_layout_edge_cases(lengths):
    _check(lengths)


@pytest.mark.parametrize("seed", range(6))
@pytest.mark.parametrize("dtype", [np.uint32, np.uint64])
def test_layout_random_log_uniform(seed, dtype):
    rng = np.random.default_rng(seed)
    nseg = int(rng.integers(1, 3000))
    lengths = np.exp2(rng.uniform(0, 18, size=nseg)).astype(np.int64)
    lengths[rng.random(nseg) < 0.1] = 0
    kinds, counts = _check(lengths, dtype)
    # every non-empty segment is sorted by exactly one of the three kernels
    assert np.all((kinds == capi.SEG_EMPTY) == (lengths == 0))


def test_layout_counts_partition_the_keys():
    rng = np.random.default_rng(9)
    lengths = np.concatenate([rng.integers(1, 33, 500), rng.integers(33, 4097, 200),
                              rng.integers(4097, 60000, 20)])
    rng.shuffle(lengths)
    kinds, counts = _check(lengths)
    tile = _tile(int(lengths.sum()), lengths.size, 4)
    large = lengths[kinds == capi.SEG_PASSES]
    assert counts["tiles"] == int(np.sum(-(-large // tile)))
    assert counts["pass_segments"] == large.size
    assert counts["warp_segments"] == int(np.sum(kinds == capi.SEG_WARP))


def test_layout_rejects_bad_offsets():
    with pytest.raises(capi.GsError):
        capi.segmented_layout(np.uint32, 10, np.array([0, 7, 5, 10], dtype=np.uint64))
    with pytest.raises(capi.GsError):
        capi.segmented_layout(np.uint32, 10, np.array([1, 10], dtype=np.uint64))
