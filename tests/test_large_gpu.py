"""Sorts past 2^31 elements on the device: element indexes, tile counts and
scatter destinations must not overflow 32-bit signed arithmetic anywhere
(the engine accepts up to 2^32 - 1 elements). Checked by size-independent
properties, since the oracle would take minutes: sortedness, the key sum,
and for pairs that the index payload is a permutation kept in input order
within ties."""
import numpy as np
import pytest

from gpusort_gb300 import capi, datagen

pytestmark = pytest.mark.gpu

N = (1 << 31) + 12345


STEP = 1 << 28


def _sum_u32(t) -> int:
    """Sum of int32 storage read as uint32, in chunks."""
    import torch
    return sum(int((t[i:i + STEP].to(torch.int64) & 0xFFFFFFFF).sum())
               for i in range(0, t.numel(), STEP))


def _sorted_unsigned(t) -> bool:
    import torch
    sign = torch.tensor(-2**31, dtype=t.dtype, device=t.device)  # int32 storage of uint32
    for i in range(0, t.numel() - 1, STEP):
        a = t[i:i + STEP + 1] ^ sign
        if not bool((a[1:] >= a[:-1]).all()):
            return False
    return True


def test_keys_past_2e31(ctx):
    import torch
    a = datagen.device("uniform", N, np.uint32, seed=31)
    want_sum = _sum_u32(a)
    o = torch.empty_like(a)
    st = ctx.sort_keys(a, o, dtype=np.uint32, flags=capi.FLAG_SYNC)
    assert st == capi.GS_OK, ctx.last_error()
    assert _sorted_unsigned(o)
    assert _sum_u32(o) == want_sum
    del a


def test_stable_pairs_past_2e31(ctx):
    import torch
    k = datagen.device("distinct8", N, np.uint32, seed=32)
    v = torch.arange(N, dtype=torch.int32, device=k.device)  # wraps past 2^31: order by uint32
    ko, vo = torch.empty_like(k), torch.empty_like(v)
    st = ctx.sort_pairs(k, v, ko, vo, key_dtype=np.uint32, val_dtype=np.uint32, stable=True,
                        flags=capi.FLAG_SYNC)
    assert st == capi.GS_OK, ctx.last_error()
    del k, v
    assert _sorted_unsigned(ko)
    # Within each run of equal keys the payload (input index) increases.
    for i in range(0, N - 1, STEP):
        kk = ko[i:i + STEP + 1]
        vv = vo[i:i + STEP + 1].to(torch.int64) & 0xFFFFFFFF
        ties = kk[1:] == kk[:-1]
        assert bool((vv[1:][ties] > vv[:-1][ties]).all())
    assert _sum_u32(vo) == N * (N - 1) // 2
