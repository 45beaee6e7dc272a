"""More than 256 buckets (B from 257 to 65536; range to 8192 splitters): the
one-call multisplit runs two stable digit passes and must equal the oracle's
single multisplit bit for bit (keys, values, offsets); the histogram takes the
same counts."""
import numpy as np
import pytest
import torch

import gpumultisplit_gb300 as gms
from gpumultisplit_gb300 import datagen
from gpu_util import KIND_NAMES, host, run_multisplit, to_dev

pytestmark = pytest.mark.gpu


def big_identifiers(o, kind, B, seed=3):
    if kind == o.DELTA:
        return gms.delta_bucket(), o.Desc(o.DELTA, B), None
    if kind == o.DIV:
        p = (1 << 32) // B + 777
        return gms.delta_func(p), o.Desc(o.DIV, B, param=p), None
    if kind == o.BITS:
        return gms.bits_bucket(32 - B.bit_length() + 1), o.Desc(o.BITS, B, shift=32 - B.bit_length() + 1), None
    if kind == o.RANGE:
        spl = datagen.range_splitters(B, seed, "cuda")
        return gms.range_bucket(spl), o.Desc(o.RANGE, B, splitters=datagen.as_u32(spl)), spl
    inv = 1.3 * B / 2**32  # ids above B wrap modulo B
    return gms.even_float_bucket(0, inv), o.Desc(o.EVEN_FLOAT, B, lower=0, inverse_delta=inv), None


CASES = [(257, 0), (300, 3), (1000, 0), (1000, 1), (1000, 3), (1000, 5), (4096, 2), (4096, 3), (8192, 3),
         (12345, 0), (12345, 5), (65536, 0), (65536, 1), (65536, 2)]


@pytest.mark.parametrize("B,kind", CASES, ids=[f"{b}-{KIND_NAMES[k]}" for b, k in CASES])
@pytest.mark.parametrize("with_values", [False, True], ids=["keys", "pairs"])
def test_big_b_matches_oracle(gms_lib, oracle_mod, B, kind, with_values):
    o = oracle_mod
    ident, d, keep = big_identifiers(o, kind, B, seed=B)
    for i, n in enumerate([1, 4097, 300007]):
        keys = datagen.as_u32(datagen.uniform_u32(n, 50 * B + kind + i))
        keys[: min(n, 3)] = [0, 0xFFFFFFFF, 0x80000000][: min(n, 3)]
        vals = np.arange(n, dtype=np.uint32) if with_values else None
        gk, gv, offs, err = run_multisplit(keys, B, ident, vals)
        rk, rv, roffs = o.multisplit(keys, d, vals)
        assert err == 0
        np.testing.assert_array_equal(gk, rk)
        if with_values:
            np.testing.assert_array_equal(gv, rv)
        assert len(offs) == B and offs == [int(x) for x in roffs]
    del keep


@pytest.mark.parametrize("B", [300, 8192])
def test_big_range_duplicates_and_low_keys(gms_lib, oracle_mod, B):
    o = oracle_mod
    rng = np.random.default_rng(B)
    spl = np.sort((np.uint32(0x20000000) + rng.integers(0, 8 * B, B)).astype(np.uint32))
    spl[B // 3] = spl[B // 3 - 1]
    n = 100003
    keys = np.concatenate([spl, spl - np.uint32(1), spl + np.uint32(1),
                           rng.integers(0, 2**32, n - 3 * B, dtype=np.uint64).astype(np.uint32)])
    rng.shuffle(keys)
    d_spl = datagen.from_u32(spl, "cuda")
    vals = np.arange(n, dtype=np.uint32)
    gk, gv, offs, err = run_multisplit(keys, B, gms.range_bucket(d_spl), vals)
    rk, rv, roffs = o.multisplit(keys, o.Desc(o.RANGE, B, splitters=spl), vals)
    assert err == 0
    np.testing.assert_array_equal(gk, rk)
    np.testing.assert_array_equal(gv, rv)
    assert offs == [int(x) for x in roffs]
    h = torch.zeros(B, dtype=torch.int32, device="cuda")
    gms.histogram_range(to_dev(keys), n, h, B, d_spl)
    np.testing.assert_array_equal(h.cpu().numpy(), o.histogram(keys, o.Desc(o.RANGE, B, splitters=spl)))


@pytest.mark.parametrize("B,kind", [(1000, 0), (4096, 3), (65536, 5)])
def test_big_b_histogram(gms_lib, oracle_mod, B, kind):
    """B bins counted; the words after the B-entry histogram are left alone."""
    o = oracle_mod
    ident, d, keep = big_identifiers(o, kind, B)
    n = 1 << 20
    keys = datagen.as_u32(datagen.uniform_u32(n, 8 + B))
    buf = torch.full((B + 64,), -7, dtype=torch.int32, device="cuda")
    buf[:B].zero_()
    gms.multisplit_histogram(to_dev(keys), n, buf[:B], B, ident)
    got = buf.cpu().numpy()
    np.testing.assert_array_equal(got[:B], o.histogram(keys, d))
    assert (got[B:] == -7).all()


def test_big_b_skewed_keys(gms_lib, oracle_mod):
    o = oracle_mod
    keys = datagen.as_u32(datagen.zipf_u32(500009, 5, distinct=1 << 14))
    vals = np.arange(keys.size, dtype=np.uint32)
    gk, gv, offs, err = run_multisplit(keys, 20000, gms.delta_bucket(), vals)
    rk, rv, roffs = o.multisplit(keys, o.Desc(o.DELTA, 20000), vals)
    assert err == 0
    np.testing.assert_array_equal(gk, rk)
    np.testing.assert_array_equal(gv, rv)
    assert offs == [int(x) for x in roffs]


def test_big_b_full_size_properties(gms_lib):
    """2^26 pairs into 65536 delta buckets: buckets ascending, the values a
    permutation in stable order, and the offsets equal the bucket starts."""
    n, B = 1 << 26, 65536
    kin = datagen.uniform_u32(n, 99, device="cuda")
    vin = torch.arange(n, dtype=torch.int32, device="cuda")
    kout, vout = torch.empty_like(kin), torch.empty_like(vin)
    ctx = gms.multisplit_context(B)
    gms.multisplit_allocate_key_value(n, ctx)
    offs = gms.multisplit_key_value(kin, vin, kout, vout, n, ctx, gms.delta_bucket(), multisplit_offset=True)
    torch.cuda.synchronize()
    b = ((kout.long() & 0xFFFFFFFF) * B) >> 32
    assert bool((b[1:] >= b[:-1]).all())
    same = b[1:] == b[:-1]
    assert bool((vout[1:][same] > vout[:-1][same]).all())
    assert torch.equal(kin[vout.long()], kout)
    starts = torch.searchsorted(b, torch.arange(B, device="cuda"))
    assert starts.cpu().tolist() == offs
    assert host(kout).size == n
