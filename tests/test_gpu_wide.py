"""64-bit keys and values (beyond the reference, whose kernels hold 32-bit
elements): multisplit with 64-bit keys (key-only, 32- and 64-bit values), 32-bit
keys with 64-bit values, offsets, every identifier kind, ragged sizes, buffers
aligned to 8 but not 16 bytes, and stable sorts by any bit range, each compared
bit-exactly with the oracle's 64-bit restatement (itself checked against
numpy's stable argsort on the CPU)."""
import ctypes

import numpy as np
import pytest
import torch

import gpumultisplit_gb300 as gms
from gpumultisplit_gb300 import datagen
from gpu_util import KIND_NAMES, host, identifiers, to_dev

pytestmark = pytest.mark.gpu

SIZES = [1, 33, 2047, 2049, 4097, 100003]


def dev64(a: np.ndarray, pad_front: int = 0) -> torch.Tensor:
    """Device int64 copy; pad_front > 0 starts the view that many elements into
    its allocation (8-byte but not 16-byte aligned for odd counts)."""
    t = torch.zeros(a.size + pad_front, dtype=torch.int64, device="cuda")
    if a.size:
        t[pad_front:] = datagen.from_u64(a, "cuda")
    return t[pad_front:]


def identifiers64(o, kind, B, seed=7):
    """(library identifier, oracle Desc64, keep-alive) on 64-bit keys."""
    if kind == o.DELTA:
        return gms.delta_bucket(), o.Desc64(o.DELTA, B), None
    if kind == o.DIV:
        p = (1 << 64) // (3 * B) + 987654321
        return gms.delta_func(p), o.Desc64(o.DIV, B, param=p), None
    if kind == o.BITS:
        return gms.bits_bucket(45), o.Desc64(o.BITS, B, shift=45), None
    if kind == o.RANGE:
        spl = np.concatenate([[0], np.sort(datagen.as_u64(datagen.uniform_u64(B - 1, seed)))]).astype(np.uint64)
        d_spl = datagen.from_u64(spl, "cuda")
        return gms.range_bucket(d_spl), o.Desc64(o.RANGE, B, splitters=spl), d_spl
    if kind == o.MASK:
        return gms.mask_bucket(1 << 50), o.Desc64(o.MASK, B, param=1 << 50), None
    inv = float(B) / 2**64 * 1.5  # ids up to 1.5 B: the upper ones wrap modulo B
    return gms.even_float_bucket(1 << 20, inv), o.Desc64(o.EVEN_FLOAT, B, lower=1 << 20, inverse_delta=inv), None


def run_wide(keys, B, ident, vals, pad=0):
    """keys: uint64 or uint32 numpy; vals: None, uint32 or uint64 numpy."""
    n = keys.size
    dk = dev64(keys, pad) if keys.dtype == np.uint64 else to_dev(keys, pad)
    ok = torch.zeros_like(dk)
    dv = ov = None
    if vals is not None:
        dv = dev64(vals, pad) if vals.dtype == np.uint64 else to_dev(vals, pad)
        ov = torch.zeros_like(dv)
    ctx = gms.multisplit_context(B)
    gms.multisplit_wide_allocate(n, ctx, dk.element_size(), 0 if dv is None else dv.element_size())
    offs = gms.multisplit_wide(dk, ok, n, ctx, ident, dv, ov, multisplit_offset=True)
    torch.cuda.synchronize()
    assert gms.read_device_error(ctx) == 0
    ko = datagen.as_u64(ok) if keys.dtype == np.uint64 else host(ok)
    vo = None if ov is None else (datagen.as_u64(ov) if vals.dtype == np.uint64 else host(ov))
    return ko, vo, offs


@pytest.mark.parametrize("B", [2, 7, 32, 100, 256])
@pytest.mark.parametrize("kind", [0, 1, 2, 3, 4, 5], ids=lambda k: KIND_NAMES[k])
@pytest.mark.parametrize("values", [None, 4, 8], ids=["keys", "v32", "v64"])
def test_u64_keys_match_oracle(gms_lib, oracle_mod, B, kind, values):
    o = oracle_mod
    if kind == o.BITS and B & (B - 1):
        pytest.skip("bit-field buckets are powers of two")
    ident, d, keep = identifiers64(o, kind, B, seed=B + kind)
    for i, n in enumerate(SIZES[(B + kind) % 2::2]):
        keys = datagen.as_u64(datagen.uniform_u64(n, 100 * B + 10 * kind + i))
        keys[: min(n, 3)] = np.array([0, 2**64 - 1, 2**63], np.uint64)[: min(n, 3)]
        vals = None
        if values == 4:
            vals = np.arange(n, dtype=np.uint32)
        elif values == 8:
            vals = (np.arange(n, dtype=np.uint64) << np.uint64(33)) | np.uint64(5)
        gk, gv, offs = run_wide(keys, B, ident, vals)
        rk, rv, roffs = o.multisplit64(keys, d, vals)
        np.testing.assert_array_equal(gk, rk)
        if vals is not None:
            np.testing.assert_array_equal(gv, rv)
        assert offs == [int(x) for x in roffs]
    del keep


@pytest.mark.parametrize("B", [2, 12, 256])
@pytest.mark.parametrize("kind", [0, 1, 3, 5], ids=lambda k: KIND_NAMES[k])
def test_u32_keys_u64_values(gms_lib, oracle_mod, B, kind):
    """32-bit keys with 64-bit values: the 32-bit identifiers, values moved whole."""
    o = oracle_mod
    ident, d, keep = identifiers(o, kind, B)
    for i, n in enumerate([1, 2049, 65537]):
        keys = datagen.as_u32(datagen.uniform_u32(n, 300 + B + kind + i))
        vals = datagen.as_u64(datagen.uniform_u64(n, 900 + i))
        gk, gv, offs = run_wide(keys, B, ident, vals)
        rk, perm, roffs = o.multisplit(keys, d, np.arange(n, dtype=np.uint32))
        np.testing.assert_array_equal(gk, rk)
        np.testing.assert_array_equal(gv, vals[perm])
        assert offs == [int(x) for x in roffs]
        # the minimum scratch (no bucket bytes): costly identifiers run in both passes
        full = ctypes.c_size_t()
        assert gms_lib.gms_multisplit_wide_scratch_bytes(n, B, 4, 8, ctypes.byref(full)) == 0
        minimum = full.value - (n + 255) // 256 * 256
        scratch = torch.zeros(minimum, dtype=torch.uint8, device="cuda")
        dk, dv = to_dev(keys), dev64(vals)
        ok, ov = torch.zeros_like(dk), torch.zeros_like(dv)
        desc = ident.desc64(B)
        assert gms_lib.gms_multisplit_wide(dk.data_ptr(), dv.data_ptr(), ok.data_ptr(), ov.data_ptr(), n, 4, 8,
                                           ctypes.byref(desc), scratch.data_ptr(), minimum, None,
                                           torch.cuda.current_stream().cuda_stream) == 0
        torch.cuda.synchronize()
        np.testing.assert_array_equal(host(ok), rk)
        np.testing.assert_array_equal(datagen.as_u64(ov), vals[perm])
    del keep


@pytest.mark.parametrize("pad", [1, 3])
def test_u64_buffers_not_16_byte_aligned(gms_lib, oracle_mod, pad):
    """Arrays 8-byte aligned but not 16: plain loads instead of bulk copies."""
    o = oracle_mod
    n = 30011
    keys = datagen.as_u64(datagen.uniform_u64(n, 55))
    vals = datagen.as_u64(datagen.uniform_u64(n, 56))
    for kind in (o.DELTA, o.RANGE):
        ident, d, keep = identifiers64(o, kind, 256)
        gk, gv, _ = run_wide(keys, 256, ident, vals, pad)
        rk, rv, _ = o.multisplit64(keys, d, vals)
        np.testing.assert_array_equal(gk, rk)
        np.testing.assert_array_equal(gv, rv)


def test_u64_skewed_and_constant_keys(gms_lib, oracle_mod):
    o = oracle_mod
    n = 200003
    zipf32 = datagen.as_u32(datagen.zipf_u32(n, 3, distinct=1 << 12)).astype(np.uint64)
    for keys in (zipf32 << np.uint64(32) | zipf32, np.full(n, 2**64 - 1, np.uint64), np.zeros(n, np.uint64)):
        vals = np.arange(n, dtype=np.uint32)
        gk, gv, offs = run_wide(keys, 256, gms.delta_bucket(), vals)
        rk, rv, roffs = o.multisplit64(keys, o.Desc64(o.DELTA, 256), vals)
        np.testing.assert_array_equal(gk, rk)
        np.testing.assert_array_equal(gv, rv)
        assert offs == [int(x) for x in roffs]


def run_sort(keys, vals, begin, end, digit):
    n = keys.size
    dk = dev64(keys) if keys.dtype == np.uint64 else to_dev(keys)
    ok = torch.zeros_like(dk)
    dv = ov = None
    if vals is not None:
        dv = dev64(vals) if vals.dtype == np.uint64 else to_dev(vals)
        ov = torch.zeros_like(dv)
    ctx = gms.ms_sort_context()
    gms.multisplit_sort_wide_allocate(n, ctx, dk.element_size(), 0 if dv is None else dv.element_size(), begin, end,
                                      digit)
    gms.multisplit_sort_wide(dk, ok, n, ctx, dv, ov)
    torch.cuda.synchronize()
    ko = datagen.as_u64(ok) if keys.dtype == np.uint64 else host(ok)
    vo = None if ov is None else (datagen.as_u64(ov) if vals.dtype == np.uint64 else host(ov))
    return ko, vo


@pytest.mark.parametrize("begin,end,digit", [(0, 64, 8), (0, 64, 7), (0, 64, 4), (13, 47, 6), (40, 40, 8),
                                             (60, 64, 8)])
@pytest.mark.parametrize("values", [None, 4, 8], ids=["keys", "v32", "v64"])
def test_u64_sort_matches_oracle(gms_lib, oracle_mod, begin, end, digit, values):
    o = oracle_mod
    n = 70001
    keys = datagen.as_u64(datagen.uniform_u64(n, begin * 100 + end + digit))
    vals = None if values is None else (np.arange(n, dtype=np.uint32) if values == 4
                                        else datagen.as_u64(datagen.uniform_u64(n, 77)))
    gk, gv = run_sort(keys, vals, begin, end, digit)
    rk, rv = o.sort_bits64(keys, vals, begin, end, digit)
    np.testing.assert_array_equal(gk, rk)
    if vals is not None:
        np.testing.assert_array_equal(gv, rv)
    if (begin, end) == (0, 64):
        np.testing.assert_array_equal(gk, np.sort(keys))


def test_u32_keys_u64_values_sort(gms_lib, oracle_mod):
    n = 100003
    keys = datagen.as_u32(datagen.uniform_u32(n, 9))
    vals = datagen.as_u64(datagen.uniform_u64(n, 10))
    gk, gv = run_sort(keys, vals, 0, 32, 8)
    order = np.argsort(keys, kind="stable")
    np.testing.assert_array_equal(gk, keys[order])
    np.testing.assert_array_equal(gv, vals[order])


def test_u64_sort_large_is_a_stable_permutation(gms_lib):
    """2^24 64-bit keys with values = index: sorted, and the values are the
    stable order (equal keys in index order), checked on the device."""
    n = 1 << 24
    dk = datagen.uniform_u64(n, 1234, "cuda")
    dk[: n // 2] &= 0xFFFF  # many equal keys
    dv = torch.arange(n, dtype=torch.int64, device="cuda")
    ok, ov = torch.empty_like(dk), torch.empty_like(dv)
    ctx = gms.ms_sort_context()
    gms.multisplit_sort_wide_allocate(n, ctx, 8, 8)
    gms.multisplit_sort_wide(dk, ok, n, ctx, dv, ov)
    torch.cuda.synchronize()
    # unsigned order of int64 bit patterns: flip the sign bit
    u = ok ^ torch.tensor(-(1 << 63), dtype=torch.int64, device="cuda")
    assert bool((u[1:] >= u[:-1]).all())
    same = ok[1:] == ok[:-1]
    assert bool((ov[1:][same] > ov[:-1][same]).all())
    assert torch.equal(torch.sort(ov).values, dv)
    assert torch.equal(dk[ov], ok)


def test_wide_checks_alignment_on_device_buffers(gms_lib):
    """A 64-bit key array that is only 4-byte aligned is rejected."""
    t = torch.zeros(1001, dtype=torch.int32, device="cuda")
    ctx = gms.multisplit_context(16)
    gms.multisplit_wide_allocate(500, ctx, 8, 0)
    lib = gms.load()
    d = gms.delta_bucket().desc64(16)
    st = lib.gms_multisplit_wide(t.data_ptr() + 4, None, t.data_ptr() + 4 + 8 * 500, None, 100, 8, 0,
                                 ctypes.byref(d), ctx.d_temp_storage.data_ptr(), ctx.temp_storage_bytes, None,
                                 torch.cuda.current_stream().cuda_stream)
    assert st == gms._lib.GMS_ERROR_INVALID_VALUE


@pytest.mark.parametrize("B", [7, 32, 256])
@pytest.mark.parametrize("kind", [0, 1, 2, 3, 4, 5], ids=lambda k: KIND_NAMES[k])
def test_u64_histogram(gms_lib, oracle_mod, B, kind):
    """Histogram of 64-bit keys: B bins, the words after them untouched; an
    array 8- but not 16-byte aligned takes the element loads."""
    o = oracle_mod
    if kind == o.BITS and B & (B - 1):
        pytest.skip("bit-field buckets are powers of two")
    ident, d, keep = identifiers64(o, kind, B, seed=B)
    n = 300007
    keys = datagen.as_u64(datagen.uniform_u64(n, 70 + B + kind))
    want = o.histogram64(keys, d)
    for pad in (0, 1):
        buf = torch.full((B + 64,), -7, dtype=torch.int32, device="cuda")
        buf[:B].zero_()
        gms.multisplit_histogram_wide(dev64(keys, pad), n, buf[:B], B, ident)
        got = buf.cpu().numpy()
        np.testing.assert_array_equal(got[:B], want)
        assert (got[B:] == -7).all()
    del keep


def test_histogram_wide_32bit_keys_is_the_plain_histogram(gms_lib, oracle_mod):
    o = oracle_mod
    n, B = 100003, 100
    keys = datagen.as_u32(datagen.uniform_u32(n, 5))
    h = torch.zeros(B, dtype=torch.int32, device="cuda")
    gms.multisplit_histogram_wide(to_dev(keys), n, h, B, gms.delta_bucket())
    np.testing.assert_array_equal(h.cpu().numpy(), o.histogram(keys, o.Desc(o.DELTA, B)))
