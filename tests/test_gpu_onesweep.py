"""The two ways the 32-bit radix sorts run their digits give the same bytes.

GMS_SORT_MULTISPLIT runs prescan, scan and postscan per digit, as the
reference's multisplit sorts do (src/api/multisplit_sort.cuh:320-559,
src/api/multisplit_sort_pairs.cuh:21-260); GMS_SORT_ONESWEEP counts every
digit in one histogram pass and finds each tile's offsets by decoupled
look-back.  Both are checked against the CPU oracle's LSD sort, including
sizes far below a tile, ragged last tiles, skewed keys whose digits fall in
one bucket, and partial-key sorts.
"""
import numpy as np
import pytest
import torch

import gpumultisplit_gb300 as gms
from gpumultisplit_gb300 import datagen
from gpu_util import host, to_dev

pytestmark = pytest.mark.gpu


@pytest.fixture
def sort_method():
    def use(method):
        gms.set_sort_method(method)
        assert gms.sort_method() == method

    yield use
    gms.set_sort_method("auto")


def sort_gpu(keys, values, bits):
    n = keys.size
    dk, ok = to_dev(keys), to_dev(np.zeros(n, np.uint32))
    fn = f"multisplit_sort_{bits}bit"
    ctx = gms.ms_sort_context()
    if values is None:
        getattr(gms, fn + "_allocate")(n, ctx)
        getattr(gms, fn)(dk, ok, n, ctx)
        torch.cuda.synchronize()
        assert n == 0 or gms.read_device_error(ctx) == 0
        return host(ok), None
    dv, ov = to_dev(values), to_dev(np.zeros(n, np.uint32))
    getattr(gms, fn + "_allocate_pairs")(n, ctx)
    getattr(gms, fn + "_pairs")(dk, ok, dv, ov, n, ctx)
    torch.cuda.synchronize()
    assert n == 0 or gms.read_device_error(ctx) == 0
    np.testing.assert_array_equal(host(dk), keys)  # the input is not written
    return host(ok), host(ov)


@pytest.mark.parametrize("method", ["multisplit", "onesweep"])
@pytest.mark.parametrize("bits", [4, 5, 6, 7, 8])
@pytest.mark.parametrize("n", [1, 33, 4096, 4097, 70001])
def test_sort_methods_match_oracle(gms_lib, oracle_mod, sort_method, method, bits, n):
    sort_method(method)
    keys = datagen.as_u32(datagen.uniform_u32(n, 900 + bits + n))
    vals = np.arange(n, dtype=np.uint32)
    rk, rv = oracle_mod.sort(keys, vals, bits)
    gk, _ = sort_gpu(keys, None, bits)
    np.testing.assert_array_equal(gk, rk)
    gk, gv = sort_gpu(keys, vals, bits)
    np.testing.assert_array_equal(gk, rk)
    np.testing.assert_array_equal(gv, rv)


@pytest.mark.parametrize("keys_kind", ["all_equal", "two_values", "and4", "one_digit_bucket"])
def test_onesweep_skewed_keys(gms_lib, oracle_mod, sort_method, keys_kind):
    """Digits whose counts are zero in most tiles (the look-back adds zeros) or
    whose one bucket holds every key of a tile."""
    sort_method("onesweep")
    n = 300007
    if keys_kind == "all_equal":
        keys = np.full(n, 0xDEADBEEF, np.uint32)
    elif keys_kind == "two_values":
        keys = np.where(np.arange(n) % 3 == 0, 7, 0xFFFFFFF0).astype(np.uint32)
    elif keys_kind == "and4":
        keys = datagen.as_u32(datagen.and4_u32(n, 5))
    else:  # bits 11..17 constant: one bucket of that 7-bit digit holds everything
        keys = datagen.as_u32(datagen.uniform_u32(n, 6)) & np.uint32(~(0x7F << 11) & 0xFFFFFFFF)
    vals = np.arange(n, dtype=np.uint32)
    rk, rv = oracle_mod.sort(keys, vals, 7)
    gk, gv = sort_gpu(keys, vals, 7)
    np.testing.assert_array_equal(gk, rk)
    np.testing.assert_array_equal(gv, rv)


@pytest.mark.parametrize("begin,end,digit", [(0, 32, 8), (3, 17, 5), (20, 21, 6), (12, 32, 7)])
def test_onesweep_partial_key_sort(gms_lib, oracle_mod, sort_method, begin, end, digit):
    sort_method("onesweep")
    n = 200003
    keys = datagen.as_u32(datagen.uniform_u32(n, 700 + begin))
    vals = np.arange(n, dtype=np.uint32)
    rk, rv = oracle_mod.sort_bits(keys, vals, begin, end, digit)
    dk, ok = to_dev(keys), to_dev(np.zeros(n, np.uint32))
    dv, ov = to_dev(vals), to_dev(np.zeros(n, np.uint32))
    ctx = gms.ms_sort_context()
    gms.multisplit_sort_bits_allocate(n, ctx, begin, end, digit, pairs=True)
    gms.multisplit_sort_bits_pairs(dk, ok, dv, ov, n, ctx)
    torch.cuda.synchronize()
    np.testing.assert_array_equal(host(ok), rk)
    np.testing.assert_array_equal(host(ov), rv)


def test_methods_give_the_same_bytes_at_scale(gms_lib, sort_method):
    """2^24 + 77 pairs, 7-bit digits: one-sweep output equals the multisplit
    passes' output, and it is sorted and stable (values are input indices)."""
    n = (1 << 24) + 77
    keys = datagen.uniform_u32(n, 31, device="cuda")
    vals = datagen.index_values(n, "cuda")
    outs = {}
    for method in ("multisplit", "onesweep"):
        sort_method(method)
        ko, vo = torch.empty_like(keys), torch.empty_like(vals)
        ctx = gms.ms_sort_context()
        gms.multisplit_sort_7bit_allocate_pairs(n, ctx)
        gms.multisplit_sort_7bit_pairs(keys, ko, vals, vo, n, ctx)
        torch.cuda.synchronize()
        assert gms.read_device_error(ctx) == 0
        outs[method] = (ko, vo)
    assert torch.equal(outs["multisplit"][0], outs["onesweep"][0])
    assert torch.equal(outs["multisplit"][1], outs["onesweep"][1])
    u = outs["onesweep"][0].long() & 0xFFFFFFFF
    assert bool((u[1:] >= u[:-1]).all())
    same = u[1:] == u[:-1]
    v = outs["onesweep"][1]
    assert bool((v[1:][same] > v[:-1][same]).all())
    assert torch.equal(keys[v.long()], outs["onesweep"][0])
