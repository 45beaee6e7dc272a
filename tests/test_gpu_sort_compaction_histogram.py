"""GPU parity of the multisplit radix sorts (4- to 8-bit digits), the two-bucket compaction and
the histogram entry points against the CPU oracle (bit-exact)."""
import hashlib

import numpy as np
import pytest
import torch

import gpumultisplit_gb300 as gms
from gpumultisplit_gb300 import datagen
from gpu_util import KIND_NAMES, host, identifiers, to_dev

pytestmark = pytest.mark.gpu


def sort_gpu(keys, values=None, misalign=0, bits=7):
    n = keys.size
    dk, ok = to_dev(keys, misalign), to_dev(np.zeros(n, np.uint32), misalign)
    ctx = gms.ms_sort_context()
    fn = f"multisplit_sort_{bits}bit"
    if values is None:
        getattr(gms, fn + "_allocate")(n, ctx)
        getattr(gms, fn)(dk, ok, n, ctx)
        torch.cuda.synchronize()
        out = host(ok), None
    else:
        dv, ov = to_dev(values, misalign), to_dev(np.zeros(n, np.uint32), misalign)
        getattr(gms, fn + "_allocate_pairs")(n, ctx)
        getattr(gms, fn + "_pairs")(dk, ok, dv, ov, n, ctx)
        torch.cuda.synchronize()
        out = host(ok), host(ov)
    # the input is not modified (src/api/multisplit_sort.cuh:340-363 never writes d_key_in)
    np.testing.assert_array_equal(host(dk), keys)
    return out


@pytest.mark.parametrize("n", [0, 1, 33, 896, 4097, 100003, 1 << 20])
@pytest.mark.parametrize("dist", ["uniform", "and4"])
def test_sort7_keys_and_pairs(gms_lib, oracle_mod, n, dist):
    gen = datagen.uniform_u32 if dist == "uniform" else datagen.and4_u32
    keys = datagen.as_u32(gen(n, 40 + n))
    vals = np.arange(n, dtype=np.uint32)
    gk, _ = sort_gpu(keys)
    np.testing.assert_array_equal(gk, np.sort(keys))
    gk, gv = sort_gpu(keys, vals)
    rk, rv = oracle_mod.sort_7bit(keys, vals)
    np.testing.assert_array_equal(gk, rk)
    np.testing.assert_array_equal(gv, rv)
    np.testing.assert_array_equal(gv, np.argsort(keys, kind="stable"))


def test_sort7_misaligned(gms_lib):
    keys = datagen.as_u32(datagen.uniform_u32(30001, 3))
    gk, gv = sort_gpu(keys, np.arange(keys.size, dtype=np.uint32), misalign=1)
    np.testing.assert_array_equal(gk, np.sort(keys))
    np.testing.assert_array_equal(gv, np.argsort(keys, kind="stable"))


@pytest.mark.parametrize("bits", [4, 5, 6, 8])
@pytest.mark.parametrize("n", [0, 1, 4097, 100003, 1 << 20])
def test_sort_other_widths(gms_lib, oracle_mod, bits, n):
    """multisplit_sort_{4,5,6,8}bit[_pairs] (src/api/multisplit_sort.cuh:366-559,
    src/api/multisplit_sort_pairs.cuh:67-260)."""
    keys = datagen.as_u32(datagen.uniform_u32(n, 300 + bits + n))
    vals = np.arange(n, dtype=np.uint32)
    gk, _ = sort_gpu(keys, bits=bits)
    np.testing.assert_array_equal(gk, np.sort(keys))
    gk, gv = sort_gpu(keys, vals, misalign=bits & 1, bits=bits)
    rk, rv = oracle_mod.sort(keys, vals, bits)
    np.testing.assert_array_equal(gk, rk)
    np.testing.assert_array_equal(gv, rv)


@pytest.mark.parametrize("begin,end,digit", [(0, 32, 8), (0, 8, 4), (3, 17, 5), (20, 21, 6), (9, 9, 7),
                                              (12, 32, 7)])
@pytest.mark.parametrize("n", [0, 1, 4097, 300007])
def test_partial_key_sort(gms_lib, oracle_mod, begin, end, digit, n):
    """Stable sort by key bits [begin, end) (the CUB begin/end-bit form)."""
    keys = datagen.as_u32(datagen.uniform_u32(n, 500 + n + begin))
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
    ok2 = to_dev(np.zeros(n, np.uint32))
    ctx2 = gms.ms_sort_context()
    gms.multisplit_sort_bits_allocate(n, ctx2, begin, end, digit)
    gms.multisplit_sort_bits(dk, ok2, n, ctx2)
    torch.cuda.synchronize()
    np.testing.assert_array_equal(host(ok2), rk)
    np.testing.assert_array_equal(host(dk), keys)


def test_sort7_golden(gms_lib, golden):
    from test_oracle_golden import gen_keys, sha

    for case in golden:
        if case["op"] not in ("sort7", "sort"):
            continue
        keys = gen_keys(case)
        vals = np.arange(case["n"], dtype=np.uint32) if case["values"] else None
        gk, gv = sort_gpu(keys, vals, bits=case.get("digit_bits", 7))
        assert sha(gk) == case["keys_out_sha256"], case["name"]
        if vals is not None:
            assert sha(gv) == case["values_out_sha256"], case["name"]


@pytest.mark.parametrize("n", [0, 1, 2, 383, 384, 385, 4096, 100001, 1 << 20])
@pytest.mark.parametrize("with_values", [False, True], ids=["keys", "pairs"])
def test_compaction_key_and_1(gms_lib, oracle_mod, n, with_values):
    """test_bucket<1> = key & 1 (src/main/main_compaction.cu:26-31): even keys first."""
    o = oracle_mod
    keys = datagen.as_u32(datagen.uniform_u32(n, 60 + n))
    vals = np.arange(n, dtype=np.uint32) if with_values else None
    dk, ok = to_dev(keys), to_dev(np.zeros(n, np.uint32))
    ctx = gms.compaction_context()
    if with_values:
        dv, ov = to_dev(vals), to_dev(np.zeros(n, np.uint32))
        gms.compaction_allocate_key_value(n, ctx)
        n0 = gms.compaction_key_value(dk, dv, ok, ov, n, ctx, gms.test_bucket(1))
    else:
        gms.compaction_allocate_key_only(n, ctx)
        n0 = gms.compaction_key_only(dk, ok, n, ctx, gms.test_bucket(1))
    rk, rv, r0 = o.compaction(keys, o.Desc(o.BITS, 2), vals)
    assert n0 == r0 == int(np.count_nonzero((keys & 1) == 0))
    np.testing.assert_array_equal(host(ok), rk)
    if with_values:
        np.testing.assert_array_equal(host(ov), rv)


def test_compaction_golden(gms_lib, golden):
    from test_oracle_golden import gen_keys, sha

    for case in golden:
        if case["op"] != "compaction":
            continue
        keys = gen_keys(case)
        n = case["n"]
        dk, ok = to_dev(keys), to_dev(np.zeros(n, np.uint32))
        ctx = gms.compaction_context()
        if case["values"]:
            dv, ov = to_dev(np.arange(n, dtype=np.uint32)), to_dev(np.zeros(n, np.uint32))
            gms.compaction_allocate_key_value(n, ctx)
            n0 = gms.compaction_key_value(dk, dv, ok, ov, n, ctx, gms.test_bucket(1))
            assert sha(host(ov)) == case["values_out_sha256"]
        else:
            gms.compaction_allocate_key_only(n, ctx)
            n0 = gms.compaction_key_only(dk, ok, n, ctx, gms.test_bucket(1))
        assert n0 == case["num_bucket0"]
        assert sha(host(ok)) == case["keys_out_sha256"]


@pytest.mark.parametrize("B", [2, 4, 8, 16, 32, 64, 128, 256])
@pytest.mark.parametrize("kind", [0, 1, 2, 3, 4, 5], ids=lambda k: KIND_NAMES[k])
def test_histogram_matches_oracle(gms_lib, oracle_mod, B, kind):
    o = oracle_mod
    for n, dist in ((1, "u"), (4097, "u"), (300007, "u"), (200003, "z")):
        keys = datagen.as_u32(datagen.uniform_u32(n, B + kind) if dist == "u"
                              else datagen.zipf_u32(n, B + kind, distinct=1 << 16))
        ident, d, keep = identifiers(o, kind, B)
        hist = torch.zeros(B, dtype=torch.int32, device="cuda")
        gms.multisplit_histogram(to_dev(keys), n, hist, B, ident)
        np.testing.assert_array_equal(hist.cpu().numpy(), o.histogram(keys, d))


def test_histogram_accumulates_and_misaligned(gms_lib, oracle_mod):
    o = oracle_mod
    keys = datagen.as_u32(datagen.uniform_u32(99999, 5))
    hist = torch.full((64,), 7, dtype=torch.int32, device="cuda")
    gms.multisplit_histogram(to_dev(keys, 3), keys.size, hist, 64, gms.delta_bucket())
    np.testing.assert_array_equal(hist.cpu().numpy(), o.histogram(keys, o.Desc(o.DELTA, 64)) + 7)


def test_histogram_even_and_range_entry_points(gms_lib, oracle_mod):
    """histogram_even bins like multisplit2_histogram_even_256bin_128 (float math,
    top keys wrap to bin 0); histogram_range like the _range_ kernels."""
    o = oracle_mod
    n = 1 << 20
    keys = datagen.as_u32(datagen.uniform_u32(n, 8))
    keys[:4] = [2**32 - 1, 2**32 - 128, 2**32 - 129, 2**24 - 1]
    hist = torch.zeros(256, dtype=torch.int32, device="cuda")
    gms.histogram_even(to_dev(keys), n, hist, 256, 0, 0xFFFFFFFF, 2.0 ** -24)
    np.testing.assert_array_equal(hist.cpu().numpy(), o.histogram(keys, o.Desc(o.EVEN_FLOAT, 256,
                                                                                 inverse_delta=2.0 ** -24)))
    levels = datagen.range_splitters(256, 9)
    hist.zero_()
    gms.histogram_range(to_dev(keys), n, hist, 256, levels.cuda())
    np.testing.assert_array_equal(hist.cpu().numpy(),
                                  o.histogram(keys, o.Desc(o.RANGE, 256, splitters=datagen.as_u32(levels))))
    # integer definition: same identifier as the multisplit -> equals its bucket sizes
    hist.zero_()
    gms.multisplit_histogram(to_dev(keys), n, hist, 256, gms.delta_bucket())
    _, _, offs = o.multisplit(keys, o.Desc(o.DELTA, 256))
    sizes = np.diff(np.append(offs.astype(np.int64), n))
    np.testing.assert_array_equal(hist.cpu().numpy(), sizes)
