"""The CPU oracle, pinned against golden vectors produced by the reference's own
CPU multisplit (tests/golden/make_golden.py), and against that reference code
directly where it is built (oracle/_ref, only where the reference tree exists)."""
import hashlib

import numpy as np
import pytest

from gpumultisplit_gb300 import datagen


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a, dtype=np.uint32).tobytes()).hexdigest()


def gen_keys(case):
    dist, n, seed = case["dist"], case["n"], case.get("seed", 0)
    if dist == "explicit":
        return np.array(case["keys_in"], np.uint32)
    if dist == "uniform":
        return datagen.as_u32(datagen.uniform_u32(n, seed))
    if dist == "zipf":
        return datagen.as_u32(datagen.zipf_u32(n, seed, distinct=1 << 12))
    if dist == "and4":
        return datagen.as_u32(datagen.and4_u32(n, seed))
    if dist == "iota":
        return np.arange(n, dtype=np.uint32)
    raise ValueError(dist)


def desc_of(o, case):
    spl = None
    if case.get("kind") == o.RANGE:
        spl = datagen.as_u32(datagen.range_splitters(case["buckets"], case["splitter_seed"]))
    return o.Desc(case["kind"], case["buckets"], shift=case.get("shift", 0), param=case.get("param", 0),
                  lower=case.get("lower", 0), inverse_delta=case.get("inverse_delta", 0.0), splitters=spl)


def test_golden_inputs_regenerate(golden):
    for case in golden:
        assert sha(gen_keys(case)) == case["input_sha256"], case["name"]


def test_oracle_matches_golden(golden, oracle_mod):
    o = oracle_mod
    for case in golden:
        keys = gen_keys(case)
        vals = np.arange(case["n"], dtype=np.uint32) if case["values"] else None
        if case["op"] == "multisplit":
            ko, vo, offs = o.multisplit(keys, desc_of(o, case), vals)
            if "offsets" in case:
                assert [int(x) for x in offs] == case["offsets"], case["name"]
            if "offsets_sha256" in case:
                assert sha(np.asarray(offs, dtype=np.uint32)) == case["offsets_sha256"], case["name"]
        elif case["op"] == "compaction":
            ko, vo, n0 = o.compaction(keys, desc_of(o, case), vals)
            assert n0 == case["num_bucket0"], case["name"]
        elif case["op"] == "sort7":
            ko, vo = o.sort_7bit(keys, vals)
        elif case["op"] == "sort":
            ko, vo = o.sort(keys, vals, case["digit_bits"])
        else:
            raise AssertionError(case["op"])
        assert sha(ko) == case["keys_out_sha256"], case["name"]
        if vals is not None:
            assert sha(vo) == case["values_out_sha256"], case["name"]
        if "keys_out" in case:
            assert [int(x) for x in ko] == case["keys_out"], case["name"]


def test_known_answer_delta_func(oracle_mod):
    """keys 7 1 6 2 5 3 4 0, bucket a/2, B=4 -> 1 0 2 3 5 4 7 6 (reference CPU output)."""
    o = oracle_mod
    ko, _, offs = o.multisplit(np.array([7, 1, 6, 2, 5, 3, 4, 0], np.uint32), o.Desc(o.DIV, 4, param=2))
    assert list(ko) == [1, 0, 2, 3, 5, 4, 7, 6]
    assert list(offs) == [0, 2, 4, 6]


def test_even_float_edges(oracle_mod):
    """Float binning of the reference's even histogram (multisplit2_histograms.cuh:60):
    keys >= 2^32-128 round to 2^32 -> bin 256 -> wraps to 0; 2^24-1 rounds exactly."""
    o = oracle_mod
    d = o.Desc(o.EVEN_FLOAT, 256, inverse_delta=2.0 ** -24)
    keys = np.array([2**32 - 1, 2**32 - 128, 2**32 - 129, 2**24 - 1, 2**24, 2**25 - 1], np.uint32)
    assert list(o.buckets(keys, d)) == [0, 0, 255, 0, 1, 2]


def test_range_below_first_splitter_wraps(oracle_mod):
    o = oracle_mod
    d = o.Desc(o.RANGE, 4, splitters=np.array([10, 20, 30, 40], np.uint32))
    assert list(o.buckets(np.array([0, 9, 10, 19, 20, 39, 40, 2**32 - 1], np.uint32), d)) == [3, 3, 0, 0, 1, 2, 3, 3]


def test_tile_counts_layout(oracle_mod):
    o = oracle_mod
    keys = datagen.as_u32(datagen.uniform_u32(10000, 3))
    d = o.Desc(o.DELTA, 16)
    c = o.tile_counts(keys, d, 4096)
    assert c.shape == (16, 3)
    ids = keys >> np.uint32(28)
    for t in range(3):
        np.testing.assert_array_equal(c[:, t], np.bincount(ids[t * 4096:(t + 1) * 4096], minlength=16))


def test_multithreaded_port_matches(oracle_mod):
    o = oracle_mod
    keys = datagen.as_u32(datagen.zipf_u32(200003, 4, distinct=1 << 10))
    vals = np.arange(keys.size, dtype=np.uint32)
    for d in (o.Desc(o.DELTA, 256), o.Desc(o.BITS, 2), o.Desc(o.DIV, 32, param=1 << 27)):
        ko, vo, _ = o.multisplit(keys, d, vals)
        mk, mv = o.multisplit_mt(keys, d, vals, threads=5)
        assert np.array_equal(ko, mk) and np.array_equal(vo, mv)


@pytest.mark.parametrize("bits", [4, 5, 6, 7, 8])
def test_sort_oracle_is_stable_sort(oracle_mod, bits):
    o = oracle_mod
    keys = datagen.as_u32(datagen.and4_u32(50000, 9))
    vals = np.arange(keys.size, dtype=np.uint32)
    ko, vo = o.sort(keys, vals, bits)
    assert np.array_equal(ko, np.sort(keys))
    assert np.array_equal(vo, np.argsort(keys, kind="stable"))
    with pytest.raises(ValueError):
        o.sort(keys, vals, 3)


@pytest.mark.skipif("not __import__('oracle').ref_available()", reason="reference CPU library not built here")
def test_oracle_matches_reference_code(oracle_mod):
    """Random cases: the C restatement equals the reference's own CPU multisplit."""
    o = oracle_mod
    rng = np.random.default_rng(0)
    for trial in range(40):
        B = int(2 ** rng.integers(1, 9))
        n = int(rng.integers(0, 5000))
        kind = int(rng.integers(0, 6))
        keys = rng.integers(0, 2**32, n, dtype=np.uint64).astype(np.uint32)
        vals = np.arange(n, dtype=np.uint32)
        spl = np.sort(rng.integers(0, 2**32, B, dtype=np.uint64).astype(np.uint32))
        d = o.Desc(kind, B, shift=int(rng.integers(0, 32)), param=int(rng.integers(1, 2**32)),
                   lower=int(rng.integers(0, 2**32)), inverse_delta=float(B) / 2**32, splitters=spl)
        ko, vo, _ = o.multisplit(keys, d, vals)
        rk, rv = o.ref_multisplit(keys, d, vals)
        assert np.array_equal(ko, rk) and np.array_equal(vo, rv), (trial, kind, B, n)


@pytest.mark.parametrize("begin,end,digit", [(0, 32, 8), (0, 8, 4), (3, 17, 5), (20, 21, 6), (9, 9, 7), (12, 32, 7)])
def test_partial_key_sort_oracle(oracle_mod, begin, end, digit):
    """Stable sort by bits [begin, end) equals numpy's stable argsort on those bits."""
    keys = datagen.as_u32(datagen.uniform_u32(30011, 77))
    vals = np.arange(keys.size, dtype=np.uint32)
    ko, vo = oracle_mod.sort_bits(keys, vals, begin, end, digit)
    field = (keys.astype(np.uint64) >> begin) & ((1 << (end - begin)) - 1)
    order = np.argsort(field, kind="stable")
    assert np.array_equal(vo, order.astype(np.uint32))
    assert np.array_equal(ko, keys[order])
    with pytest.raises(ValueError):
        oracle_mod.sort_bits(keys, vals, 5, 4, 8)


def test_oracle_buckets_any_count(oracle_mod):
    """Bucket counts that are not powers of two: every id is below B, and the
    identifiers agree with their definitions."""
    o = oracle_mod
    keys = datagen.as_u32(datagen.uniform_u32(4000, 31))
    keys[:3] = [0, 0xFFFFFFFF, 0x80000000]
    for B in (3, 5, 12, 100, 255):
        k64 = keys.astype(np.uint64)
        assert np.array_equal(o.buckets(keys, o.Desc(o.DELTA, B)), (k64 * B >> 32).astype(np.uint32))
        assert np.array_equal(o.buckets(keys, o.Desc(o.DIV, B, param=77777)), (keys // 77777) % B)
        spl = np.concatenate([[0], np.sort(datagen.as_u32(datagen.uniform_u32(B - 1, B)))]).astype(np.uint32)
        ub = np.searchsorted(spl, keys, side="right").astype(np.int64) - 1
        assert np.array_equal(o.buckets(keys, o.Desc(o.RANGE, B, splitters=spl)), np.where(ub < 0, B - 1, ub))
        assert o.buckets(keys, o.Desc(o.EVEN_FLOAT, B, inverse_delta=B / 2**32)).max() < B
        if o.ref_available():
            vals = np.arange(keys.size, dtype=np.uint32)
            d = o.Desc(o.RANGE, B, splitters=spl)
            ko, vo, _ = o.multisplit(keys, d, vals)
            rk, rv = o.ref_multisplit(keys, d, vals)
            assert np.array_equal(ko, rk) and np.array_equal(vo, rv)


def test_oracle_64bit_keys_against_numpy(oracle_mod):
    """The 64-bit restatement equals an independent one: numpy's stable argsort
    of the bucket ids (multisplit) and of the key bits (sort)."""
    o = oracle_mod
    keys = datagen.as_u64(datagen.uniform_u64(6000, 17))
    keys[:4] = [0, 2**64 - 1, 2**63, 2**32 - 1]
    vals = np.arange(keys.size, dtype=np.uint64) * np.uint64(3)
    for B in (2, 3, 100, 256):
        k = [int(x) for x in keys]
        spl = np.concatenate([[0], np.sort(datagen.as_u64(datagen.uniform_u64(B - 1, B)))]).astype(np.uint64)
        ub = np.searchsorted(spl, keys, side="right").astype(np.int64) - 1
        cases = [
            (o.Desc64(o.DELTA, B), np.array([(x * B) >> 64 for x in k])),
            (o.Desc64(o.DIV, B, param=(1 << 60) + 12345), np.array([(x // ((1 << 60) + 12345)) % B for x in k])),
            (o.Desc64(o.RANGE, B, splitters=spl), np.where(ub < 0, B - 1, ub)),
            (o.Desc64(o.MASK, B, param=1 << 45), np.array([1 if x & (1 << 45) else 0 for x in k])),
        ]
        if B & (B - 1) == 0:
            cases.append((o.Desc64(o.BITS, B, shift=40), np.array([(x >> 40) % B for x in k])))
        for d, ids in cases:
            assert np.array_equal(o.buckets64(keys, d), ids.astype(np.uint32))
            ko, vo, offs = o.multisplit64(keys, d, vals)
            order = np.argsort(ids, kind="stable")
            assert np.array_equal(ko, keys[order]) and np.array_equal(vo, vals[order])
            assert np.array_equal(offs, np.searchsorted(np.sort(ids), np.arange(B)).astype(np.uint32))
        f = o.buckets64(keys, o.Desc64(o.EVEN_FLOAT, B, lower=2**40, inverse_delta=B / 2**64))
        assert f.max() < B
        assert np.array_equal(o.histogram64(keys, o.Desc64(o.DELTA, B)),
                              np.bincount(cases[0][1].astype(np.int64), minlength=B).astype(np.int32))
    ks, vs = o.sort_bits64(keys, vals, 0, 64, 8)
    assert np.array_equal(ks, np.sort(keys)) and np.array_equal(vs, vals[np.argsort(keys, kind="stable")])
    ks, vs = o.sort_bits64(keys, vals.astype(np.uint32), 13, 47, 7)
    sub = (keys >> np.uint64(13)) & np.uint64((1 << 34) - 1)
    assert np.array_equal(vs, vals.astype(np.uint32)[np.argsort(sub, kind="stable")])


def test_oracle_more_than_256_buckets(oracle_mod):
    """B above 256: the oracle's ids and order against numpy, and against the
    reference's CPU multisplit where it is built (it takes any bucket count)."""
    o = oracle_mod
    keys = datagen.as_u32(datagen.uniform_u32(20000, 41))
    keys[:3] = [0, 0xFFFFFFFF, 0x80000000]
    vals = np.arange(keys.size, dtype=np.uint32)
    for B in (257, 1000, 4096, 65536):
        spl = np.concatenate([[0], np.sort(datagen.as_u32(datagen.uniform_u32(B - 1, B)))]).astype(np.uint32)
        ub = np.searchsorted(spl, keys, side="right").astype(np.int64) - 1
        for d, ids in ((o.Desc(o.DELTA, B), (keys.astype(np.uint64) * B) >> 32),
                       (o.Desc(o.RANGE, B, splitters=spl), np.where(ub < 0, B - 1, ub)),
                       (o.Desc(o.DIV, B, param=4099), (keys // 4099) % B)):
            ko, vo, offs = o.multisplit(keys, d, vals)
            order = np.argsort(ids, kind="stable")
            assert np.array_equal(ko, keys[order]) and np.array_equal(vo, order)
            assert np.array_equal(offs, np.searchsorted(np.sort(ids), np.arange(B)).astype(np.uint32))
            if o.ref_available():
                rk, rv = o.ref_multisplit(keys, d, vals)
                assert np.array_equal(rk, ko) and np.array_equal(rv, vo)


def test_oracle_random_cases_against_numpy(oracle_mod):
    """Seeded random cases (kind, B from 2 to 65536, n, skew): the oracle's
    multisplit equals numpy's stable argsort of the ids numpy computes itself."""
    o = oracle_mod
    rng = np.random.default_rng(2024)
    for trial in range(40):
        B = int(rng.choice([2, 3, 7, 16, 100, 255, 256, 257, 1000, 4096, 65536]))
        kind = int(rng.choice([o.DELTA, o.DIV, o.RANGE, o.MASK] + ([o.BITS] if B & (B - 1) == 0 else [])))
        n = int(rng.integers(0, 5000))
        keys = rng.integers(0, 2**32, n, dtype=np.uint64).astype(np.uint32)
        if trial % 3 == 0:
            keys = keys & np.uint32(0xFFF0000F)  # many repeated high parts
        k64 = keys.astype(np.uint64)
        if kind == o.DELTA:
            d, ids = o.Desc(o.DELTA, B), (k64 * B) >> 32
        elif kind == o.DIV:
            p = int(rng.integers(1, 2**20))
            d, ids = o.Desc(o.DIV, B, param=p), (k64 // p) % B
        elif kind == o.BITS:
            sh = int(rng.integers(0, 32))
            d, ids = o.Desc(o.BITS, B, shift=sh), (k64 >> sh) % B
        elif kind == o.MASK:
            m = int(rng.integers(1, 2**32))
            d, ids = o.Desc(o.MASK, B, param=m), (k64 & m != 0).astype(np.uint64)
        else:
            spl = np.sort(rng.integers(0, 2**32, B, dtype=np.uint64)).astype(np.uint32)
            ub = np.searchsorted(spl, keys, side="right").astype(np.int64) - 1
            d, ids = o.Desc(o.RANGE, B, splitters=spl), np.where(ub < 0, B - 1, ub).astype(np.uint64)
        vals = np.arange(n, dtype=np.uint32)
        ko, vo, offs = o.multisplit(keys, d, vals)
        order = np.argsort(ids, kind="stable")
        assert np.array_equal(ko, keys[order]) and np.array_equal(vo, order.astype(np.uint32)), (trial, kind, B)
        assert np.array_equal(offs, np.searchsorted(np.sort(ids), np.arange(B)).astype(np.uint32)), (trial, kind, B)
