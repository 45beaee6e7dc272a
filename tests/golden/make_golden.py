"""Generates tests/golden/golden.json from the REFERENCE's own CPU code.

Run here, where the reference tree exists (the script builds oracle/_ref from
its sources first):  python tests/golden/make_golden.py

Every case records its inputs by generator + seed (gpumultisplit_gb300.datagen,
a counter-based splitmix64 generator) together with the SHA-256 of the input,
and the reference's outputs: full arrays for tiny cases, SHA-256 digests plus
bucket offsets for the rest (a digest of the offsets above 256 buckets).  Outputs come from cpu_multisplit_general /
cpu_multisplit_pairs_general (src/cpu_functions.h:155-288) compiled from the
reference sources, driven either by reference-style functors (key*B>>32 as top
bits, delta_func's key/delta, ms_bucket_sort's bit field) or by the oracle's
bucket function (range, mask, even-float identifiers).  The sort cases
run the reference's digit schedules (src/api/multisplit_sort.cuh:320-559) on
that same reference CPU multisplit and are checked against numpy's stable sort.
"""
from __future__ import annotations

import hashlib
import json
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

import oracle  # noqa: E402
from gpumultisplit_gb300 import datagen  # noqa: E402

OUT = Path(__file__).resolve().parent / "golden.json"
FULL_MAX = 64


def sha(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a, dtype=np.uint32).tobytes()).hexdigest()


def gen_keys(dist: str, n: int, seed: int) -> np.ndarray:
    if dist == "uniform":
        return datagen.as_u32(datagen.uniform_u32(n, seed))
    if dist == "zipf":
        return datagen.as_u32(datagen.zipf_u32(n, seed, distinct=1 << 12))
    if dist == "and4":
        return datagen.as_u32(datagen.and4_u32(n, seed))
    if dist == "iota":
        return np.arange(n, dtype=np.uint32)
    raise ValueError(dist)


def offsets_of(bucket_ids_sorted: np.ndarray, B: int) -> list[int]:
    counts = np.bincount(bucket_ids_sorted.astype(np.int64), minlength=B)
    return [int(x) for x in np.concatenate([[0], np.cumsum(counts)[:-1]])]


def record(case: dict, keys: np.ndarray, kout: np.ndarray, vout, offsets) -> dict:
    case = dict(case)
    case["input_sha256"] = sha(keys)
    case["keys_out_sha256"] = sha(kout)
    if vout is not None:
        case["values_out_sha256"] = sha(vout)
    if keys.size <= FULL_MAX:
        case["keys_in"] = [int(x) for x in keys]
        case["keys_out"] = [int(x) for x in kout]
        if vout is not None:
            case["values_out"] = [int(x) for x in vout]
    if offsets is not None:
        if len(offsets) > 256:  # above 256 buckets: a digest of the offsets keeps the file small
            case["offsets_sha256"] = sha(np.array(offsets, dtype=np.uint32))
        else:
            case["offsets"] = offsets
    return case


def desc_from(case: dict) -> oracle.Desc:
    spl = None
    if case["kind"] == oracle.RANGE:
        spl = datagen.as_u32(datagen.range_splitters(case["buckets"], case["splitter_seed"]))
    return oracle.Desc(case["kind"], case["buckets"], shift=case.get("shift", 0), param=case.get("param", 0),
                       lower=case.get("lower", 0), inverse_delta=case.get("inverse_delta", 0.0), splitters=spl)


def main() -> None:
    oracle.build(with_ref=True)
    assert oracle.ref_available(), "reference CPU library missing"
    cases = []

    # Known answer from the reference's own CPU multisplit: keys 7 1 6 2 5 3 4 0, a/2, B=4.
    k = np.array([7, 1, 6, 2, 5, 3, 4, 0], np.uint32)
    ko, _ = oracle.ref_multisplit_functor(k, 1, 4, 2)
    assert list(ko) == [1, 0, 2, 3, 5, 4, 7, 6]
    cases.append(record({"name": "kat_delta_func_b4", "op": "multisplit", "dist": "explicit", "n": 8,
                         "kind": oracle.DIV, "buckets": 4, "param": 2, "values": False}, k, ko, None,
                        offsets_of(ko // 2, 4)))

    # Reference-functor multisplits (the functor is the reference's own style).
    functor_cases = [
        # config 1: 2^20 uniform keys, seed 1, B = 8, key >> 29
        ("config1_keys_b8", "uniform", 1 << 20, 1, 0, 8, 0, False),
        ("delta_b256_pairs", "uniform", 100003, 2, 0, 256, 0, True),
        ("delta_b2_pairs", "uniform", 4097, 3, 0, 2, 0, True),
        ("delta_b32_keys", "uniform", 33, 4, 0, 32, 0, False),
        ("delta_b64_pairs_zipf", "zipf", 70001, 5, 0, 64, 0, True),
        ("delta_b128_keys_zipf", "zipf", 65536, 6, 0, 128, 0, False),
        ("div_b16_pairs", "iota", 50000, 0, 1, 16, 3125, True),
        ("div_b32_keys", "uniform", 31, 8, 1, 32, 134217728, False),
        ("bits_b128_shift11_pairs", "uniform", 12345, 9, 2, 128, 11, True),
        ("bits_b16_shift0_keys", "uniform", 4096, 10, 2, 16, 0, False),
    ]
    kind_map = {0: oracle.DELTA, 1: oracle.DIV, 2: oracle.BITS}
    for name, dist, n, seed, fkind, B, param, with_values in functor_cases:
        keys = gen_keys(dist, n, seed)
        vals = np.arange(n, dtype=np.uint32) if with_values else None
        ko, vo = oracle.ref_multisplit_functor(keys, fkind, B, param, vals)
        case = {"name": name, "op": "multisplit", "dist": dist, "n": n, "seed": seed, "kind": kind_map[fkind],
                "buckets": B, "values": with_values}
        if fkind == 1:
            case["param"] = param
        if fkind == 2:
            case["shift"] = param
        logb = B.bit_length() - 1
        ids = {0: lambda a: a >> np.uint32(32 - logb), 1: lambda a: (a // np.uint32(param)) & np.uint32(B - 1),
               2: lambda a: (a >> np.uint32(param)) & np.uint32(B - 1)}[fkind](ko)
        cases.append(record(case, keys, ko, vo, offsets_of(ids, B)))

    # Descriptor identifiers (range / mask / even-float) through the reference CPU multisplit.
    desc_cases = [
        {"name": "range_b256_pairs", "dist": "uniform", "n": 100000, "seed": 11, "kind": oracle.RANGE,
         "buckets": 256, "splitter_seed": 12, "values": True},
        {"name": "range_b8_keys_zipf", "dist": "zipf", "n": 9999, "seed": 13, "kind": oracle.RANGE, "buckets": 8,
         "splitter_seed": 14, "values": False},
        {"name": "mask_b2_pairs", "dist": "uniform", "n": 20000, "seed": 15, "kind": oracle.MASK, "buckets": 2,
         "param": 0x10, "values": True},
        {"name": "even_float_b256_pairs", "dist": "uniform", "n": 100000, "seed": 16, "kind": oracle.EVEN_FLOAT,
         "buckets": 256, "lower": 0, "inverse_delta": 2.0 ** -24, "values": True},
        {"name": "even_float_b32_keys", "dist": "uniform", "n": 5000, "seed": 17, "kind": oracle.EVEN_FLOAT,
         "buckets": 32, "lower": 1000, "inverse_delta": 32.0 / 4294967296.0, "values": False},
        # Bucket counts the reference's GPU API does not take (powers of two to 256
        # only); its CPU multisplit takes any count, so the order is still its own.
        {"name": "delta_b12_pairs", "dist": "uniform", "n": 30011, "seed": 41, "kind": oracle.DELTA, "buckets": 12,
         "values": True},
        {"name": "div_b5_keys", "dist": "uniform", "n": 7777, "seed": 42, "kind": oracle.DIV, "buckets": 5,
         "param": 100003, "values": False},
        {"name": "range_b100_pairs_zipf", "dist": "zipf", "n": 20001, "seed": 43, "kind": oracle.RANGE,
         "buckets": 100, "splitter_seed": 44, "values": True},
        {"name": "delta_b1000_pairs", "dist": "uniform", "n": 50001, "seed": 45, "kind": oracle.DELTA,
         "buckets": 1000, "values": True},
        {"name": "range_b4096_pairs", "dist": "uniform", "n": 60000, "seed": 46, "kind": oracle.RANGE,
         "buckets": 4096, "splitter_seed": 47, "values": True},
        {"name": "delta_b65536_keys", "dist": "uniform", "n": 100000, "seed": 48, "kind": oracle.DELTA,
         "buckets": 65536, "values": False},
    ]
    for case in desc_cases:
        case = dict(case, op="multisplit")
        keys = gen_keys(case["dist"], case["n"], case["seed"])
        vals = np.arange(case["n"], dtype=np.uint32) if case["values"] else None
        d = desc_from(case)
        ko, vo = oracle.ref_multisplit(keys, d, vals)
        cases.append(record(case, keys, ko, vo, offsets_of(oracle.buckets(ko, d), case["buckets"])))

    # Even-float edge keys: the top keys round to 2^32 and wrap to bin 0.
    edge = np.array([0, 1, 2**24 - 1, 2**24, 2**24 + 1, 2**31, 2**32 - 129, 2**32 - 128, 2**32 - 1, 12345678,
                     2**25 - 1, 2**25], np.uint32)
    case = {"name": "even_float_b256_edges", "op": "multisplit", "dist": "explicit", "n": int(edge.size),
            "kind": oracle.EVEN_FLOAT, "buckets": 256, "lower": 0, "inverse_delta": 2.0 ** -24, "values": True}
    d = desc_from(case)
    ko, vo = oracle.ref_multisplit(edge, d, np.arange(edge.size, dtype=np.uint32))
    cases.append(record(case, edge, ko, vo, offsets_of(oracle.buckets(ko, d), 256)))

    # Compaction: key & 1 (test_bucket<1>, src/main/main_compaction.cu:26-31), bucket-0 count.
    for name, n, seed, with_values in (("compaction_keys", 30001, 21, False), ("compaction_pairs", 4096, 22, True)):
        keys = gen_keys("uniform", n, seed)
        vals = np.arange(n, dtype=np.uint32) if with_values else None
        ko, vo = oracle.ref_multisplit_functor(keys, 2, 2, 0, vals)
        case = {"name": name, "op": "compaction", "dist": "uniform", "n": n, "seed": seed, "kind": oracle.BITS,
                "buckets": 2, "shift": 0, "values": with_values}
        rec = record(case, keys, ko, vo, None)
        rec["num_bucket0"] = int(np.count_nonzero((keys & 1) == 0))
        cases.append(rec)

    # 7-bit sort: the reference's digit schedule on the reference's CPU multisplit.
    for name, dist, n, seed, with_values in (("sort7_keys_uniform", "uniform", 100000, 31, False),
                                             ("sort7_pairs_and4", "and4", 65537, 32, True),
                                             ("sort7_pairs_uniform_small", "uniform", 40, 33, True)):
        keys = gen_keys(dist, n, seed)
        vals = np.arange(n, dtype=np.uint32) if with_values else None
        ko, vo = oracle.ref_sort_7bit(keys, vals)
        assert np.array_equal(ko, np.sort(keys))
        if with_values:
            assert np.array_equal(vo, np.argsort(keys, kind="stable").astype(np.uint32))
        case = {"name": name, "op": "sort7", "dist": dist, "n": n, "seed": seed, "values": with_values}
        cases.append(record(case, keys, ko, vo, None))

    # The other digit widths (src/api/multisplit_sort.cuh:366-559), same check.
    for bits, n, seed in ((4, 50001, 34), (5, 50002, 35), (6, 50003, 36), (8, 50004, 37)):
        keys = gen_keys("uniform", n, seed)
        vals = np.arange(n, dtype=np.uint32)
        ko, vo = oracle.ref_sort(keys, vals, bits)
        assert np.array_equal(ko, np.sort(keys))
        assert np.array_equal(vo, np.argsort(keys, kind="stable").astype(np.uint32))
        case = {"name": f"sort{bits}_pairs_uniform", "op": "sort", "digit_bits": bits, "dist": "uniform", "n": n,
                "seed": seed, "values": True}
        cases.append(record(case, keys, ko, vo, None))

    OUT.write_text(json.dumps({"generator": "tests/golden/make_golden.py", "cases": cases}, indent=1) + "\n")
    print(f"wrote {len(cases)} cases to {OUT}")


if __name__ == "__main__":
    main()
