"""Batched multisplit: every segment's output equals the plain multisplit of
that segment alone (bit-exact), for mixed bucket counts, identifier kinds,
key-only and key-value segments, empty and tiny segments, with and without
the captured CUDA graph, and across repeated runs."""
import numpy as np
import pytest
import torch

import gpumultisplit_gb300 as gms
from gpumultisplit_gb300 import datagen
from gpu_util import host, identifiers, to_dev

pytestmark = pytest.mark.gpu


def make_segments(o, sizes, seed, kinds=(0, 3), buckets=(2, 8, 32, 256), kv_pattern=None):
    rng = np.random.default_rng(seed)
    segs, refs = [], []
    for i, n in enumerate(sizes):
        B = int(buckets[rng.integers(len(buckets))])
        kind = int(kinds[rng.integers(len(kinds))])
        kv = True if kv_pattern is None else bool(kv_pattern[i % len(kv_pattern)])
        keys = datagen.as_u32(datagen.uniform_u32(int(n), seed * 1000 + i))
        vals = np.arange(n, dtype=np.uint32) if kv else None
        ident, d, keep = identifiers(o, kind, B, splitter_seed=seed + i)
        kin, kout = to_dev(keys), torch.zeros(int(n), dtype=torch.int32, device="cuda")
        vin = to_dev(vals) if kv else None
        vout = torch.zeros(int(n), dtype=torch.int32, device="cuda") if kv else None
        segs.append(gms.Segment(kin, kout, int(n), B, ident, vin, vout))
        refs.append((keys, vals, d, keep))
    return segs, refs


def check_against_oracle(o, segs, refs):
    for s, (keys, vals, d, _) in zip(segs, refs):
        rk, rv, _ = o.multisplit(keys, d, vals)
        np.testing.assert_array_equal(host(s.keys_out), rk)
        if vals is not None:
            np.testing.assert_array_equal(host(s.values_out), rv)


@pytest.mark.parametrize("use_graph", [False, True])
def test_batched_matches_oracle_mixed(gms_lib, oracle_mod, use_graph):
    sizes = [0, 1, 7, 1024, 4095, 4096, 4097, 10000, 65537, 3, 300001, 1 << 17, 2, 99999]
    segs, refs = make_segments(oracle_mod, sizes, 5, kinds=(0, 1, 2, 3, 4, 5),
                               buckets=(2, 4, 8, 16, 32, 64, 128, 256), kv_pattern=(1, 0, 1))
    plan = gms.BatchedMultisplit(segs)
    plan.run(use_graph=use_graph)
    torch.cuda.synchronize()
    assert plan.device_error() == 0
    check_against_oracle(oracle_mod, segs, refs)
    plan.close()


def test_batched_equals_plain_path_and_replays(gms_lib, oracle_mod):
    """Graph replays give the same bytes; outputs equal the plain per-call path."""
    rng = np.random.default_rng(7)
    sizes = np.exp(rng.uniform(np.log(1024), np.log(1 << 18), 200)).astype(np.int64)
    segs, refs = make_segments(oracle_mod, sizes, 7)
    plan = gms.BatchedMultisplit(segs)
    # one prescan and one postscan per (kind, B, key/value, tile variant) class, one scan
    table = gms.tuning_table()
    classes = {(s.identifier.desc(s.num_buckets).kind, s.num_buckets,
                table[(s.num_buckets, True, gms.batched.size_class(s.n))]) for s in segs}
    assert plan.launches == 2 * len(classes) + 1
    for _ in range(3):
        for s in segs:
            s.keys_out.zero_()
            s.values_out.zero_()
        plan.run(use_graph=True)
        torch.cuda.synchronize()
        for s in segs:
            ko, vo = torch.empty_like(s.keys_out), torch.empty_like(s.values_out)
            ctx = gms.multisplit_context(s.num_buckets)
            gms.multisplit_allocate_key_value(s.n, ctx)
            gms.multisplit_key_value(s.keys_in, s.values_in, ko, vo, s.n, ctx, s.identifier)
            torch.cuda.synchronize()
            assert torch.equal(ko, s.keys_out) and torch.equal(vo, s.values_out)
    assert plan.device_error() == 0
    plan.close()


def test_batched_rejects_bad_segments(gms_lib):
    k = torch.zeros(10, dtype=torch.int32, device="cuda")
    with pytest.raises(gms.GmsError):
        gms.BatchedMultisplit([gms.Segment(k, k.clone(), 10, 300, gms.delta_bucket())])
    with pytest.raises(gms.GmsError):  # bit-field buckets need a power of two
        gms.BatchedMultisplit([gms.Segment(k, k.clone(), 10, 3, gms.bits_bucket(0))])
    with pytest.raises(gms.GmsError):
        gms.BatchedMultisplit([gms.Segment(k, k.clone(), 10, 8, gms.delta_func(0))])


def test_batched_empty_plan(gms_lib):
    plan = gms.BatchedMultisplit([])
    plan.run()
    plan.close()


@pytest.mark.parametrize("variant", [0, 1, 2, 3])
def test_batched_each_tile_variant_matches_oracle(gms_lib, oracle_mod, variant):
    """Every tile shape the tuning table can pick gives the oracle's output."""
    warps, ipt, tile = gms.tile_variant_shape(variant)
    assert tile == warps * 32 * ipt
    buckets = tuple(b for b in (2, 8, 32, 128, 256) if b <= warps * 32)
    sizes = [1, 700, 1024, 1025, 2048, 2049, 4097, 30000, 70001, 0, 5]
    segs, refs = make_segments(oracle_mod, sizes, 11 + variant, kinds=(0, 2, 3, 5), buckets=buckets,
                               kv_pattern=(1, 0))
    plan = gms.BatchedMultisplit(segs, variant=variant)
    plan.run(use_graph=True)
    torch.cuda.synchronize()
    assert plan.device_error() == 0
    check_against_oracle(oracle_mod, segs, refs)
    plan.close()


def test_batched_variant_needs_a_thread_per_bucket(gms_lib):
    k = torch.zeros(10, dtype=torch.int32, device="cuda")
    with pytest.raises(gms.GmsError):
        gms.BatchedMultisplit([gms.Segment(k, k.clone(), 10, 256, gms.delta_bucket())], variant=3)


def test_autotune_fills_table_and_keeps_outputs(gms_lib, oracle_mod):
    """The autotuner times every class, stores valid variants, and a plan built
    from the tuned table still gives the oracle's output."""
    gms.reset_tuning()
    try:
        ms = gms.autotune(buckets=(2, 256), key_value=(False, True), keys_per_trial=1 << 20, reps=1)
        assert len(ms) == 2 * 2 * gms.batched.NUM_SIZE_CLASSES
        assert all(t > 0 for t in ms.values())
        table = gms.tuning_table()
        for (b, kv, c), v in table.items():
            assert gms.tile_variant_shape(v)[0] * 32 >= b
        sizes = [1, 900, 1500, 3000, 9000, 40000, 200000]
        segs, refs = make_segments(oracle_mod, sizes, 17, kinds=(0, 3), buckets=(2, 256), kv_pattern=(1, 0, 1))
        plan = gms.BatchedMultisplit(segs)
        plan.run(use_graph=True)
        torch.cuda.synchronize()
        assert plan.device_error() == 0
        check_against_oracle(oracle_mod, segs, refs)
        plan.close()
    finally:
        gms.reset_tuning()


@pytest.mark.parametrize("use_graph", [False, True])
def test_small_segments_one_warp_each(gms_lib, oracle_mod, use_graph):
    """Segments of at most 512 keys take the one-warp path (one launch per class,
    no scan); every kind, power-of-two and other bucket counts, key-only and
    key-value, beside tiled segments: each equals the oracle and the plan with
    a forced tile shape (the tiled path for every segment)."""
    o = oracle_mod
    rng = np.random.default_rng(17)
    sizes = [1, 2, 31, 32, 33, 100, 255, 256, 257, 511, 512, 513, 1000, 5000] + \
        [int(x) for x in rng.integers(1, 513, 120)]
    buckets = (2, 3, 8, 12, 32, 33, 64, 100, 128, 256)
    segs, refs = [], []
    for i, n in enumerate(sizes):
        B = int(buckets[rng.integers(len(buckets))])
        kind = int(rng.integers(6))
        if kind == o.BITS and B & (B - 1):
            kind = o.DELTA  # bit-field buckets are powers of two
        kv = i % 4 != 1
        keys = datagen.as_u32(datagen.uniform_u32(n, 3000 + i))
        vals = np.arange(n, dtype=np.uint32) if kv else None
        ident, d, keep = identifiers(o, kind, B, splitter_seed=40 + i)
        segs.append(gms.Segment(to_dev(keys), torch.zeros(n, dtype=torch.int32, device="cuda"), n, B, ident,
                                to_dev(vals) if kv else None,
                                torch.zeros(n, dtype=torch.int32, device="cuda") if kv else None))
        refs.append((keys, vals, d, keep))
    plan = gms.BatchedMultisplit(segs)
    plan.run(use_graph=use_graph)
    torch.cuda.synchronize()
    assert plan.device_error() == 0
    check_against_oracle(o, segs, refs)
    outs = [(s_.keys_out.clone(), None if s_.values_out is None else s_.values_out.clone()) for s_ in segs]
    plan.close()
    for s_ in segs:
        s_.keys_out.zero_()
        if s_.values_out is not None:
            s_.values_out.zero_()
    tiled = gms.BatchedMultisplit(segs, variant=2)
    tiled.run(use_graph=use_graph)
    torch.cuda.synchronize()
    for s_, (k, v) in zip(segs, outs):
        assert torch.equal(s_.keys_out, k)
        if v is not None:
            assert torch.equal(s_.values_out, v)
    tiled.close()


def test_many_tiny_segments(gms_lib, oracle_mod):
    """20000 segments of 1..512 keys, B = 256 delta, key-value: one launch."""
    o = oracle_mod
    rng = np.random.default_rng(5)
    sizes = rng.integers(1, 513, 20000)
    total = int(sizes.sum())
    keys = datagen.uniform_u32(total, 77, device="cuda")
    vals = torch.arange(total, dtype=torch.int32, device="cuda")
    kout, vout = torch.empty_like(keys), torch.empty_like(vals)
    starts = np.concatenate([[0], np.cumsum(sizes)])
    segs = [gms.Segment(keys[a:b], kout[a:b], int(b - a), 256, gms.delta_bucket(), vals[a:b], vout[a:b])
            for a, b in zip(starts[:-1], starts[1:])]
    plan = gms.BatchedMultisplit(segs)
    assert plan.launches == 1
    plan.run(use_graph=True)
    torch.cuda.synchronize()
    hk, hv, hko, hvo = host(keys), host(vals), host(kout), host(vout)
    for i in range(0, len(sizes), 97):
        a, b = starts[i], starts[i + 1]
        rk, rv, _ = o.multisplit(hk[a:b], o.Desc(o.DELTA, 256), hv[a:b])
        np.testing.assert_array_equal(hko[a:b], rk)
        np.testing.assert_array_equal(hvo[a:b], rv)
    plan.close()


# ------------------------------------------------------------ the queue schedule
@pytest.mark.parametrize("use_graph", [False, True])
def test_queue_schedule_matches_oracle_mixed(gms_lib, oracle_mod, use_graph):
    """One persistent launch over the work list: every identifier kind, power-of-two
    and other bucket counts, key-only and key-value, empty, one-key and ragged
    segments, each equal to the oracle."""
    sizes = [0, 1, 7, 1024, 4095, 4096, 4097, 10000, 65537, 3, 300001, 1 << 17, 2, 99999, 32768, 33000]
    segs, refs = make_segments(oracle_mod, sizes, 15, kinds=(0, 1, 2, 3, 4, 5),
                               buckets=(2, 3, 4, 8, 16, 32, 64, 100, 128, 200, 256), kv_pattern=(1, 0, 1))
    # BITS needs a power of two
    segs = [s if not (s.identifier.desc(s.num_buckets).kind == 2 and s.num_buckets & (s.num_buckets - 1)) else None
            for s in segs]
    keep = [(s, r) for s, r in zip(segs, refs) if s is not None]
    segs, refs = [s for s, _ in keep], [r for _, r in keep]
    plan = gms.BatchedMultisplit(segs, schedule="queue")
    assert plan.schedule == "queue" and plan.launches == 1
    plan.run(use_graph=use_graph)
    torch.cuda.synchronize()
    assert plan.device_error() == 0
    check_against_oracle(oracle_mod, segs, refs)
    plan.close()


def test_queue_equals_classes_and_replays(gms_lib, oracle_mod):
    """The two schedules give the same bytes, over graph replays and after switching back and forth."""
    rng = np.random.default_rng(17)
    sizes = np.exp(rng.uniform(np.log(1024), np.log(1 << 18), 300)).astype(np.int64)
    segs, refs = make_segments(oracle_mod, sizes, 17)
    plan = gms.BatchedMultisplit(segs)
    plan.run(use_graph=True)
    torch.cuda.synchronize()
    want = [(s.keys_out.clone(), s.values_out.clone()) for s in segs]
    for schedule in ("queue", "classes", "queue"):
        plan.schedule = schedule
        for _ in range(2):
            for s in segs:
                s.keys_out.zero_()
                s.values_out.zero_()
            plan.run(use_graph=True)
            torch.cuda.synchronize()
            assert plan.device_error() == 0
            for s, (k, v) in zip(segs, want):
                assert torch.equal(s.keys_out, k) and torch.equal(s.values_out, v), schedule
    check_against_oracle(oracle_mod, segs, refs)
    plan.close()


def test_queue_segments_longer_than_the_lag(gms_lib, oracle_mod):
    """Segments of thousands of tiles, whose reorder items start while their own
    counting items are still being claimed by other blocks, beside small ones;
    skewed keys put a whole segment into one bucket."""
    sizes = [1 << 23, 5000, (1 << 22) + 123, 1 << 12, 777]
    segs, refs = make_segments(oracle_mod, sizes, 23, kinds=(0, 3), buckets=(2, 256), kv_pattern=(1, 0))
    # the fourth segment: every key equal
    s, (keys, vals, d, keep) = segs[3], refs[3]
    keys[:] = 0x12345678
    s.keys_in.copy_(datagen.from_u32(keys, "cuda"))
    plan = gms.BatchedMultisplit(segs, schedule="queue")
    for _ in range(2):
        plan.run(use_graph=True)
        torch.cuda.synchronize()
        assert plan.device_error() == 0
        check_against_oracle(oracle_mod, segs, refs)
    plan.close()
