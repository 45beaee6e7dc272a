"""Serving form: requests submitted while others run are batched into shared
rounds, admitted against the arena budget as memory frees up, and every result
equals the plain call on that request alone."""
import threading
import time

import numpy as np
import pytest
import torch

import gpumultisplit_gb300 as gms
from gpumultisplit_gb300 import _lib, datagen

pytestmark = pytest.mark.gpu


def plain_result(op, keys, vals, n, B, ident):
    """The plain (per-call) API on one request."""
    if op == "histogram":
        h = torch.zeros(B, dtype=torch.int32, device="cuda")
        gms.multisplit_histogram(keys, n, h, B, ident)
        return h, None, None
    ko = torch.empty(n, dtype=torch.int32, device="cuda")
    vo = torch.empty(n, dtype=torch.int32, device="cuda") if vals is not None else None
    if op == "sort7":
        ctx = gms.ms_sort_context()
        if vals is None:
            gms.multisplit_sort_7bit_allocate(n, ctx)
            gms.multisplit_sort_7bit(keys, ko, n, ctx)
        else:
            gms.multisplit_sort_7bit_allocate_pairs(n, ctx)
            gms.multisplit_sort_7bit_pairs(keys, ko, vals, vo, n, ctx)
        return ko, vo, None
    if op == "compaction":
        ctx = gms.compaction_context()
        if vals is None:
            gms.compaction_allocate_key_only(n, ctx)
            c = gms.compaction_key_only(keys, ko, n, ctx, ident)
        else:
            gms.compaction_allocate_key_value(n, ctx)
            c = gms.compaction_key_value(keys, vals, ko, vo, n, ctx, ident)
        return ko, vo, c
    ctx = gms.multisplit_context(B)
    if vals is None:
        gms.multisplit_allocate_key_only(n, ctx)
        gms.multisplit_key_only(keys, ko, n, ctx, ident)
    else:
        gms.multisplit_allocate_key_value(n, ctx)
        gms.multisplit_key_value(keys, vals, ko, vo, n, ctx, ident)
    return ko, vo, None


def make_requests(count, seed, max_n=200_000):
    rng = np.random.default_rng(seed)
    reqs = []
    for i in range(count):
        op = ["multisplit", "sort7", "histogram", "compaction"][rng.choice(4, p=[0.6, 0.2, 0.1, 0.1])]
        n = int(np.exp(rng.uniform(np.log(64), np.log(max_n)))) if i % 17 else int(rng.integers(0, 5))
        kv = bool(rng.integers(2))
        keys = datagen.uniform_u32(n, seed * 10000 + i, device="cuda")
        vals = datagen.index_values(n, "cuda") if kv and op != "histogram" else None
        if op == "compaction":
            B, ident = 2, gms.test_bucket(1)
        elif op == "sort7":
            B, ident = 2, None
        else:
            B = int(rng.choice([2, 8, 32, 256]))
            ident = gms.delta_bucket() if rng.integers(2) else gms.range_bucket(
                datagen.range_splitters(B, seed + i, "cuda"))
        reqs.append((op, keys, vals, n, B, ident))
    return reqs


def check(res, ref, op):
    ko, vo, extra = ref
    assert res.status == 0
    if op == "histogram":
        assert torch.equal(res.histogram, ko)
        return
    assert torch.equal(res.keys, ko)
    if vo is not None:
        assert torch.equal(res.values, vo)
    if op == "compaction":
        assert res.num_bucket0 == extra


def test_results_same_alone_and_in_the_mix(gms_lib):
    reqs = make_requests(80, 3)
    server = gms.Server(arena_bytes=1 << 30)
    ids = []
    for i, (op, k, v, n, B, ident) in enumerate(reqs):
        ids.append(server.submit(op, k, v, n, B, ident))
        if i % 10 == 9:
            time.sleep(0.002)  # later requests arrive while earlier ones are on the GPU
    results = [server.wait(rid) for rid in ids]
    stats = server.stats()
    torch.cuda.synchronize()
    for (op, k, v, n, B, ident), res in zip(reqs, results):
        check(res, plain_result(op, k, v, n, B, ident), op)
        assert res.done_s >= res.admit_s >= res.submit_s
    assert stats["completed"] == len(reqs)
    assert stats["max_requests_in_round"] > 1, "requests were never batched together"
    assert stats["rounds"] < sum(5 if r[0] == "sort7" else 1 for r in reqs)
    for rid in ids:
        server.release(rid)
    server.close()


def test_admission_waits_for_budget(gms_lib):
    """Outputs of ~20 requests exceed the arena; they are admitted as earlier
    results are released, and all finish with the right answer."""
    arena = 24 << 20
    server = gms.Server(arena_bytes=arena)
    n = 1 << 20  # 8 MiB of key-value output each
    keys = [datagen.uniform_u32(n, 50 + i, device="cuda") for i in range(20)]
    vals = datagen.index_values(n, "cuda")
    ids = [server.submit("multisplit", k, vals, n, 256, gms.delta_bucket()) for k in keys]
    done = {}
    deadline = time.time() + 60
    while len(done) < len(ids) and time.time() < deadline:
        for rid in server.take_completed():
            res = server.poll(rid)
            ref = plain_result("multisplit", keys[ids.index(rid)], vals, n, 256, gms.delta_bucket())
            check(res, ref, "multisplit")
            done[rid] = res
            server.release(rid)
        time.sleep(0.001)
    assert len(done) == len(ids)
    assert server.stats()["arena_peak_bytes"] <= arena
    with pytest.raises(gms.GmsError):  # can never fit
        server.submit("multisplit", keys[0], vals, 1 << 22, 256, gms.delta_bucket())
    server.close()


def test_drain_returns_when_only_releases_can_free_the_arena(gms_lib):
    """Finished results the caller keeps fill the arena, so the queued rest can
    never be admitted: drain and wait return GMS_ERROR_SCRATCH_TOO_SMALL instead
    of blocking forever.  After the results are released, drain finishes the
    rest, and every result is right."""
    arena = 24 << 20
    server = gms.Server(arena_bytes=arena)
    n = 1 << 20  # 8 MiB of key-value output each: two fit the request part of the arena
    keys = [datagen.uniform_u32(n, 80 + i, device="cuda") for i in range(6)]
    vals = datagen.index_values(n, "cuda")
    ids = [server.submit("multisplit", k, vals, n, 256, gms.delta_bucket()) for k in keys]
    t0 = time.time()
    with pytest.raises(gms.GmsError) as e:
        server.drain()
    assert e.value.status == _lib.GMS_ERROR_SCRATCH_TOO_SMALL
    with pytest.raises(gms.GmsError) as e:
        server.wait(ids[-1])
    assert e.value.status == _lib.GMS_ERROR_SCRATCH_TOO_SMALL
    assert time.time() - t0 < 30
    checked = 0
    while checked < len(ids):
        done = server.take_completed()
        for rid in done:
            res = server.poll(rid)
            i = ids.index(rid)
            check(res, plain_result("multisplit", keys[i], vals, n, 256, gms.delta_bucket()), "multisplit")
            server.release(rid)
            checked += 1
        if not done:
            time.sleep(0.001)
        assert time.time() - t0 < 60
    server.drain()  # nothing left: returns at once
    server.close()


def test_concurrent_submitters(gms_lib):
    reqs = make_requests(40, 9, max_n=50_000)
    server = gms.Server(arena_bytes=1 << 28)
    ids = [None] * len(reqs)

    def worker(lo, hi):
        for i in range(lo, hi):
            op, k, v, n, B, ident = reqs[i]
            ids[i] = server.submit(op, k, v, n, B, ident)

    th = [threading.Thread(target=worker, args=(j * 10, (j + 1) * 10)) for j in range(4)]
    for t in th:
        t.start()
    for t in th:
        t.join()
    server.drain()
    for i, (op, k, v, n, B, ident) in enumerate(reqs):
        check(server.poll(ids[i]), plain_result(op, k, v, n, B, ident), op)
    server.close()


def test_invalid_requests_rejected(gms_lib):
    server = gms.Server(arena_bytes=1 << 24)
    k = torch.zeros(16, dtype=torch.int32, device="cuda")
    with pytest.raises(gms.GmsError):
        server.submit("multisplit", k, None, 16, 300, gms.delta_bucket())
    with pytest.raises(gms.GmsError):  # bit-field buckets need a power of two
        server.submit("multisplit", k, None, 16, 3, gms.bits_bucket(0))
    with pytest.raises(gms.GmsError):
        server.submit("compaction", k, None, 16, 4, gms.delta_bucket())
    server.close()
