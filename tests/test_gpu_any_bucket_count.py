"""Bucket counts that are not powers of two (B in [2, 256]).  The reference
takes powers of two only; the C ABI takes any count, and the kernels run with
the next power of two, its buckets from B up staying empty.  Every result is
compared bit-exactly with the oracle, whose identifiers reduce modulo B:
multisplit (key-only and key-value, each identifier kind, with and without
the scratch's bucket bytes), offsets, histograms, the batched form and the
serving form."""
import ctypes

import numpy as np
import pytest
import torch

import gpumultisplit_gb300 as gms
from gpumultisplit_gb300 import datagen
from gpu_util import KIND_NAMES, host, identifiers, run_multisplit, to_dev

pytestmark = pytest.mark.gpu

ODD_BUCKETS = [3, 5, 7, 12, 100, 129, 255]
KINDS = [0, 1, 3, 4, 5]  # delta, div, range, mask, even-float (bits needs a power of two)


def check(o, keys, B, kind, with_values, **kw):
    ident, d, keep = identifiers(o, kind, B, **kw)
    vals = np.arange(keys.size, dtype=np.uint32) if with_values else None
    gk, gv, goffs, err = run_multisplit(keys, B, ident, vals)
    rk, rv, roffs = o.multisplit(keys, d, vals)
    assert err == 0
    np.testing.assert_array_equal(gk, rk)
    if with_values:
        np.testing.assert_array_equal(gv, rv)
    assert len(goffs) == B and goffs == [int(x) for x in roffs]


@pytest.mark.parametrize("B", ODD_BUCKETS)
@pytest.mark.parametrize("kind", KINDS, ids=lambda k: KIND_NAMES[k])
@pytest.mark.parametrize("with_values", [False, True], ids=["keys", "pairs"])
def test_multisplit_odd_bucket_counts(gms_lib, oracle_mod, B, kind, with_values):
    for i, n in enumerate([1, 33, 4097, 100003]):
        keys = datagen.as_u32(datagen.uniform_u32(n, 9000 + B * 10 + kind + i))
        keys[: min(n, 3)] = [0, 0xFFFFFFFF, 0x80000000][: min(n, 3)]
        check(oracle_mod, keys, B, kind, with_values)


@pytest.mark.parametrize("B", [3, 12, 255])
def test_even_float_ids_above_b_wrap(gms_lib, oracle_mod, B):
    """A bin width that sends keys to ids from B up: they wrap modulo B, as on
    the oracle (and as the reference's power-of-two masks do)."""
    keys = datagen.as_u32(datagen.uniform_u32(50001, B))
    check(oracle_mod, keys, B, oracle_mod.EVEN_FLOAT, True, inverse_delta=3.7 * B / 2**32)
    check(oracle_mod, keys, B, oracle_mod.DIV, True, param=(1 << 32) // (3 * B) + 1)


@pytest.mark.parametrize("B", [3, 7, 12, 100])
def test_range_odd_b_duplicates_and_low_keys(gms_lib, oracle_mod, B):
    """Splitters with duplicates and a first splitter above zero; keys below it
    go to bucket B-1."""
    o = oracle_mod
    rng = np.random.default_rng(B)
    spl = np.sort((np.uint32(0x40000000) + rng.integers(0, 4 * B, B)).astype(np.uint32))
    spl[B // 2] = spl[B // 2 - 1]
    n = 60001
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


@pytest.mark.parametrize("kind", [1, 3, 5], ids=lambda k: KIND_NAMES[k])
@pytest.mark.parametrize("B", [5, 100])
def test_minimum_scratch_and_stages(gms_lib, oracle_mod, kind, B):
    """Costly identifiers with only the minimum scratch (no bucket bytes, the
    identifier runs in both passes) and through the three stage calls."""
    o = oracle_mod
    n = 5 * 4096 + 77
    keys = datagen.as_u32(datagen.uniform_u32(n, 7000 + kind + B))
    vals = np.arange(n, dtype=np.uint32)
    ident, d, keep = identifiers(o, kind, B)
    rk, rv, roffs = o.multisplit(keys, d, vals)
    full = ctypes.c_size_t()
    assert gms_lib.gms_multisplit_scratch_bytes(n, B, 1, ctypes.byref(full)) == 0
    minimum = full.value - (n + 255) // 256 * 256
    desc = ident.desc(B)
    stream = torch.cuda.current_stream().cuda_stream
    dk, dv = to_dev(keys), to_dev(vals)
    for nbytes in (full.value, minimum):
        scratch = torch.zeros(nbytes, dtype=torch.uint8, device="cuda")
        ok, ov = torch.zeros_like(dk), torch.zeros_like(dv)
        offs = (ctypes.c_uint32 * B)()
        assert gms_lib.gms_multisplit_key_value(dk.data_ptr(), dv.data_ptr(), ok.data_ptr(), ov.data_ptr(), n,
                                                ctypes.byref(desc), scratch.data_ptr(), nbytes, offs, stream) == 0
        torch.cuda.synchronize()
        np.testing.assert_array_equal(host(ok), rk)
        np.testing.assert_array_equal(host(ov), rv)
        assert list(offs) == [int(x) for x in roffs]
        ok.zero_()
        ov.zero_()
        args = (ctypes.byref(desc), 1, scratch.data_ptr(), nbytes, stream)
        assert gms_lib.gms_multisplit_prescan(dk.data_ptr(), n, *args) == 0
        assert gms_lib.gms_multisplit_scan(n, *args) == 0
        assert gms_lib.gms_multisplit_postscan(dk.data_ptr(), dv.data_ptr(), ok.data_ptr(), ov.data_ptr(), n,
                                               ctypes.byref(desc), scratch.data_ptr(), nbytes, stream) == 0
        torch.cuda.synchronize()
        np.testing.assert_array_equal(host(ok), rk)
        np.testing.assert_array_equal(host(ov), rv)
        code = ctypes.c_uint32()
        gms_lib.gms_read_device_error(scratch.data_ptr(), ctypes.byref(code), stream)
        assert code.value == 0
    del keep


@pytest.mark.parametrize("B", ODD_BUCKETS)
@pytest.mark.parametrize("kind", KINDS, ids=lambda k: KIND_NAMES[k])
def test_histogram_odd_bins(gms_lib, oracle_mod, B, kind):
    """B bins counted; the words after the B-entry histogram are left alone."""
    o = oracle_mod
    n = 300007
    keys = datagen.as_u32(datagen.uniform_u32(n, 600 + B + kind))
    ident, d, keep = identifiers(o, kind, B)
    buf = torch.full((B + 64,), -7, dtype=torch.int32, device="cuda")
    buf[:B].zero_()
    gms.multisplit_histogram(to_dev(keys), n, buf[:B], B, ident)
    torch.cuda.synchronize()
    got = buf.cpu().numpy()
    np.testing.assert_array_equal(got[:B], o.histogram(keys, d))
    assert (got[B:] == -7).all()


def test_histogram_even_and_range_entry_points(gms_lib, oracle_mod):
    o = oracle_mod
    n, B = 1 << 20, 100
    keys = datagen.as_u32(datagen.uniform_u32(n, 4242))
    spl = datagen.range_splitters(B, 5, "cuda")
    h = torch.zeros(B, dtype=torch.int32, device="cuda")
    gms.histogram_range(to_dev(keys), n, h, B, spl)
    np.testing.assert_array_equal(h.cpu().numpy(), o.histogram(keys, o.Desc(o.RANGE, B, splitters=datagen.as_u32(spl))))
    inv = float(B) / 2**32
    h.zero_()
    gms.histogram_even(to_dev(keys), n, h, B, 0, 0xFFFFFFFF, inv)
    np.testing.assert_array_equal(h.cpu().numpy(),
                                  o.histogram(keys, o.Desc(o.EVEN_FLOAT, B, lower=0, inverse_delta=inv)))


@pytest.mark.parametrize("use_graph", [False, True])
def test_batched_odd_bucket_counts(gms_lib, oracle_mod, use_graph):
    """Segments with B = 3 .. 255 beside powers of two in one plan; each equals
    the oracle on that segment alone."""
    o = oracle_mod
    rng = np.random.default_rng(11)
    buckets = [3, 5, 8, 12, 100, 129, 255, 256]
    segs, refs = [], []
    for i, n in enumerate([0, 1, 4095, 4097, 30011, 200003, 7, 65536, 12345, 99999, 131071, 2]):
        B = buckets[i % len(buckets)]
        kind = KINDS[int(rng.integers(len(KINDS)))]
        kv = bool(i % 3)
        keys = datagen.as_u32(datagen.uniform_u32(n, 5000 + i))
        vals = np.arange(n, dtype=np.uint32) if kv else None
        ident, d, keep = identifiers(o, kind, B, splitter_seed=100 + i)
        kout = torch.zeros(n, dtype=torch.int32, device="cuda")
        vin = to_dev(vals) if kv else None
        vout = torch.zeros(n, dtype=torch.int32, device="cuda") if kv else None
        segs.append(gms.Segment(to_dev(keys), kout, n, B, ident, vin, vout))
        refs.append((keys, vals, d, keep))
    plan = gms.BatchedMultisplit(segs)
    plan.run(use_graph=use_graph)
    torch.cuda.synchronize()
    assert plan.device_error() == 0
    for s, (keys, vals, d, _) in zip(segs, refs):
        rk, rv, _ = o.multisplit(keys, d, vals)
        np.testing.assert_array_equal(host(s.keys_out), rk)
        if vals is not None:
            np.testing.assert_array_equal(host(s.values_out), rv)
    plan.close()


def test_serving_odd_bucket_counts(gms_lib, oracle_mod):
    """Requests with odd bucket counts, multisplit and histogram, in one server."""
    o = oracle_mod
    server = gms.Server(arena_bytes=1 << 28)
    reqs = []
    for i, B in enumerate([3, 12, 100, 255, 7, 129]):
        n = 20000 + 3331 * i
        keys = datagen.as_u32(datagen.uniform_u32(n, 8100 + i))
        ident, d, keep = identifiers(o, KINDS[i % len(KINDS)], B, splitter_seed=i)
        op = "histogram" if i % 3 == 2 else "multisplit"
        dv = datagen.index_values(n, "cuda") if op == "multisplit" else None
        dk = to_dev(keys)  # the server holds pointers: keep the inputs alive
        rid = server.submit(op, dk, dv, n, B, ident)
        reqs.append((rid, op, keys, d, (keep, dk, dv)))
    for rid, op, keys, d, _ in reqs:
        res = server.wait(rid)
        assert res.status == 0
        if op == "histogram":
            np.testing.assert_array_equal(res.histogram.cpu().numpy(), o.histogram(keys, d))
        else:
            rk, rv, _ = o.multisplit(keys, d, np.arange(keys.size, dtype=np.uint32))
            np.testing.assert_array_equal(host(res.keys), rk)
            np.testing.assert_array_equal(host(res.values), rv)
        server.release(rid)
    server.close()
