"""GPU parity of the stable multisplit (key-only and key-value) against the CPU
oracle, through the C ABI: every bucket count 2..256, every identifier kind,
ragged sizes, skew, misaligned buffers, the stage-by-stage entry points and the
reference-derived golden vectors.  Bit-exact (integer work)."""
import hashlib

import numpy as np
import pytest
import torch

import gpumultisplit_gb300 as gms
from gpumultisplit_gb300 import datagen
from gpu_util import KIND_NAMES, host, identifiers, run_multisplit, to_dev

pytestmark = pytest.mark.gpu

BUCKETS = [2, 4, 8, 16, 32, 64, 128, 256]
SIZES = [1, 31, 33, 4095, 4096, 4097, 8193, 100003]


def check(o, keys, B, kind, with_values, misalign=0, **kw):
    ident, d, keep = identifiers(o, kind, B, **kw)
    vals = np.arange(keys.size, dtype=np.uint32) if with_values else None
    gk, gv, goffs, err = run_multisplit(keys, B, ident, vals, misalign)
    rk, rv, roffs = o.multisplit(keys, d, vals)
    assert err == 0
    np.testing.assert_array_equal(gk, rk)
    if with_values:
        np.testing.assert_array_equal(gv, rv)
    assert goffs == [int(x) for x in roffs]


@pytest.mark.parametrize("B", BUCKETS)
@pytest.mark.parametrize("kind", [0, 1, 2, 3, 4, 5], ids=lambda k: KIND_NAMES[k])
@pytest.mark.parametrize("with_values", [False, True], ids=["keys", "pairs"])
def test_multisplit_matches_oracle(gms_lib, oracle_mod, B, kind, with_values):
    seed = B * 10 + kind
    for i, n in enumerate(SIZES[(B + kind) % 3::3] + [12289]):
        keys = datagen.as_u32(datagen.uniform_u32(n, seed + i))
        check(oracle_mod, keys, B, kind, with_values)


@pytest.mark.parametrize("n", [0, 1, 2, 3, 4, 5, 31, 32, 33, 4095, 4096, 4097, 65535, 65536, 65537, 1 << 20])
def test_ragged_sizes_pairs_b256(gms_lib, oracle_mod, n):
    keys = datagen.as_u32(datagen.uniform_u32(n, 1000 + n))
    check(oracle_mod, keys, 256, oracle_mod.DELTA, True)


@pytest.mark.parametrize("B", [2, 32, 64, 256])
def test_zipf_skew(gms_lib, oracle_mod, B):
    keys = datagen.as_u32(datagen.zipf_u32(300007, B, distinct=1 << 20))
    check(oracle_mod, keys, B, oracle_mod.DELTA, True)
    check(oracle_mod, keys, B, oracle_mod.RANGE, True, splitter_seed=B)


@pytest.mark.parametrize("B", [2, 16, 128, 256])
def test_one_bucket_and_alternating(gms_lib, oracle_mod, B):
    o = oracle_mod
    n = 50001
    check(o, np.zeros(n, np.uint32), B, o.DELTA, True)                  # everything in bucket 0
    check(o, np.full(n, 0xFFFFFFFF, np.uint32), B, o.DELTA, True)       # everything in bucket B-1
    alt = (np.arange(n, dtype=np.uint32) % B).astype(np.uint32)
    check(o, alt, B, o.BITS, True, shift=0)                            # round-robin buckets


@pytest.mark.parametrize("misalign", [1, 2, 3])
@pytest.mark.parametrize("B", [8, 256])
def test_misaligned_buffers(gms_lib, oracle_mod, misalign, B):
    """Buffers not 16-byte aligned take the plain-load path; same result."""
    keys = datagen.as_u32(datagen.uniform_u32(20011, 77))
    check(oracle_mod, keys, B, oracle_mod.DELTA, True, misalign=misalign)
    check(oracle_mod, keys, B, oracle_mod.DELTA, False, misalign=misalign)


def test_config1_keys_b8(gms_lib, oracle_mod, golden):
    """2^20 uniform keys (seed 1), 8 buckets by key >> 29, key-only: equal to the
    reference CPU multisplit's output (golden digest) and to the oracle."""
    case = next(c for c in golden if c["name"] == "config1_keys_b8")
    keys = datagen.as_u32(datagen.uniform_u32(1 << 20, 1))
    gk, _, offs, err = run_multisplit(keys, 8, gms.bits_bucket(29), None)
    assert err == 0
    assert hashlib.sha256(gk.tobytes()).hexdigest() == case["keys_out_sha256"]
    assert offs == case["offsets"]


def test_golden_cases_on_gpu(gms_lib, oracle_mod, golden):
    from test_oracle_golden import desc_of, gen_keys, sha

    o = oracle_mod
    for case in golden:
        if case["op"] != "multisplit":
            continue
        keys = gen_keys(case)
        B = case["buckets"]
        kind = case["kind"]
        kw = {}
        if kind == o.RANGE:
            kw["splitter_seed"] = case["splitter_seed"]
        if kind == o.BITS:
            kw["shift"] = case.get("shift", 0)
        if kind in (o.DIV, o.MASK):
            kw["param"] = case["param"]
        if kind == o.EVEN_FLOAT:
            kw["lower"] = case.get("lower", 0)
            kw["inverse_delta"] = case["inverse_delta"]
        ident, d, keep = identifiers(o, kind, B, **kw)
        assert d.c().kind == desc_of(o, case).c().kind
        vals = np.arange(case["n"], dtype=np.uint32) if case["values"] else None
        gk, gv, offs, err = run_multisplit(keys, B, ident, vals)
        assert err == 0, case["name"]
        assert sha(gk) == case["keys_out_sha256"], case["name"]
        if vals is not None:
            assert sha(gv) == case["values_out_sha256"], case["name"]
        if "offsets" in case:
            assert offs == case["offsets"], case["name"]
        else:
            assert sha(np.asarray(offs, dtype=np.uint32)) == case["offsets_sha256"], case["name"]


@pytest.mark.parametrize("with_values", [False, True])
def test_stage_entry_points_equal_one_call(gms_lib, oracle_mod, with_values):
    n, B = 77777, 64
    keys = datagen.as_u32(datagen.uniform_u32(n, 5))
    vals = np.arange(n, dtype=np.uint32)
    dk, dv = to_dev(keys), to_dev(vals)
    ok, ov = torch.empty_like(dk), torch.empty_like(dv)
    ctx = gms.multisplit_context(B)
    (gms.multisplit_allocate_key_value if with_values else gms.multisplit_allocate_key_only)(n, ctx)
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
    gms.multisplit_stages(dk, dv if with_values else None, ok, ov if with_values else None, n, ctx,
                          gms.delta_bucket(), events=ev)
    torch.cuda.synchronize()
    rk, rv, _ = oracle_mod.multisplit(keys, oracle_mod.Desc(oracle_mod.DELTA, B), vals if with_values else None)
    np.testing.assert_array_equal(host(ok), rk)
    if with_values:
        np.testing.assert_array_equal(host(ov), rv)
    # After the scan, the context's count matrix holds global offsets; column 0 = bucket starts.
    m = ctx.d_histogram.cpu().numpy().view(np.uint32).reshape(B, ctx.num_sub_prob)
    assert list(m[:, 0]) == [int(x) for x in oracle_mod.multisplit(keys, oracle_mod.Desc(oracle_mod.DELTA, B))[2]]


def test_prescan_counts_match_oracle_tiles(gms_lib, oracle_mod):
    """The prescan's bucket-major count matrix equals the oracle's per-tile counts
    (the check cpu_prescan_test makes, src/cpu_functions.h:55-103)."""
    import ctypes

    o = oracle_mod
    for B, with_values in ((8, False), (256, True), (32, True)):
        n = 50003
        keys = datagen.as_u32(datagen.uniform_u32(n, B))
        ctx = gms.multisplit_context(B)
        (gms.multisplit_allocate_key_value if with_values else gms.multisplit_allocate_key_only)(n, ctx)
        desc = gms.delta_bucket().desc(B)
        dk = to_dev(keys)
        st = gms_lib.gms_multisplit_prescan(dk.data_ptr(), n, ctypes.byref(desc), int(with_values),
                                            ctx.d_temp_storage.data_ptr(), ctx.temp_storage_bytes,
                                            torch.cuda.current_stream().cuda_stream)
        assert st == 0
        torch.cuda.synchronize()
        m = ctx.d_histogram.cpu().numpy().view(np.uint32).reshape(B, ctx.num_sub_prob)
        np.testing.assert_array_equal(m, o.tile_counts(keys, o.Desc(o.DELTA, B), ctx.size_sub_prob))


def test_repeated_calls_reuse_scratch(gms_lib, oracle_mod):
    """Scan state is reset by every call: back-to-back calls on one context agree."""
    o = oracle_mod
    n, B = 123457, 128
    ctx = gms.multisplit_context(B)
    gms.multisplit_allocate_key_value(n, ctx)
    for it in range(3):
        m = n - it * 1000
        keys = datagen.as_u32(datagen.uniform_u32(m, 900 + it))
        vals = np.arange(m, dtype=np.uint32)
        dk, dv = to_dev(keys), to_dev(vals)
        ok, ov = torch.empty_like(dk), torch.empty_like(dv)
        gms.multisplit_key_value(dk, dv, ok, ov, m, ctx, gms.delta_bucket())
        torch.cuda.synchronize()
        rk, rv, _ = o.multisplit(keys, o.Desc(o.DELTA, B), vals)
        np.testing.assert_array_equal(host(ok), rk)
        np.testing.assert_array_equal(host(ov), rv)
    assert gms.read_device_error(ctx) == 0


def test_errors_are_reported(gms_lib):
    ctx = gms.multisplit_context(70000)
    with pytest.raises(gms.GmsError):
        gms.multisplit_allocate_key_only(100, ctx)
    ctx = gms.multisplit_context(16)
    gms.multisplit_allocate_key_only(1000, ctx)
    dk = torch.zeros(100000, dtype=torch.int32, device="cuda")
    ok = torch.zeros_like(dk)
    with pytest.raises(gms.GmsError):  # over the context's capacity
        gms.multisplit_key_only(dk, ok, 100000, ctx, gms.delta_bucket())
    with pytest.raises(gms.GmsError):  # in place is not supported
        gms.multisplit_key_only(dk, dk, 1000, ctx, gms.delta_bucket())


@pytest.mark.parametrize("B", [4, 32, 256])
@pytest.mark.parametrize("with_values", [False, True], ids=["keys", "pairs"])
def test_range_adversarial_splitters(gms_lib, oracle_mod, B, with_values):
    """Splitters packed into one narrow key range, with duplicates and a first
    splitter above zero (keys below it wrap to bucket B-1), and keys aimed at
    the splitters themselves and their neighbours."""
    o = oracle_mod
    rng = np.random.default_rng(B)
    base = np.uint32(0x12345600)
    spl = np.sort((base + rng.integers(0, 3 * B, B)).astype(np.uint32))
    spl[B // 2] = spl[B // 2 - 1]  # a duplicate splitter
    n = 70001
    keys = np.concatenate([spl, spl - np.uint32(1), spl + np.uint32(1),
                           rng.integers(0, 2**32, n - 3 * B, dtype=np.uint64).astype(np.uint32)])
    rng.shuffle(keys)
    d_spl = datagen.from_u32(spl, "cuda")
    vals = np.arange(n, dtype=np.uint32) if with_values else None
    gk, gv, offs, err = run_multisplit(keys, B, gms.range_bucket(d_spl), vals)
    rk, rv, roffs = o.multisplit(keys, o.Desc(o.RANGE, B, splitters=spl), vals)
    assert err == 0
    np.testing.assert_array_equal(gk, rk)
    if with_values:
        np.testing.assert_array_equal(gv, rv)
    assert offs == [int(x) for x in roffs]
    hist = torch.zeros(B, dtype=torch.int32, device="cuda")
    gms.histogram_range(to_dev(keys), n, hist, B, d_spl)
    np.testing.assert_array_equal(hist.cpu().numpy(), o.histogram(keys, o.Desc(o.RANGE, B, splitters=spl)))


@pytest.mark.parametrize("kind", [1, 3, 5], ids=lambda k: KIND_NAMES[k])
@pytest.mark.parametrize("B", [8, 64, 256])
@pytest.mark.parametrize("with_values", [False, True], ids=["keys", "pairs"])
def test_bucket_bytes_and_fallback(gms_lib, oracle_mod, kind, B, with_values):
    """Costly identifiers (div, range, even-float) are evaluated once when the
    scratch holds a byte per key, and twice when it holds only the minimum;
    both give the oracle's output, through the one call and the three stages,
    full tiles, a ragged tail and misaligned buffers alike."""
    import ctypes

    o = oracle_mod
    n = 3 * 4096 + 1234
    keys = datagen.as_u32(datagen.uniform_u32(n, 4000 + kind * 7 + B))
    vals = np.arange(n, dtype=np.uint32) if with_values else None
    ident, d, keep = identifiers(o, kind, B)
    rk, rv, roffs = o.multisplit(keys, d, vals)
    full = ctypes.c_size_t()
    assert gms_lib.gms_multisplit_scratch_bytes(n, B, int(with_values), ctypes.byref(full)) == 0
    minimum = full.value - (n + 255) // 256 * 256
    desc = ident.desc(B)
    stream = torch.cuda.current_stream().cuda_stream
    for nbytes in (full.value, minimum):
        for misalign in (0, 1):
            scratch = torch.zeros(nbytes, dtype=torch.uint8, device="cuda")
            dk = to_dev(keys, misalign)
            dv = to_dev(vals, misalign) if with_values else None
            ok = to_dev(np.zeros(n, np.uint32), misalign)
            ov = to_dev(np.zeros(n, np.uint32), misalign) if with_values else None
            offs = (ctypes.c_uint32 * B)()
            if with_values:
                st = gms_lib.gms_multisplit_key_value(dk.data_ptr(), dv.data_ptr(), ok.data_ptr(), ov.data_ptr(), n,
                                                      ctypes.byref(desc), scratch.data_ptr(), nbytes, offs, stream)
            else:
                st = gms_lib.gms_multisplit_key_only(dk.data_ptr(), ok.data_ptr(), n, ctypes.byref(desc),
                                                     scratch.data_ptr(), nbytes, offs, stream)
            assert st == 0
            torch.cuda.synchronize()
            np.testing.assert_array_equal(host(ok), rk)
            if with_values:
                np.testing.assert_array_equal(host(ov), rv)
            assert list(offs) == [int(x) for x in roffs]
            # the three stages with the same scratch size
            ok.zero_()
            args = (ctypes.byref(desc), int(with_values), scratch.data_ptr(), nbytes, stream)
            assert gms_lib.gms_multisplit_prescan(dk.data_ptr(), n, *args) == 0
            assert gms_lib.gms_multisplit_scan(n, *args) == 0
            assert gms_lib.gms_multisplit_postscan(dk.data_ptr(), dv.data_ptr() if with_values else None,
                                                   ok.data_ptr(), ov.data_ptr() if with_values else None, n,
                                                   ctypes.byref(desc), scratch.data_ptr(), nbytes, stream) == 0
            torch.cuda.synchronize()
            np.testing.assert_array_equal(host(ok), rk)
            code = ctypes.c_uint32()
            gms_lib.gms_read_device_error(scratch.data_ptr(), ctypes.byref(code), stream)
            assert code.value == 0
    del keep
