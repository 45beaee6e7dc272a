"""The C-ABI library without a GPU: it loads, exports every entry point that
include/*.h declares, and its host-only logic (scratch sizing, tile geometry,
argument checks that fail before any CUDA call) behaves."""
import ctypes
import re
from pathlib import Path

import numpy as np
import pytest

import gpumultisplit_gb300 as gms
from gpumultisplit_gb300 import _lib

ROOT = Path(__file__).resolve().parents[1]


def declared_symbols():
    names = set()
    for h in (ROOT / "include").glob("*.h"):
        text = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        names |= set(re.findall(r"\b(gms_[a-z0-9_]+)\s*\(", text))
    return names


def test_library_exports_every_declared_symbol(gms_lib):
    decl = declared_symbols()
    assert len(decl) >= 20
    for name in decl:
        assert hasattr(gms_lib, name), name
    # and the Python binding prototypes cover the same set
    assert decl == set(_lib.EXPORTED)


def test_version_and_status_strings(gms_lib):
    assert gms_lib.gms_version() >= 100
    for s in range(7):
        assert gms_lib.gms_status_string(s)


def scratch_bytes(n, B, kv):
    out = ctypes.c_size_t()
    st = gms_lib_().gms_multisplit_scratch_bytes(n, B, kv, ctypes.byref(out))
    return st, out.value


def gms_lib_():
    return gms.load()


def multisplit_min_bytes(n, B, kv):
    """Scratch a multisplit needs without the optional byte per key (what the
    sorts reserve for their passes: bit-field digits are cheap to evaluate)."""
    return scratch_bytes(n, B, kv)[1] - (n + 255) // 256 * 256


@pytest.mark.parametrize("B", [2, 4, 8, 16, 32, 64, 128, 256])
@pytest.mark.parametrize("kv", [0, 1])
def test_scratch_and_geometry(gms_lib, B, kv):
    for n in (0, 1, 4095, 4096, 4097, 1 << 20, 1 << 28, 0xFFFFFFFF):
        st, nbytes = scratch_bytes(n, B, kv)
        assert st == 0
        tile, tiles, off = ctypes.c_uint32(), ctypes.c_uint32(), ctypes.c_size_t()
        assert gms_lib.gms_multisplit_geometry(n, B, kv, ctypes.byref(tile), ctypes.byref(tiles),
                                               ctypes.byref(off)) == 0
        assert tiles.value == (n + tile.value - 1) // tile.value
        assert off.value == 256  # the count matrix always starts after the 256-byte header
        assert nbytes >= 256 + 4 * B * tiles.value + n  # matrix, plus a bucket byte per key
        assert nbytes % 256 == 0


def test_unsupported_bucket_counts(gms_lib):
    for B in (0, 1, 65537, 1 << 20):
        st, _ = scratch_bytes(100, B, 0)
        assert st == _lib.GMS_ERROR_UNSUPPORTED_BUCKETS
    # any count in [2, 256] is taken (the kernels round it up to a power of two) ...
    for B in (3, 12, 100, 255):
        st, nbytes = scratch_bytes(100000, B, 1)
        assert st == 0 and nbytes == scratch_bytes(100000, 1 << (B - 1).bit_length(), 1)[1]
    # ... except by a bit-field identifier, whose buckets are a power of two
    d = gms.bits_bucket(3).desc(12)
    st = gms_lib.gms_multisplit_key_only(1 << 20, 2 << 20, 10, ctypes.byref(d), 1 << 24, 1 << 30, None, None)
    assert st == _lib.GMS_ERROR_UNSUPPORTED_BUCKETS


def test_argument_checks_before_cuda(gms_lib):
    """These calls fail on their arguments, before any CUDA work."""
    d = _lib.BucketDesc(kind=_lib.GMS_BUCKET_DELTA, num_buckets=70000)
    assert gms_lib.gms_multisplit_key_only(1 << 20, 2 << 20, 10, ctypes.byref(d), 1 << 24, 1 << 20, None,
                                           None) == _lib.GMS_ERROR_UNSUPPORTED_BUCKETS
    # more than 256 buckets: RANGE to 8192 splitters, BITS a power of two, not through the stage calls
    for kind, B, want in ((_lib.GMS_BUCKET_RANGE, 8193, _lib.GMS_ERROR_UNSUPPORTED_BUCKETS),
                          (_lib.GMS_BUCKET_BITS, 1000, _lib.GMS_ERROR_UNSUPPORTED_BUCKETS),
                          (_lib.GMS_BUCKET_DIV, 1000, _lib.GMS_ERROR_INVALID_VALUE)):
        d = _lib.BucketDesc(kind=kind, num_buckets=B, d_splitters=1 << 26)
        assert gms_lib.gms_multisplit_key_value(1 << 20, 2 << 20, 3 << 20, 4 << 20, 10, ctypes.byref(d), 1 << 24,
                                                1 << 26, None, None) == want
    d = _lib.BucketDesc(kind=_lib.GMS_BUCKET_DELTA, num_buckets=1000)
    assert gms_lib.gms_multisplit_prescan(1 << 20, 10, ctypes.byref(d), 1, 1 << 24, 1 << 26, None) == \
        _lib.GMS_ERROR_UNSUPPORTED_BUCKETS
    need = ctypes.c_size_t()
    assert gms_lib.gms_multisplit_scratch_bytes(100000, 1000, 1, ctypes.byref(need)) == 0
    assert gms_lib.gms_multisplit_key_value(1 << 20, 2 << 21, 3 << 21, 4 << 21, 100000, ctypes.byref(d), 1 << 24,
                                            need.value - 256, None, None) == _lib.GMS_ERROR_SCRATCH_TOO_SMALL
    d = _lib.BucketDesc(kind=99, num_buckets=8)
    assert gms_lib.gms_multisplit_key_only(1 << 20, 2 << 20, 10, ctypes.byref(d), 1 << 24, 1 << 20, None,
                                           None) == _lib.GMS_ERROR_INVALID_VALUE
    d = _lib.BucketDesc(kind=_lib.GMS_BUCKET_DIV, num_buckets=8, param=0)
    assert gms_lib.gms_multisplit_key_only(1 << 20, 2 << 20, 10, ctypes.byref(d), 1 << 24, 1 << 20, None,
                                           None) == _lib.GMS_ERROR_INVALID_VALUE
    d = _lib.BucketDesc(kind=_lib.GMS_BUCKET_RANGE, num_buckets=8)
    assert gms_lib.gms_multisplit_key_only(1 << 20, 2 << 20, 10, ctypes.byref(d), 1 << 24, 1 << 20, None,
                                           None) == _lib.GMS_ERROR_INVALID_VALUE
    d = _lib.BucketDesc(kind=_lib.GMS_BUCKET_DELTA, num_buckets=8)
    # scratch too small for n
    assert gms_lib.gms_multisplit_key_only(1 << 30, 2 << 30, 1 << 20, ctypes.byref(d), 1 << 24, 1024, None,
                                           None) == _lib.GMS_ERROR_SCRATCH_TOO_SMALL
    # scratch not 256-byte aligned
    assert gms_lib.gms_multisplit_key_only(1 << 20, 2 << 20, 10, ctypes.byref(d), (1 << 24) + 4, 1 << 20, None,
                                           None) == _lib.GMS_ERROR_INVALID_VALUE
    # in place (input and output overlap)
    assert gms_lib.gms_multisplit_key_only(1 << 20, (1 << 20) + 16, 10, ctypes.byref(d), 1 << 24, 1 << 20, None,
                                           None) == _lib.GMS_ERROR_INVALID_VALUE
    # n = 0 is a no-op that succeeds
    assert gms_lib.gms_multisplit_key_only(None, None, 0, ctypes.byref(d), None, 0, None, None) == 0
    # compaction needs exactly two buckets
    assert gms_lib.gms_compaction_key_only(1 << 20, 2 << 20, 10, ctypes.byref(d), 1 << 24, 1 << 20, None,
                                           None) == _lib.GMS_ERROR_INVALID_VALUE


def test_wide_argument_checks_before_cuda(gms_lib):
    """64-bit entry points: calls that fail on their arguments, before any CUDA work."""
    f = gms_lib.gms_multisplit_wide
    k_in, k_out, v_in, v_out, scr = 1 << 20, 1 << 24, 1 << 28, 1 << 30, 1 << 32
    d = _lib.BucketDesc64(kind=_lib.GMS_BUCKET_DELTA, num_buckets=256)
    ok = ctypes.c_size_t()
    assert gms_lib.gms_multisplit_wide_scratch_bytes(1000, 256, 8, 8, ctypes.byref(ok)) == 0
    big = 1 << 26
    for kb, vb in ((3, 0), (8, 2), (16, 8), (8, 12)):  # widths other than 4/8 (keys) and 0/4/8 (values)
        assert f(k_in, v_in, k_out, v_out, 1000, kb, vb, ctypes.byref(d), scr, big, None, None) == \
            _lib.GMS_ERROR_INVALID_VALUE
        assert gms_lib.gms_multisplit_wide_scratch_bytes(1000, 256, kb, vb, ctypes.byref(ok)) == \
            _lib.GMS_ERROR_INVALID_VALUE
    bad = [
        (_lib.BucketDesc64(kind=_lib.GMS_BUCKET_DELTA, num_buckets=300), _lib.GMS_ERROR_UNSUPPORTED_BUCKETS),
        (_lib.BucketDesc64(kind=_lib.GMS_BUCKET_BITS, num_buckets=12), _lib.GMS_ERROR_UNSUPPORTED_BUCKETS),
        (_lib.BucketDesc64(kind=_lib.GMS_BUCKET_BITS, num_buckets=16, shift=64), _lib.GMS_ERROR_INVALID_VALUE),
        (_lib.BucketDesc64(kind=_lib.GMS_BUCKET_DIV, num_buckets=16, param=0), _lib.GMS_ERROR_INVALID_VALUE),
        (_lib.BucketDesc64(kind=_lib.GMS_BUCKET_RANGE, num_buckets=16), _lib.GMS_ERROR_INVALID_VALUE),
        (_lib.BucketDesc64(kind=42, num_buckets=16), _lib.GMS_ERROR_INVALID_VALUE),
    ]
    for bd, want in bad:
        assert f(k_in, v_in, k_out, v_out, 1000, 8, 8, ctypes.byref(bd), scr, big, None, None) == want
    # 32-bit keys: 64-bit parameters must fit in 32 bits
    wide_param = _lib.BucketDesc64(kind=_lib.GMS_BUCKET_MASK, num_buckets=2, param=1 << 40)
    assert f(k_in, v_in, k_out, v_out, 1000, 4, 8, ctypes.byref(wide_param), scr, big, None, None) == \
        _lib.GMS_ERROR_INVALID_VALUE
    # keys not aligned to their 8 bytes, values not aligned to theirs
    assert f(k_in + 4, v_in, k_out, v_out, 1000, 8, 8, ctypes.byref(d), scr, big, None, None) == \
        _lib.GMS_ERROR_INVALID_VALUE
    assert f(k_in, v_in + 4, k_out, v_out, 1000, 8, 8, ctypes.byref(d), scr, big, None, None) == \
        _lib.GMS_ERROR_INVALID_VALUE
    # outputs overlapping (8-byte elements: 8 bytes apart overlap)
    assert f(k_in, v_in, k_out, k_out + 8, 1000, 8, 8, ctypes.byref(d), scr, big, None, None) == \
        _lib.GMS_ERROR_INVALID_VALUE
    # 64-bit keys need the bucket bytes: the reported size, not less
    need = ctypes.c_size_t()
    assert gms_lib.gms_multisplit_wide_scratch_bytes(100000, 256, 8, 8, ctypes.byref(need)) == 0
    assert f(k_in, v_in, k_out, v_out, 100000, 8, 8, ctypes.byref(d), scr, need.value - 256, None, None) == \
        _lib.GMS_ERROR_SCRATCH_TOO_SMALL
    # sorts: bit ranges beyond the key width
    s = gms_lib.gms_sort_wide_scratch_bytes
    assert s(1000, 8, 8, 0, 64, 8, ctypes.byref(ok)) == 0
    assert s(1000, 8, 8, 0, 65, 8, ctypes.byref(ok)) == _lib.GMS_ERROR_INVALID_VALUE
    assert s(1000, 4, 8, 0, 33, 8, ctypes.byref(ok)) == _lib.GMS_ERROR_INVALID_VALUE
    assert s(1000, 8, 0, 0, 64, 9, ctypes.byref(ok)) == _lib.GMS_ERROR_INVALID_VALUE
    # n = 0 is a no-op that succeeds
    assert f(None, None, None, None, 0, 8, 8, ctypes.byref(d), None, 0, None, None) == 0


def test_wide_scratch_sizes(gms_lib):
    """64-bit elements: 4096-key tiles up to 12 bytes per key, 3072 at 16,
    bucket bytes always counted; a sort adds its ping-pong keys and values."""
    def nbytes(n, B, kb, vb):
        out = ctypes.c_size_t()
        assert gms_lib.gms_multisplit_wide_scratch_bytes(n, B, kb, vb, ctypes.byref(out)) == 0
        return out.value

    def align(x):
        return (x + 255) // 256 * 256

    n = 1 << 20
    # 32-bit keys and values: the same as gms_multisplit_scratch_bytes
    for kv in (0, 1):
        ref = ctypes.c_size_t()
        assert gms_lib.gms_multisplit_scratch_bytes(n, 256, kv, ctypes.byref(ref)) == 0
        assert nbytes(n, 256, 4, 4 * kv) == ref.value
    for kb, vb, tile in ((8, 0, 4096), (4, 8, 4096), (8, 4, 4096), (8, 8, 3072)):
        tiles = (n + tile - 1) // tile
        m = 256 * tiles
        chunks = (m + 4095) // 4096
        expect = align(align(align(256 + 4 * m) + 8 * chunks) + n)
        assert nbytes(n, 256, kb, vb) == expect, (kb, vb)
    srt = ctypes.c_size_t()
    assert gms_lib.gms_sort_wide_scratch_bytes(n, 8, 8, 0, 64, 8, ctypes.byref(srt)) == 0
    assert srt.value == align(align(nbytes(n, 256, 8, 8)) + 8 * n) + 8 * n


def test_sort_scratch_covers_both_digit_widths(gms_lib):
    for n in (1, 1000, 1 << 20):
        for kv in (0, 1):
            sb = ctypes.c_size_t()
            assert gms_lib.gms_sort_7bit_scratch_bytes(n, kv, ctypes.byref(sb)) == 0
            m16 = multisplit_min_bytes(n, 16, kv)
            m128 = multisplit_min_bytes(n, 128, kv)
            assert sb.value >= max(m16, m128) + 4 * n * (1 + kv)


def test_sort_scratch_all_digit_widths(gms_lib):
    """The sort scratch holds the widest pass's count matrix plus the ping-pong buffers."""
    widths = {4: (16,), 5: (32, 4), 6: (16, 64), 7: (16, 128), 8: (256,)}
    for bits, bs in widths.items():
        for n in (1, 4097, 1 << 20):
            for kv in (0, 1):
                sb = ctypes.c_size_t()
                assert gms_lib.gms_sort_scratch_bytes(n, bits, kv, ctypes.byref(sb)) == 0
                need = max(multisplit_min_bytes(n, b, kv) for b in bs) + 4 * n * (1 + kv)
                assert sb.value >= need, (bits, n, kv)
    sb = ctypes.c_size_t()
    for bad in (3, 9, 0):
        assert gms_lib.gms_sort_scratch_bytes(100, bad, 0, ctypes.byref(sb)) == _lib.GMS_ERROR_INVALID_VALUE


def test_partial_key_sort_scratch_and_checks(gms_lib):
    sb = ctypes.c_size_t()
    for begin, end, digit, widths in ((0, 32, 8, (256,)), (3, 17, 5, (32, 16)), (20, 21, 6, (2,))):
        assert gms_lib.gms_sort_bits_scratch_bytes(1 << 20, begin, end, digit, 1, ctypes.byref(sb)) == 0
        need = max(multisplit_min_bytes(1 << 20, b, 1) for b in widths) + 8 * (1 << 20)
        assert sb.value >= need
    assert gms_lib.gms_sort_bits_scratch_bytes(100, 9, 9, 8, 0, ctypes.byref(sb)) == 0 and sb.value == 0
    for begin, end, digit in ((5, 4, 8), (0, 33, 8), (-1, 8, 8), (0, 8, 3), (0, 8, 9)):
        assert gms_lib.gms_sort_bits_scratch_bytes(100, begin, end, digit, 0, ctypes.byref(sb)) == \
            _lib.GMS_ERROR_INVALID_VALUE
        assert gms_lib.gms_sort_bits_key_only(1 << 20, 2 << 20, 10, begin, end, digit, 1 << 24, 1 << 20, None) == \
            _lib.GMS_ERROR_INVALID_VALUE


def test_sort_method_setting(gms_lib):
    """gms_sort_set_method / get (host only): the three methods, and invalid values refused."""
    v = ctypes.c_int()
    assert gms_lib.gms_sort_get_method(ctypes.byref(v)) == 0 and v.value == _lib.GMS_SORT_AUTO
    for m in ("multisplit", "onesweep", "auto"):
        gms.set_sort_method(m)
        assert gms.sort_method() == m
    assert gms_lib.gms_sort_set_method(3) == _lib.GMS_ERROR_INVALID_VALUE
    assert gms_lib.gms_sort_set_method(-1) == _lib.GMS_ERROR_INVALID_VALUE
    assert gms_lib.gms_sort_get_method(None) == _lib.GMS_ERROR_INVALID_VALUE
    assert gms.sort_method() == "auto"


def test_tuning_table_host_logic(gms_lib):
    """Tile variants, the built-in table, set/get/reset and their checks (host only)."""
    from gpumultisplit_gb300 import batched

    shapes = [gms.tile_variant_shape(v) for v in range(batched.NUM_TILE_VARIANTS)]
    assert shapes[0] == (8, 16, 4096)
    assert all(t == w * 32 * i for w, i, t in shapes)
    gms.reset_tuning()
    base = gms.tuning_table()
    # built-in: the plain path's 4096-key tile for every class
    for (b, kv, c), v in base.items():
        assert gms.tile_variant_shape(v)[2] == 4096
    assert [batched.size_class(n) for n in (0, 1, 1024, 1025, 2048, 2049, 65536, 65537, 1 << 30)] == \
        [0, 0, 0, 1, 1, 2, 6, 7, 7]
    gms.set_tuning({(128, True, 3): 3})
    assert gms.tuning_table()[(128, True, 3)] == 3
    v = ctypes.c_int()
    assert gms_lib.gms_tuning_set(256, 1, 3, 3) == _lib.GMS_ERROR_INVALID_VALUE  # 128 threads < 256 buckets
    assert gms_lib.gms_tuning_set(256, 1, 8, 0) == _lib.GMS_ERROR_INVALID_VALUE  # no size class 8
    assert gms_lib.gms_tuning_set(3, 1, 0, 0) == _lib.GMS_ERROR_UNSUPPORTED_BUCKETS
    assert gms_lib.gms_tuning_get(512, 0, 0, ctypes.byref(v)) == _lib.GMS_ERROR_UNSUPPORTED_BUCKETS
    assert gms_lib.gms_tile_variant_shape(4, None, None, None) == _lib.GMS_ERROR_INVALID_VALUE
    gms.reset_tuning()
    assert gms.tuning_table() == base
    # autotune argument checks fail before any CUDA call
    assert gms_lib.gms_autotune(1, 1, 1 << 20, 1, None, None) == _lib.GMS_ERROR_INVALID_VALUE    # bit 0 = 1 bucket
    assert gms_lib.gms_autotune(4, 0, 1 << 20, 1, None, None) == _lib.GMS_ERROR_INVALID_VALUE    # no shape
    assert gms_lib.gms_autotune(4, 1, 1000, 1, None, None) == _lib.GMS_ERROR_INVALID_VALUE       # too few keys
    assert gms_lib.gms_autotune(4, 1, 1 << 20, 0, None, None) == _lib.GMS_ERROR_INVALID_VALUE    # no repetitions


def test_batch_plan_classes_follow_the_table(gms_lib):
    """Plans are host-only: launches = 2 per (kind, B, key/value, variant) class + 1 scan,
    and 1 per class of segments small enough for one warp each."""
    from gpumultisplit_gb300 import batched

    gms.reset_tuning()
    fake = 1 << 32  # never dereferenced: plan creation does no device work

    def plan(sizes, B=256, variant=None):
        arr = (batched.GmsSegment * len(sizes))()
        for i, n in enumerate(sizes):
            arr[i] = batched.GmsSegment(fake, fake, fake, fake, n, gms.delta_bucket().desc(B))
        h = ctypes.c_void_p()
        if variant is None:
            st = gms_lib.gms_batch_create(arr, len(sizes), ctypes.byref(h))
        else:
            st = gms_lib.gms_batch_create_with_variant(arr, len(sizes), variant, ctypes.byref(h))
        assert st == 0
        n = ctypes.c_uint32()
        assert gms_lib.gms_batch_launch_count(h, ctypes.byref(n)) == 0
        gms_lib.gms_batch_destroy(h)
        return n.value

    assert plan([1000, 1000, 5000]) == 2 + 1            # the built-in table: 4096-key tiles for every class
    assert plan([1000, 1500, 5000], variant=0) == 2 + 1
    gms.set_tuning({(256, True, 0): 2, (256, True, 1): 1})  # 1024-key tiles, 2048-key tiles, 4096 above
    assert plan([1000, 1000, 5000]) == 2 * 2 + 1
    assert plan([1000, 1500, 5000]) == 2 * 3 + 1
    gms.reset_tuning()
    # segments of at most 512 keys: one warp each, one launch per class, no scan
    assert plan([100, 512]) == 1
    assert plan([100, 512, 513]) == 1 + 2 + 1
    assert plan([100, 7, 0], B=5) == 1
    assert plan([100, 512], variant=2) == 2 + 1  # a forced tile shape keeps them tiled
    # two scan groups (keys past 2^32) beside one-warp segments: 2 classes x 2 + 2 scans + 1
    assert plan([(1 << 31) + 5, 100, (1 << 31) + 77, 50]) == 2 * 1 + 2 + 1
    arr = (batched.GmsSegment * 1)()
    arr[0] = batched.GmsSegment(fake, fake, fake, fake, 10, gms.delta_bucket().desc(256))
    h = ctypes.c_void_p()
    assert gms_lib.gms_batch_create_with_variant(arr, 1, 3, ctypes.byref(h)) == _lib.GMS_ERROR_INVALID_VALUE
    assert gms_lib.gms_batch_create_with_variant(arr, 1, -1, ctypes.byref(h)) == _lib.GMS_ERROR_INVALID_VALUE


def test_batch_schedule_setting(gms_lib):
    """gms_batch_set_schedule / get (host only): the queue schedule is one launch;
    invalid schedules are refused and leave the plan's schedule unchanged."""
    from gpumultisplit_gb300 import batched

    fake = 1 << 32
    arr = (batched.GmsSegment * 3)()
    for i, n in enumerate((5000, 100, 70000)):
        arr[i] = batched.GmsSegment(fake, fake, fake, fake, n, gms.delta_bucket().desc(8 << i))
    h = ctypes.c_void_p()
    assert gms_lib.gms_batch_create(arr, 3, ctypes.byref(h)) == 0
    v, n = ctypes.c_int(), ctypes.c_uint32()
    assert gms_lib.gms_batch_get_schedule(h, ctypes.byref(v)) == 0 and v.value == _lib.GMS_BATCH_SCHEDULE_CLASSES
    assert gms_lib.gms_batch_launch_count(h, ctypes.byref(n)) == 0 and n.value > 1
    assert gms_lib.gms_batch_set_schedule(h, _lib.GMS_BATCH_SCHEDULE_QUEUE) == 0
    assert gms_lib.gms_batch_get_schedule(h, ctypes.byref(v)) == 0 and v.value == _lib.GMS_BATCH_SCHEDULE_QUEUE
    assert gms_lib.gms_batch_launch_count(h, ctypes.byref(n)) == 0 and n.value == 1
    assert gms_lib.gms_batch_set_schedule(h, 2) == _lib.GMS_ERROR_INVALID_VALUE
    assert gms_lib.gms_batch_set_schedule(h, -1) == _lib.GMS_ERROR_INVALID_VALUE
    assert gms_lib.gms_batch_set_schedule(None, 0) == _lib.GMS_ERROR_INVALID_VALUE
    assert gms_lib.gms_batch_get_schedule(h, ctypes.byref(v)) == 0 and v.value == _lib.GMS_BATCH_SCHEDULE_QUEUE
    assert gms_lib.gms_batch_set_schedule(h, _lib.GMS_BATCH_SCHEDULE_CLASSES) == 0
    gms_lib.gms_batch_destroy(h)


@pytest.mark.parametrize("spec", ["bench", "big_and_small"])
def test_queue_work_list_has_no_forward_waits(gms_lib, spec):
    """The queue's work list is built on the host and checked there: every item
    waits only on items listed before it, else the schedule is refused.  Plans
    over the 4096-segment batched workload and over a mix of very large and
    tiny segments must be accepted (an ordering that put a segment's reorder
    items between its scan items would be refused here)."""
    from gpumultisplit_gb300 import batched, datagen

    fake = 1 << 32
    if spec == "bench":
        sizes, buckets, kinds = datagen.batched_spec()
    else:
        rng = np.random.default_rng(3)
        sizes = np.array([1 << 26, 5, 1 << 24, 4096, 3, (1 << 25) + 7] * 40, dtype=np.int64)
        buckets = rng.choice([2, 3, 8, 100, 256], size=sizes.size)
        kinds = ["delta" if k else "range" for k in rng.integers(0, 2, sizes.size)]
    arr = (batched.GmsSegment * len(sizes))()
    for i, (n, B, kind) in enumerate(zip(sizes.tolist(), buckets.tolist(), kinds)):
        desc = (gms.delta_bucket().desc(B) if kind == "delta"
                else _lib.BucketDesc(kind=_lib.GMS_BUCKET_RANGE, num_buckets=B, d_splitters=fake))
        arr[i] = batched.GmsSegment(fake, fake, fake, fake, int(n), desc)
    h = ctypes.c_void_p()
    assert gms_lib.gms_batch_create(arr, len(sizes), ctypes.byref(h)) == 0
    assert gms_lib.gms_batch_set_schedule(h, _lib.GMS_BATCH_SCHEDULE_QUEUE) == 0
    gms_lib.gms_batch_destroy(h)


def test_missing_library_fails_loudly(tmp_path):
    with pytest.raises(ImportError):
        _lib.load(tmp_path / "libgpumultisplit.so")


def test_big_bucket_scratch_layout(gms_lib):
    """Above 256 buckets the scratch holds the larger digit pass's scratch (with
    its bucket bytes), ping-pong keys (and values) and a B-word histogram; the
    id's bits are split in half between the passes."""
    def nbytes(n, B, kv):
        out = ctypes.c_size_t()
        assert gms_lib.gms_multisplit_scratch_bytes(n, B, kv, ctypes.byref(out)) == 0
        return out.value

    def align(x):
        return (x + 255) // 256 * 256

    def full(n, logb):  # one multisplit's scratch with bucket bytes, 4096-key tiles
        tiles = (n + 4095) // 4096
        m = (1 << logb) * tiles
        return align(align(align(256 + 4 * m) + 8 * ((m + 4095) // 4096)) + n)

    for n in (1, 4096, 1000003):
        for B in (257, 1000, 4096, 65536):
            bits = (B - 1).bit_length()
            lo, hi = (bits + 1) // 2, bits - (bits + 1) // 2
            ms = max(full(n, lo), full(n, hi))
            keys_end = align(ms) + 4 * n
            assert nbytes(n, B, 0) == align(align(keys_end) + 4 * B)
            assert nbytes(n, B, 1) == align(align(align(keys_end) + 4 * n) + 4 * B)
