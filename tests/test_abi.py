"""The C-ABI library without a GPU: it loads, exports every entry point that
include/*.h declares, and its host-only logic (scratch sizing, tile geometry,
argument checks that fail before any CUDA call) behaves."""
import ctypes
import re
from pathlib import Path

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
    for B in (0, 1, 257, 512):
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
    d = _lib.BucketDesc(kind=_lib.GMS_BUCKET_DELTA, num_buckets=300)
    assert gms_lib.gms_multisplit_key_only(1 << 20, 2 << 20, 10, ctypes.byref(d), 1 << 24, 1 << 20, None,
                                           None) == _lib.GMS_ERROR_UNSUPPORTED_BUCKETS
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


def test_tuning_table_host_logic(gms_lib):
    """Tile variants, the built-in table, set/get/reset and their checks (host only)."""
    from gpumultisplit_gb300 import batched

    shapes = [gms.tile_variant_shape(v) for v in range(batched.NUM_TILE_VARIANTS)]
    assert shapes[0] == (8, 16, 4096)
    assert all(t == w * 32 * i for w, i, t in shapes)
    gms.reset_tuning()
    base = gms.tuning_table()
    # built-in: the tile that holds the segment up to 2048 keys, the 4096-key tile above
    for (b, kv, c), v in base.items():
        assert gms.tile_variant_shape(v)[2] == {0: 1024, 1: 2048}.get(c, 4096)
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
    """Plans are host-only: launches = 2 per (kind, B, key/value, variant) class + 1 scan."""
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

    assert plan([1000, 1000, 5000]) == 2 * 2 + 1        # 1024-key tiles and 4096-key tiles
    assert plan([1000, 1500, 5000]) == 2 * 3 + 1
    assert plan([1000, 1500, 5000], variant=0) == 2 + 1
    gms.set_tuning({(256, True, c): 0 for c in range(8)})
    assert plan([1000, 1500, 5000]) == 2 + 1
    gms.reset_tuning()
    arr = (batched.GmsSegment * 1)()
    arr[0] = batched.GmsSegment(fake, fake, fake, fake, 10, gms.delta_bucket().desc(256))
    h = ctypes.c_void_p()
    assert gms_lib.gms_batch_create_with_variant(arr, 1, 3, ctypes.byref(h)) == _lib.GMS_ERROR_INVALID_VALUE
    assert gms_lib.gms_batch_create_with_variant(arr, 1, -1, ctypes.byref(h)) == _lib.GMS_ERROR_INVALID_VALUE


def test_missing_library_fails_loudly(tmp_path):
    with pytest.raises(ImportError):
        _lib.load(tmp_path / "libgpumultisplit.so")
