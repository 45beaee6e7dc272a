"""Host-side mirror of the reference's multisplit API, on the C ABI.

Names, argument order and meaning follow the reference headers:
  * multisplit_context / multisplit_allocate_key_only / _key_value /
    multisplit_release_memory / multisplit_key_only / multisplit_key_value
    (src/api/multisplit.cuh:29-313);
  * ms_sort_context / multisplit_sort_7bit_allocate / _allocate_pairs /
    multisplit_sort_7bit / multisplit_sort_7bit_pairs / multisplit_sort_release_memory
    (src/api/multisplit_sort.cuh:100-364, src/api/multisplit_sort_pairs.cuh:21-65);
  * compaction_context / compaction_allocate_key_only / _key_value /
    compaction_release_memory / compaction_key_only / compaction_key_value
    (src/kernels/compaction/multisplit2_compaction.cuh:477-573);
  * histogram_even / histogram_range: the launches of the reference's histogram
    kernels (src/main/main_histogram.cu:163-179, 272-279), plus
    multisplit_histogram for any identifier.

Device buffers are CUDA torch tensors of a 4-byte dtype (int32 or uint32) or raw
device addresses (int).  Calls run on torch's current CUDA stream.

Error behaviour: the reference's functions return void and print on an
unsupported bucket count (src/api/multisplit.cuh:135-136); these raise GmsError
instead, so a failed call is never silent.

Bucket identifiers: the reference passes a functor; a precompiled library takes
a descriptor.  The identifier classes below cover the functors the reference and
its drivers use (delta_func, ms_bucket_sort_*bit, test_bucket) and the
identifiers of the benchmark configurations (delta key*B>>32, range splitters).
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass

from . import _lib
from ._lib import BucketDesc, BucketDesc64, check

# ---------------------------------------------------------------- helpers


def _ptr(x, elem_bytes: int | None = 4) -> int | None:
    """Device address of a CUDA tensor (of `elem_bytes`-byte elements) or an int."""
    if x is None:
        return None
    if isinstance(x, int):
        return x
    if hasattr(x, "data_ptr"):
        if elem_bytes is not None and x.element_size() != elem_bytes:
            raise TypeError(f"this buffer must hold {8 * elem_bytes}-bit elements")
        if not x.is_cuda:
            raise TypeError("multisplit buffers must be CUDA tensors")
        return x.data_ptr()
    raise TypeError(f"unsupported buffer type {type(x)!r}")


def _scratch(ctx) -> int | None:
    return _ptr(ctx.d_temp_storage, None)


def _stream(stream=None) -> int | None:
    if stream is not None:
        return stream if isinstance(stream, int) else stream.cuda_stream
    import torch

    return torch.cuda.current_stream().cuda_stream


def _alloc_scratch(nbytes: int):
    """Scratch buffer; its 256-byte header (device error word, scan ticket) starts zeroed."""
    import torch

    t = torch.empty(max(int(nbytes), 256), dtype=torch.uint8, device="cuda")
    t[:256].zero_()
    return t


# ------------------------------------------------------ bucket identifiers


class BucketIdentifier:
    """Base class: produces a gms_bucket_desc for a given bucket count."""

    def desc(self, num_buckets: int) -> BucketDesc:  # pragma: no cover - abstract
        raise NotImplementedError

    def desc64(self, num_buckets: int) -> BucketDesc64:  # pragma: no cover - abstract
        """The gms_bucket_desc64 of this identifier (64-bit parameters), for
        multisplit_wide / 64-bit keys."""
        raise NotImplementedError


@dataclass
class delta_bucket(BucketIdentifier):
    """bucket = key * B >> 32 (B equal-width ranges of the 32-bit key space)."""

    def desc(self, num_buckets):
        return BucketDesc(kind=_lib.GMS_BUCKET_DELTA, num_buckets=num_buckets)

    def desc64(self, num_buckets):
        return BucketDesc64(kind=_lib.GMS_BUCKET_DELTA, num_buckets=num_buckets)


@dataclass
class delta_func(BucketIdentifier):
    """bucket = key / delta (README.md:85-91, src/main/main_multisplit.cu:41-47)."""

    delta: int

    def desc(self, num_buckets):
        return BucketDesc(kind=_lib.GMS_BUCKET_DIV, num_buckets=num_buckets, param=int(self.delta))

    def desc64(self, num_buckets):
        return BucketDesc64(kind=_lib.GMS_BUCKET_DIV, num_buckets=num_buckets, param=int(self.delta))


@dataclass
class bits_bucket(BucketIdentifier):
    """bucket = (key >> shift) & (B - 1)."""

    shift: int = 0

    def desc(self, num_buckets):
        return BucketDesc(kind=_lib.GMS_BUCKET_BITS, num_buckets=num_buckets, shift=int(self.shift))

    def desc64(self, num_buckets):
        return BucketDesc64(kind=_lib.GMS_BUCKET_BITS, num_buckets=num_buckets, shift=int(self.shift))


def ms_bucket_sort_4bit(shift: int) -> bits_bucket:
    """ms_bucket_sort_4bit<shift> (src/api/multisplit_sort.cuh:63-68)."""
    return bits_bucket(shift)


def ms_bucket_sort_7bit(shift: int) -> bits_bucket:
    """ms_bucket_sort_7bit<shift> (src/api/multisplit_sort.cuh:81-86)."""
    return bits_bucket(shift)


def test_bucket(flag: int = 1) -> BucketIdentifier:
    """test_bucket<flag>: key & ((1 << flag) - 1) (src/main/main_compaction.cu:26-31)."""
    if flag != 1:
        raise ValueError("only test_bucket<1> (key & 1) is a two-bucket identifier")
    return bits_bucket(0)


@dataclass
class mask_bucket(BucketIdentifier):
    """bucket = (key & mask) != 0."""

    mask: int

    def desc(self, num_buckets):
        return BucketDesc(kind=_lib.GMS_BUCKET_MASK, num_buckets=num_buckets, param=int(self.mask))

    def desc64(self, num_buckets):
        return BucketDesc64(kind=_lib.GMS_BUCKET_MASK, num_buckets=num_buckets, param=int(self.mask))


class range_bucket(BucketIdentifier):
    """bucket = upper_bound(splitters, key) - 1 over B sorted splitters (device
    tensor), the level search of src/kernels/histogram/multisplit2_histograms.cuh:434."""

    def __init__(self, d_splitters):
        self.d_splitters = d_splitters

    def desc(self, num_buckets):
        return BucketDesc(kind=_lib.GMS_BUCKET_RANGE, num_buckets=num_buckets, d_splitters=_ptr(self.d_splitters))

    def desc64(self, num_buckets):
        # the splitters have the keys' width (int32 for 32-bit keys, int64 for 64-bit keys)
        return BucketDesc64(kind=_lib.GMS_BUCKET_RANGE, num_buckets=num_buckets,
                            d_splitters=_ptr(self.d_splitters, None))


@dataclass
class even_float_bucket(BucketIdentifier):
    """bin = (uint32)((key - lower) * inverse_delta) in float arithmetic
    (src/kernels/histogram/multisplit2_histograms.cuh:60)."""

    lower: int
    inverse_delta: float

    def desc(self, num_buckets):
        return BucketDesc(kind=_lib.GMS_BUCKET_EVEN_FLOAT, num_buckets=num_buckets, lower=int(self.lower),
                          inverse_delta=float(self.inverse_delta))

    def desc64(self, num_buckets):
        return BucketDesc64(kind=_lib.GMS_BUCKET_EVEN_FLOAT, num_buckets=num_buckets, lower=int(self.lower),
                            inverse_delta=float(self.inverse_delta))


# -------------------------------------------------------------- multisplit


class multisplit_context:
    """multisplit_context (src/api/multisplit.cuh:29-47)."""

    def __init__(self, n_buckets: int):
        self.num_buckets = int(n_buckets)
        self.size_sub_prob = 0
        self.num_sub_prob = 0
        self.num_blocks = 0
        self.d_temp_storage = None
        self.temp_storage_bytes = 0
        self.key_value = False
        self.capacity = 0

    @property
    def d_histogram(self):
        """Bucket-major count matrix inside the scratch, laid out for num_elements =
        the allocated capacity (after a call: global offsets, offset(b, tile) at
        [b * num_sub_prob + tile]).  It always starts 256 bytes into the scratch."""
        if self.d_temp_storage is None or self.num_buckets > 256:
            return None
        import torch

        off = ctypes.c_size_t()
        check(_lib.load().gms_multisplit_geometry(self.capacity, self.num_buckets, int(self.key_value), None, None,
                                                  ctypes.byref(off)), "multisplit_geometry")
        return self.d_temp_storage[off.value:off.value + 4 * self.num_buckets * self.num_sub_prob].view(torch.int32)


def _ms_allocate(num_elements: int, context: multisplit_context, key_value: bool) -> None:
    lib = _lib.load()
    nbytes = ctypes.c_size_t()
    check(lib.gms_multisplit_scratch_bytes(num_elements, context.num_buckets, int(key_value), ctypes.byref(nbytes)),
          "multisplit_allocate")
    tile, tiles = ctypes.c_uint32(), ctypes.c_uint32()
    if context.num_buckets <= 256:  # above 256 buckets there are two digit passes and no single count matrix
        check(lib.gms_multisplit_geometry(num_elements, context.num_buckets, int(key_value), ctypes.byref(tile),
                                          ctypes.byref(tiles), None), "multisplit_geometry")
    context.size_sub_prob = tile.value
    context.num_sub_prob = tiles.value
    context.num_blocks = tiles.value
    context.temp_storage_bytes = nbytes.value
    context.d_temp_storage = _alloc_scratch(nbytes.value)
    context.key_value = key_value
    context.capacity = int(num_elements)


def multisplit_allocate_key_only(num_elements: int, context: multisplit_context) -> None:
    """src/api/multisplit.cuh:50-61."""
    _ms_allocate(num_elements, context, False)


def multisplit_allocate_key_value(num_elements: int, context: multisplit_context) -> None:
    """src/api/multisplit.cuh:63-74."""
    _ms_allocate(num_elements, context, True)


def multisplit_release_memory(context: multisplit_context) -> None:
    """src/api/multisplit.cuh:76-79."""
    context.d_temp_storage = None
    context.temp_storage_bytes = 0


def _offsets_buffer(num_buckets):
    return (ctypes.c_uint32 * num_buckets)()


def multisplit_key_only(d_key_in, d_key_out, num_elements: int, context: multisplit_context,
                        bucket_identifier: BucketIdentifier, multisplit_offset=None, stream=None):
    """src/api/multisplit.cuh:81-197.  If multisplit_offset is a list (or True),
    the B bucket start offsets are returned (and written into a given list)."""
    desc = bucket_identifier.desc(context.num_buckets)
    offs = _offsets_buffer(context.num_buckets) if multisplit_offset is not None else None
    check(_lib.load().gms_multisplit_key_only(_ptr(d_key_in), _ptr(d_key_out), num_elements, ctypes.byref(desc),
                                              _scratch(context), context.temp_storage_bytes, offs,
                                              _stream(stream)), "multisplit_key_only")
    return _export_offsets(offs, multisplit_offset)


def multisplit_key_value(d_key_in, d_value_in, d_key_out, d_value_out, num_elements: int,
                         context: multisplit_context, bucket_identifier: BucketIdentifier, multisplit_offset=None,
                         stream=None):
    """src/api/multisplit.cuh:199-313."""
    desc = bucket_identifier.desc(context.num_buckets)
    offs = _offsets_buffer(context.num_buckets) if multisplit_offset is not None else None
    check(_lib.load().gms_multisplit_key_value(_ptr(d_key_in), _ptr(d_value_in), _ptr(d_key_out), _ptr(d_value_out),
                                               num_elements, ctypes.byref(desc), _scratch(context),
                                               context.temp_storage_bytes, offs, _stream(stream)),
          "multisplit_key_value")
    return _export_offsets(offs, multisplit_offset)


def _export_offsets(offs, target):
    if offs is None:
        return None
    import numpy as np

    vals = np.ctypeslib.as_array(offs).tolist()  # far faster than list() on a ctypes array of 64 Ki entries
    if isinstance(target, list):
        target[:] = vals
    return vals


def multisplit_stages(d_key_in, d_value_in, d_key_out, d_value_out, num_elements: int,
                      context: multisplit_context, bucket_identifier: BucketIdentifier, stream=None,
                      events=None):
    """Runs prescan, scan and postscan as three C-ABI calls (same result as
    multisplit_key_only / _key_value).  If `events` holds four CUDA events they
    are recorded before, between and after the stages."""
    lib = _lib.load()
    desc = bucket_identifier.desc(context.num_buckets)
    kv = int(d_value_in is not None)
    s = _stream(stream)
    scratch, nbytes = _scratch(context), context.temp_storage_bytes
    if events:
        events[0].record()
    check(lib.gms_multisplit_prescan(_ptr(d_key_in), num_elements, ctypes.byref(desc), kv, scratch, nbytes, s),
          "multisplit_prescan")
    if events:
        events[1].record()
    check(lib.gms_multisplit_scan(num_elements, ctypes.byref(desc), kv, scratch, nbytes, s), "multisplit_scan")
    if events:
        events[2].record()
    check(lib.gms_multisplit_postscan(_ptr(d_key_in), _ptr(d_value_in), _ptr(d_key_out), _ptr(d_value_out),
                                      num_elements, ctypes.byref(desc), scratch, nbytes, s), "multisplit_postscan")
    if events:
        events[3].record()


# ------------------------------------------------ 64-bit keys and values


def _elem_bytes(t) -> int:
    return 0 if t is None else int(t.element_size())


def multisplit_wide_allocate(num_elements: int, context: multisplit_context, key_bytes: int,
                             value_bytes: int = 0) -> None:
    """Scratch for multisplit_wide with keys of key_bytes (4 or 8) and values of
    value_bytes (0 for key-only, 4 or 8)."""
    nbytes = ctypes.c_size_t()
    check(_lib.load().gms_multisplit_wide_scratch_bytes(num_elements, context.num_buckets, int(key_bytes),
                                                        int(value_bytes), ctypes.byref(nbytes)),
          "multisplit_wide_allocate")
    context.temp_storage_bytes = nbytes.value
    context.d_temp_storage = _alloc_scratch(nbytes.value)
    context.widths = (int(key_bytes), int(value_bytes))


def multisplit_wide(d_key_in, d_key_out, num_elements: int, context: multisplit_context,
                    bucket_identifier: BucketIdentifier, d_value_in=None, d_value_out=None, multisplit_offset=None,
                    stream=None):
    """Stable multisplit with 32- or 64-bit keys and 32- or 64-bit values (the
    element widths of the tensors, int32 or int64; the same as at allocation).
    Same order and offsets as multisplit_key_value; the identifier is applied
    to the key's full width."""
    kb, vb = _elem_bytes(d_key_in), _elem_bytes(d_value_in)
    if getattr(context, "widths", (kb, vb)) != (kb, vb):
        raise ValueError(f"context allocated for widths {context.widths}, called with {(kb, vb)}")
    desc = bucket_identifier.desc64(context.num_buckets)
    offs = _offsets_buffer(context.num_buckets) if multisplit_offset is not None else None
    check(_lib.load().gms_multisplit_wide(_ptr(d_key_in, kb), _ptr(d_value_in, vb or None), _ptr(d_key_out, kb),
                                          _ptr(d_value_out, vb or None), num_elements, kb, vb, ctypes.byref(desc),
                                          _scratch(context),
                                          context.temp_storage_bytes, offs, _stream(stream)), "multisplit_wide")
    return _export_offsets(offs, multisplit_offset)


def multisplit_histogram_wide(d_key_in, num_elements: int, d_histogram, num_buckets: int,
                              bucket_identifier: BucketIdentifier, stream=None) -> None:
    """Adds per-bucket counts of 32- or 64-bit keys (int32 / int64 tensor) into
    d_histogram[0..B) (int32, zeroed by the caller), B <= 256."""
    kb = _elem_bytes(d_key_in)
    desc = bucket_identifier.desc64(num_buckets)
    check(_lib.load().gms_histogram_wide(_ptr(d_key_in, kb), num_elements, kb, ctypes.byref(desc),
                                         _ptr(d_histogram), _stream(stream)), "multisplit_histogram_wide")


def multisplit_sort_wide_allocate(n_elements: int, context, key_bytes: int, value_bytes: int = 0,
                                  begin_bit: int = 0, end_bit: int | None = None, digit_bits: int = 8) -> None:
    """Scratch for a stable sort of key_bytes-wide keys (with value_bytes-wide
    values) by key bits [begin_bit, end_bit) (end_bit defaults to the key width)."""
    end = 8 * int(key_bytes) if end_bit is None else int(end_bit)
    nbytes = ctypes.c_size_t()
    check(_lib.load().gms_sort_wide_scratch_bytes(n_elements, int(key_bytes), int(value_bytes), int(begin_bit), end,
                                                  int(digit_bits), ctypes.byref(nbytes)),
          "multisplit_sort_wide_allocate")
    context.temp_storage_bytes = nbytes.value
    context.d_temp_storage = _alloc_scratch(max(nbytes.value, 256))
    context.wide = (int(key_bytes), int(value_bytes), int(begin_bit), end, int(digit_bits))


def multisplit_sort_wide(d_key_in, d_key_out, n_elements: int, context, d_value_in=None, d_value_out=None,
                         stream=None) -> None:
    """Stable sort by the key bit range given at allocation; keys and values are
    int32 or int64 tensors of the widths given there."""
    kb, vb, b, e, d = context.wide
    if (_elem_bytes(d_key_in), _elem_bytes(d_value_in)) != (kb, vb):
        raise ValueError("tensor widths differ from the allocation")
    check(_lib.load().gms_sort_wide(_ptr(d_key_in, kb), _ptr(d_key_out, kb), _ptr(d_value_in, vb or None),
                                    _ptr(d_value_out, vb or None), n_elements, kb, vb, b, e, d, _scratch(context),
                                    context.temp_storage_bytes, _stream(stream)), "multisplit_sort_wide")


SORT_METHODS = {"auto": 0, "multisplit": 1, "onesweep": 2}


def set_sort_method(method: str) -> None:
    """How the 32-bit radix sorts run their digits, process-wide: "multisplit"
    (prescan, scan, postscan per digit, the reference's way), "onesweep" (one
    histogram pass, then one look-back pass per digit) or "auto" (the
    library's choice, at present the multisplit passes).  The output is the
    same either way."""
    check(_lib.load().gms_sort_set_method(SORT_METHODS[method]), "gms_sort_set_method")


def sort_method() -> str:
    v = ctypes.c_int()
    check(_lib.load().gms_sort_get_method(ctypes.byref(v)), "gms_sort_get_method")
    return {v_: k for k, v_ in SORT_METHODS.items()}[v.value]


def read_device_error(context, stream=None) -> int:
    """Device error word of a context's scratch (0 = every bounded wait finished)."""
    code = ctypes.c_uint32()
    st = _lib.load().gms_read_device_error(_scratch(context), ctypes.byref(code), _stream(stream))
    if st not in (_lib.GMS_SUCCESS, _lib.GMS_ERROR_DEVICE_TIMEOUT):
        check(st, "read_device_error")
    return code.value


# -------------------------------------------------------------------- sort


class ms_sort_context:
    """ms_sort_context (src/api/multisplit_sort.cuh:100-116)."""

    def __init__(self):
        self.d_temp_storage = None
        self.temp_storage_bytes = 0


def _sort_allocate(n_elements, context, key_value, digit_bits=7):
    nbytes = ctypes.c_size_t()
    check(_lib.load().gms_sort_scratch_bytes(n_elements, digit_bits, int(key_value), ctypes.byref(nbytes)),
          f"multisplit_sort_{digit_bits}bit_allocate")
    context.temp_storage_bytes = nbytes.value
    context.d_temp_storage = _alloc_scratch(nbytes.value)
    context.digit_bits = digit_bits


def _sort_run(d_key_in, d_key_out, d_value_in, d_value_out, n, context, digit_bits, stream):
    lib = _lib.load()
    if d_value_in is None:
        st = lib.gms_sort_key_only(_ptr(d_key_in), _ptr(d_key_out), n, digit_bits, _scratch(context),
                                   context.temp_storage_bytes, _stream(stream))
    else:
        st = lib.gms_sort_key_value(_ptr(d_key_in), _ptr(d_key_out), _ptr(d_value_in), _ptr(d_value_out), n,
                                    digit_bits, _scratch(context), context.temp_storage_bytes, _stream(stream))
    check(st, f"multisplit_sort_{digit_bits}bit")


def multisplit_sort_7bit_allocate(n_elements: int, context: ms_sort_context) -> None:
    """src/api/multisplit_sort.cuh:151-170."""
    _sort_allocate(n_elements, context, False)


def multisplit_sort_7bit_allocate_pairs(n_elements: int, context: ms_sort_context) -> None:
    """src/api/multisplit_sort.cuh:171-191."""
    _sort_allocate(n_elements, context, True)


def multisplit_sort_release_memory(context: ms_sort_context) -> None:
    """src/api/multisplit_sort.cuh:312-318."""
    context.d_temp_storage = None
    context.temp_storage_bytes = 0


def multisplit_sort_7bit(d_key_in, d_key_out_ms, n_elements: int, context: ms_sort_context, stream=None) -> None:
    """src/api/multisplit_sort.cuh:320-364."""
    check(_lib.load().gms_sort_7bit_key_only(_ptr(d_key_in), _ptr(d_key_out_ms), n_elements,
                                             _scratch(context), context.temp_storage_bytes,
                                             _stream(stream)), "multisplit_sort_7bit")


def multisplit_sort_7bit_pairs(d_key_in, d_key_out_ms, d_value_in, d_value_out_ms, n_elements: int,
                               context: ms_sort_context, stream=None) -> None:
    """src/api/multisplit_sort_pairs.cuh:21-65 (argument order kin, kout, vin, vout)."""
    check(_lib.load().gms_sort_7bit_key_value(_ptr(d_key_in), _ptr(d_key_out_ms), _ptr(d_value_in),
                                              _ptr(d_value_out_ms), n_elements, _scratch(context),
                                              context.temp_storage_bytes, _stream(stream)),
          "multisplit_sort_7bit_pairs")


def _define_sorts(bits: int):
    """multisplit_sort_<bits>bit[_allocate][_pairs] (src/api/multisplit_sort.cuh:118-559,
    src/api/multisplit_sort_pairs.cuh:67-260)."""

    def allocate(n_elements, context):
        _sort_allocate(n_elements, context, False, bits)

    def allocate_pairs(n_elements, context):
        _sort_allocate(n_elements, context, True, bits)

    def sort(d_key_in, d_key_out_ms, n_elements, context, stream=None):
        _sort_run(d_key_in, d_key_out_ms, None, None, n_elements, context, bits, stream)

    def sort_pairs(d_key_in, d_key_out_ms, d_value_in, d_value_out_ms, n_elements, context, stream=None):
        _sort_run(d_key_in, d_key_out_ms, d_value_in, d_value_out_ms, n_elements, context, bits, stream)

    g = globals()
    g[f"multisplit_sort_{bits}bit_allocate"] = allocate
    g[f"multisplit_sort_{bits}bit_allocate_pairs"] = allocate_pairs
    g[f"multisplit_sort_{bits}bit"] = sort
    g[f"multisplit_sort_{bits}bit_pairs"] = sort_pairs


for _bits in (4, 5, 6, 8):
    _define_sorts(_bits)


def multisplit_sort_bits_allocate(n_elements, context, begin_bit=0, end_bit=32, digit_bits=8, pairs=False):
    """Scratch for a stable sort by key bits [begin_bit, end_bit) (the begin/end
    bit arguments of the CUB sorts the reference compares against,
    src/main/main_bms.cu:199)."""
    nbytes = ctypes.c_size_t()
    check(_lib.load().gms_sort_bits_scratch_bytes(n_elements, begin_bit, end_bit, digit_bits, int(pairs),
                                                  ctypes.byref(nbytes)), "multisplit_sort_bits_allocate")
    context.temp_storage_bytes = nbytes.value
    context.d_temp_storage = _alloc_scratch(max(nbytes.value, 256))
    context.bit_range = (begin_bit, end_bit, digit_bits)


def multisplit_sort_bits(d_key_in, d_key_out_ms, n_elements, context, stream=None):
    """Stable sort of keys by the bit range given at allocation."""
    b, e, d = context.bit_range
    check(_lib.load().gms_sort_bits_key_only(_ptr(d_key_in), _ptr(d_key_out_ms), n_elements, b, e, d,
                                             _scratch(context), context.temp_storage_bytes, _stream(stream)),
          "multisplit_sort_bits")


def multisplit_sort_bits_pairs(d_key_in, d_key_out_ms, d_value_in, d_value_out_ms, n_elements, context,
                               stream=None):
    """Stable sort of key-value pairs by the key bit range given at allocation."""
    b, e, d = context.bit_range
    check(_lib.load().gms_sort_bits_key_value(_ptr(d_key_in), _ptr(d_key_out_ms), _ptr(d_value_in),
                                              _ptr(d_value_out_ms), n_elements, b, e, d, _scratch(context),
                                              context.temp_storage_bytes, _stream(stream)),
          "multisplit_sort_bits_pairs")


# -------------------------------------------------------------- compaction


class compaction_context:
    """compaction_context (src/kernels/compaction/multisplit2_compaction.cuh:477-489)."""

    def __init__(self):
        self.d_temp_storage = None
        self.temp_storage_bytes = 0


def _compaction_allocate(n, context, key_value):
    nbytes = ctypes.c_size_t()
    check(_lib.load().gms_compaction_scratch_bytes(n, int(key_value), ctypes.byref(nbytes)), "compaction_allocate")
    context.temp_storage_bytes = nbytes.value
    context.d_temp_storage = _alloc_scratch(nbytes.value)


def compaction_allocate_key_only(num_elements: int, context: compaction_context) -> None:
    """multisplit2_compaction.cuh:491-503."""
    _compaction_allocate(num_elements, context, False)


def compaction_allocate_key_value(num_elements: int, context: compaction_context) -> None:
    """multisplit2_compaction.cuh:505-517."""
    _compaction_allocate(num_elements, context, True)


def compaction_release_memory(context: compaction_context) -> None:
    """multisplit2_compaction.cuh:519-523."""
    context.d_temp_storage = None
    context.temp_storage_bytes = 0


def compaction_key_only(d_key_in, d_key_out, num_elements: int, context: compaction_context,
                        bucket_identifier: BucketIdentifier, stream=None) -> int:
    """multisplit2_compaction.cuh:525-548; returns the number of bucket-0 keys."""
    desc = bucket_identifier.desc(2)
    n0 = ctypes.c_uint32()
    check(_lib.load().gms_compaction_key_only(_ptr(d_key_in), _ptr(d_key_out), num_elements, ctypes.byref(desc),
                                              _scratch(context), context.temp_storage_bytes,
                                              ctypes.byref(n0), _stream(stream)), "compaction_key_only")
    return n0.value


def compaction_key_value(d_key_in, d_value_in, d_key_out, d_value_out, num_elements: int,
                         context: compaction_context, bucket_identifier: BucketIdentifier, stream=None) -> int:
    """multisplit2_compaction.cuh:550-573; returns the number of bucket-0 keys."""
    desc = bucket_identifier.desc(2)
    n0 = ctypes.c_uint32()
    check(_lib.load().gms_compaction_key_value(_ptr(d_key_in), _ptr(d_value_in), _ptr(d_key_out), _ptr(d_value_out),
                                               num_elements, ctypes.byref(desc), _scratch(context),
                                               context.temp_storage_bytes, ctypes.byref(n0), _stream(stream)),
          "compaction_key_value")
    return n0.value


# --------------------------------------------------------------- histogram


def multisplit_histogram(d_key_in, num_elements: int, d_histogram, num_buckets: int,
                         bucket_identifier: BucketIdentifier, stream=None) -> None:
    """Adds per-bucket counts into d_histogram[0..B) (int32, zeroed by the caller)."""
    desc = bucket_identifier.desc(num_buckets)
    check(_lib.load().gms_histogram(_ptr(d_key_in), num_elements, ctypes.byref(desc), _ptr(d_histogram),
                                    _stream(stream)), "multisplit_histogram")


def histogram_even(d_key_in, num_elements: int, d_histogram, num_bins: int, lower_level: int, upper_level: int,
                   inverse_delta: float, stream=None) -> None:
    """multisplit2_histogram_even_* (src/kernels/histogram/multisplit2_histograms.cuh:36-400)."""
    check(_lib.load().gms_histogram_even(_ptr(d_key_in), num_elements, _ptr(d_histogram), num_bins, lower_level,
                                         upper_level, float(inverse_delta), _stream(stream)), "histogram_even")


def histogram_range(d_key_in, num_elements: int, d_histogram, num_bins: int, d_levels, stream=None) -> None:
    """multisplit2_histogram_range_* (src/kernels/histogram/multisplit2_histograms.cuh:403-699)."""
    check(_lib.load().gms_histogram_range(_ptr(d_key_in), num_elements, _ptr(d_histogram), num_bins, _ptr(d_levels),
                                          _stream(stream)), "histogram_range")
