"""Batched multisplit: many independent multisplits of uneven sizes and bucket
counts run as one plan (one launch per stage and segment class, one scan over
all count matrices), optionally replayed from a captured CUDA graph.  Each
segment's output equals the plain multisplit of that segment alone."""
from __future__ import annotations

import ctypes
from dataclasses import dataclass

from . import _lib
from ._lib import BucketDesc, check
from .api import BucketIdentifier, _alloc_scratch, _ptr, _stream


class GmsSegment(ctypes.Structure):
    """gms_segment."""

    _fields_ = [
        ("d_key_in", ctypes.c_void_p),
        ("d_value_in", ctypes.c_void_p),
        ("d_key_out", ctypes.c_void_p),
        ("d_value_out", ctypes.c_void_p),
        ("n", ctypes.c_uint32),
        ("desc", BucketDesc),
    ]


@dataclass
class Segment:
    """One multisplit of a batch: device buffers (tensors or addresses), n keys,
    B buckets and the bucket identifier.  values_in/values_out None = key-only."""

    keys_in: object
    keys_out: object
    n: int
    num_buckets: int
    identifier: BucketIdentifier
    values_in: object = None
    values_out: object = None


class BatchedMultisplit:
    """A plan over a list of Segment; run() executes every segment's multisplit."""

    def __init__(self, segments: list[Segment]):
        lib = _lib.load()
        self._segments = list(segments)
        arr = (GmsSegment * max(1, len(segments)))()
        self._keep = []
        for i, s in enumerate(segments):
            desc = s.identifier.desc(s.num_buckets)
            self._keep.append(s.identifier)
            arr[i] = GmsSegment(_ptr(s.keys_in), _ptr(s.values_in), _ptr(s.keys_out), _ptr(s.values_out), int(s.n),
                                desc)
        handle = ctypes.c_void_p()
        check(lib.gms_batch_create(arr, len(segments), ctypes.byref(handle)), "gms_batch_create")
        self._handle = handle
        nbytes = ctypes.c_size_t()
        check(lib.gms_batch_scratch_bytes(self._handle, ctypes.byref(nbytes)), "gms_batch_scratch_bytes")
        self.scratch_bytes = nbytes.value
        self.scratch = _alloc_scratch(nbytes.value)

    @property
    def launches(self) -> int:
        n = ctypes.c_uint32()
        check(_lib.load().gms_batch_launch_count(self._handle, ctypes.byref(n)), "gms_batch_launch_count")
        return n.value

    def run(self, use_graph: bool = True, stream=None) -> None:
        check(_lib.load().gms_batch_run(self._handle, _ptr(self.scratch, None), self.scratch_bytes,
                                        int(bool(use_graph)), _stream(stream)), "gms_batch_run")

    def device_error(self, stream=None) -> int:
        code = ctypes.c_uint32()
        st = _lib.load().gms_read_device_error(_ptr(self.scratch, None), ctypes.byref(code), _stream(stream))
        if st not in (_lib.GMS_SUCCESS, _lib.GMS_ERROR_DEVICE_TIMEOUT):
            check(st, "read_device_error")
        return code.value

    def close(self) -> None:
        if self._handle:
            _lib.load().gms_batch_destroy(self._handle)
            self._handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
