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


NUM_TILE_VARIANTS = 4
NUM_SIZE_CLASSES = 8


def size_class(n: int) -> int:
    """Tuning-table size class of a segment of n keys (0: n <= 2^10 ... 7: n > 2^16)."""
    c = 0
    while c < NUM_SIZE_CLASSES - 1 and n > (1 << (10 + c)):
        c += 1
    return c


def tile_variant_shape(variant: int) -> tuple[int, int, int]:
    """(warps per block, keys per thread, keys per tile) of a tile variant."""
    w, i, t = ctypes.c_uint32(), ctypes.c_uint32(), ctypes.c_uint32()
    check(_lib.load().gms_tile_variant_shape(variant, ctypes.byref(w), ctypes.byref(i), ctypes.byref(t)),
          "gms_tile_variant_shape")
    return w.value, i.value, t.value


def tuning_table() -> dict:
    """The current table: {(num_buckets, key_value, size_class): variant}."""
    lib = _lib.load()
    out = {}
    v = ctypes.c_int()
    for k in range(1, 9):
        for kv in (False, True):
            for c in range(NUM_SIZE_CLASSES):
                check(lib.gms_tuning_get(1 << k, int(kv), c, ctypes.byref(v)), "gms_tuning_get")
                out[(1 << k, kv, c)] = v.value
    return out


def set_tuning(table: dict) -> None:
    """Loads entries {(num_buckets, key_value, size_class): variant} into the table."""
    lib = _lib.load()
    for (b, kv, c), v in table.items():
        check(lib.gms_tuning_set(int(b), int(bool(kv)), int(c), int(v)), "gms_tuning_set")


def reset_tuning() -> None:
    check(_lib.load().gms_tuning_reset(), "gms_tuning_reset")


def autotune(buckets=(2, 4, 8, 16, 32, 64, 128, 256), key_value=(False, True), keys_per_trial: int = 1 << 24,
             reps: int = 3, stream=None) -> dict:
    """Times every valid tile variant per (bucket count, key/value, size class)
    on this device and stores the fastest in the table.  Returns
    {(num_buckets, key_value, size_class): best milliseconds}."""
    bmask = 0
    for b in buckets:
        if b < 2 or b > 256 or b & (b - 1):
            raise ValueError(f"unsupported bucket count {b}")
        bmask |= b
    kvmask = sum(1 << int(bool(kv)) for kv in set(key_value))
    ms = (ctypes.c_float * (16 * NUM_SIZE_CLASSES))()
    check(_lib.load().gms_autotune(bmask, kvmask, int(keys_per_trial), int(reps), ms, _stream(stream)),
          "gms_autotune")
    out = {}
    for b in buckets:
        k = b.bit_length() - 1
        for kv in set(key_value):
            for c in range(NUM_SIZE_CLASSES):
                out[(b, bool(kv), c)] = float(ms[((k - 1) * 2 + int(bool(kv))) * NUM_SIZE_CLASSES + c])
    return out


class BatchedMultisplit:
    """A plan over a list of Segment; run() executes every segment's multisplit.
    variant=None takes each segment's tile shape from the tuning table; an int
    forces that tile variant for every segment (the "classes" schedule).
    schedule: "classes" or "queue" (see the `schedule` property)."""

    def __init__(self, segments: list[Segment], variant: int | None = None, schedule: str = "classes"):
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
        if variant is None:
            check(lib.gms_batch_create(arr, len(segments), ctypes.byref(handle)), "gms_batch_create")
        else:
            check(lib.gms_batch_create_with_variant(arr, len(segments), int(variant), ctypes.byref(handle)),
                  "gms_batch_create_with_variant")
        self._handle = handle
        nbytes = ctypes.c_size_t()
        check(lib.gms_batch_scratch_bytes(self._handle, ctypes.byref(nbytes)), "gms_batch_scratch_bytes")
        self.scratch_bytes = nbytes.value
        self.scratch = _alloc_scratch(nbytes.value)
        if schedule != "classes":
            self.schedule = schedule

    SCHEDULES = {"classes": _lib.GMS_BATCH_SCHEDULE_CLASSES, "queue": _lib.GMS_BATCH_SCHEDULE_QUEUE}

    @property
    def schedule(self) -> str:
        """"classes": one prescan and postscan launch per segment class (the
        default); "queue": one persistent launch over a device-side work list."""
        v = ctypes.c_int()
        check(_lib.load().gms_batch_get_schedule(self._handle, ctypes.byref(v)), "gms_batch_get_schedule")
        return {c: n for n, c in self.SCHEDULES.items()}[v.value]

    @schedule.setter
    def schedule(self, name: str) -> None:
        if name not in self.SCHEDULES:
            raise ValueError(f"schedule must be one of {sorted(self.SCHEDULES)}")
        check(_lib.load().gms_batch_set_schedule(self._handle, self.SCHEDULES[name]), "gms_batch_set_schedule")

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
