"""ctypes binding of the C ABI in include/gpumultisplit.h.

The CUDA library is required: loading fails loudly (ImportError) when
libgpumultisplit.so has not been built.  There is no CPU fallback.
"""
from __future__ import annotations

import ctypes
import os
from pathlib import Path

LIB_PATH = Path(__file__).resolve().parent / "lib" / "libgpumultisplit.so"

GMS_SUCCESS = 0
GMS_ERROR_INVALID_VALUE = 1
GMS_ERROR_UNSUPPORTED_BUCKETS = 2
GMS_ERROR_SCRATCH_TOO_SMALL = 3
GMS_ERROR_CUDA = 4
GMS_ERROR_DEVICE_TIMEOUT = 5
# gms_sort_set_method
GMS_SORT_AUTO, GMS_SORT_MULTISPLIT, GMS_SORT_ONESWEEP = 0, 1, 2
GMS_BATCH_SCHEDULE_CLASSES, GMS_BATCH_SCHEDULE_QUEUE = 0, 1
GMS_ERROR_NOT_SUPPORTED = 6

GMS_BUCKET_DELTA = 0
GMS_BUCKET_DIV = 1
GMS_BUCKET_BITS = 2
GMS_BUCKET_RANGE = 3
GMS_BUCKET_MASK = 4
GMS_BUCKET_EVEN_FLOAT = 5


class BucketDesc(ctypes.Structure):
    """gms_bucket_desc."""

    _fields_ = [
        ("kind", ctypes.c_int32),
        ("num_buckets", ctypes.c_uint32),
        ("shift", ctypes.c_uint32),
        ("param", ctypes.c_uint32),
        ("lower", ctypes.c_uint32),
        ("inverse_delta", ctypes.c_float),
        ("d_splitters", ctypes.c_void_p),
    ]


class BucketDesc64(ctypes.Structure):
    """gms_bucket_desc64 (identifiers for 64-bit keys, or 32-bit keys with 64-bit values)."""

    _fields_ = [
        ("kind", ctypes.c_int32),
        ("num_buckets", ctypes.c_uint32),
        ("shift", ctypes.c_uint32),
        ("inverse_delta", ctypes.c_float),
        ("param", ctypes.c_uint64),
        ("lower", ctypes.c_uint64),
        ("d_splitters", ctypes.c_void_p),
    ]


class GmsError(RuntimeError):
    def __init__(self, status: int, what: str, cuda_error: int = 0):
        self.status = status
        self.cuda_error = cuda_error
        msg = f"{what}: {status_string(status)} (status {status})"
        if status == GMS_ERROR_CUDA:
            msg += f", cudaError {cuda_error}"
        super().__init__(msg)


_P = ctypes.c_void_p
_U32 = ctypes.c_uint32
_I32 = ctypes.c_int32
_SZ = ctypes.c_size_t
_PU32 = ctypes.POINTER(ctypes.c_uint32)
_PSZ = ctypes.POINTER(ctypes.c_size_t)
_PDESC = ctypes.POINTER(BucketDesc)
_PDESC64 = ctypes.POINTER(BucketDesc64)

# name -> argtypes (every function returns gms_status as int32 unless listed in _RESTYPES)
_PROTOS = {
    "gms_version": [],
    "gms_status_string": [_I32],
    "gms_last_cuda_error": [],
    "gms_read_device_error": [_P, _PU32, _P],
    "gms_multisplit_scratch_bytes": [_U32, _U32, _I32, _PSZ],
    "gms_multisplit_geometry": [_U32, _U32, _I32, _PU32, _PU32, _PSZ],
    "gms_multisplit_key_only": [_P, _P, _U32, _PDESC, _P, _SZ, _PU32, _P],
    "gms_multisplit_key_value": [_P, _P, _P, _P, _U32, _PDESC, _P, _SZ, _PU32, _P],
    "gms_multisplit_prescan": [_P, _U32, _PDESC, _I32, _P, _SZ, _P],
    "gms_multisplit_scan": [_U32, _PDESC, _I32, _P, _SZ, _P],
    "gms_multisplit_postscan": [_P, _P, _P, _P, _U32, _PDESC, _P, _SZ, _P],
    "gms_multisplit_key_value_noalloc": [_P, _P, _P, _P, _U32, _PDESC, _P],
    "gms_sort_scratch_bytes": [_U32, _I32, _I32, _PSZ],
    "gms_sort_set_method": [_I32],
    "gms_sort_get_method": [ctypes.POINTER(ctypes.c_int)],
    "gms_sort_key_only": [_P, _P, _U32, _I32, _P, _SZ, _P],
    "gms_sort_key_value": [_P, _P, _P, _P, _U32, _I32, _P, _SZ, _P],
    "gms_sort_bits_scratch_bytes": [_U32, _I32, _I32, _I32, _I32, _PSZ],
    "gms_sort_bits_key_only": [_P, _P, _U32, _I32, _I32, _I32, _P, _SZ, _P],
    "gms_sort_bits_key_value": [_P, _P, _P, _P, _U32, _I32, _I32, _I32, _P, _SZ, _P],
    "gms_multisplit_wide_scratch_bytes": [_U32, _U32, _I32, _I32, _PSZ],
    "gms_multisplit_wide": [_P, _P, _P, _P, _U32, _I32, _I32, _PDESC64, _P, _SZ, _PU32, _P],
    "gms_histogram_wide": [_P, _U32, _I32, _PDESC64, _P, _P],
    "gms_sort_wide_scratch_bytes": [_U32, _I32, _I32, _I32, _I32, _I32, _PSZ],
    "gms_sort_wide": [_P, _P, _P, _P, _U32, _I32, _I32, _I32, _I32, _I32, _P, _SZ, _P],
    "gms_sort_7bit_scratch_bytes": [_U32, _I32, _PSZ],
    "gms_sort_7bit_key_only": [_P, _P, _U32, _P, _SZ, _P],
    "gms_sort_7bit_key_value": [_P, _P, _P, _P, _U32, _P, _SZ, _P],
    "gms_compaction_scratch_bytes": [_U32, _I32, _PSZ],
    "gms_compaction_key_only": [_P, _P, _U32, _PDESC, _P, _SZ, _PU32, _P],
    "gms_compaction_key_value": [_P, _P, _P, _P, _U32, _PDESC, _P, _SZ, _PU32, _P],
    "gms_batch_create": [_P, _U32, _P],
    "gms_batch_scratch_bytes": [_P, _PSZ],
    "gms_batch_run": [_P, _P, _SZ, _I32, _P],
    "gms_batch_launch_count": [_P, _PU32],
    "gms_batch_destroy": [_P],
    "gms_batch_create_with_variant": [_P, _U32, _I32, _P],
    "gms_batch_set_schedule": [_P, _I32],
    "gms_batch_get_schedule": [_P, ctypes.POINTER(ctypes.c_int)],
    "gms_tile_variant_shape": [_I32, _PU32, _PU32, _PU32],
    "gms_tuning_get": [_U32, _I32, _I32, ctypes.POINTER(ctypes.c_int)],
    "gms_tuning_set": [_U32, _I32, _I32, _I32],
    "gms_tuning_reset": [],
    "gms_autotune": [_U32, _U32, _U32, _I32, ctypes.POINTER(ctypes.c_float), _P],
    "gms_server_create": [_P, _SZ, _P],
    "gms_server_submit": [_P, _P, _P],
    "gms_server_poll": [_P, ctypes.c_uint64, _P],
    "gms_server_wait": [_P, ctypes.c_uint64, _P],
    "gms_server_take_completed": [_P, _P, _U32, _PU32],
    "gms_server_release": [_P, ctypes.c_uint64],
    "gms_server_drain": [_P],
    "gms_server_get_stats": [_P, _P],
    "gms_server_clock": [_P],
    "gms_server_destroy": [_P],
    "gms_histogram": [_P, _U32, _PDESC, _P, _P],
    "gms_histogram_even": [_P, _U32, _P, _U32, _U32, _U32, ctypes.c_float, _P],
    "gms_histogram_range": [_P, _U32, _P, _U32, _P, _P],
}
_RESTYPES = {"gms_version": ctypes.c_int, "gms_status_string": ctypes.c_char_p, "gms_last_cuda_error": ctypes.c_int,
             "gms_server_clock": ctypes.c_double}

# Symbols declared in include/*.h (checked by the CPU test suite).
EXPORTED = tuple(_PROTOS)

_lib = None


def load(path: str | os.PathLike | None = None) -> ctypes.CDLL:
    """Load libgpumultisplit.so (once) and attach prototypes."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    override = os.environ.get("GMS_LIBRARY")
    p = Path(path) if path is not None else (Path(override) if override else LIB_PATH)
    if not p.exists():
        raise ImportError(
            f"{p} is missing: build the CUDA library first "
            "(python -c 'import __graft_entry__ as g; g.build()' or python gpumultisplit_gb300/build.py)")
    lib = ctypes.CDLL(str(p))
    for name, argtypes in _PROTOS.items():
        fn = getattr(lib, name)
        fn.argtypes = argtypes
        fn.restype = _RESTYPES.get(name, ctypes.c_int32)
    if path is None:
        _lib = lib
    return lib


def status_string(status: int) -> str:
    try:
        return load().gms_status_string(status).decode()
    except ImportError:
        return "unknown"


def check(status: int, what: str) -> None:
    if status != GMS_SUCCESS:
        cuda_err = load().gms_last_cuda_error() if status == GMS_ERROR_CUDA else 0
        raise GmsError(status, what, cuda_err)
