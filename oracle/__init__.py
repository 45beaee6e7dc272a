"""CPU oracle for the multisplit hot path -- TEST INFRASTRUCTURE ONLY.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use this
package, and only as the checker or the timed CPU baseline; the library never
calls it.

  liboracle.so   plain-C restatement of the reference's CPU multisplit
                 (src/cpu_functions.h:155-288) plus histogram, tile counts,
                 the sort digit schedules, partial-key sorts and compaction
                 (oracle.c cites each), and the same multisplit and sort
                 for 64-bit keys.
  libgms_ref.so  the reference's OWN cpu_multisplit_general /
                 cpu_multisplit_pairs_general compiled from its sources
                 (ref_shim.cpp, `make ref`); built only where the reference
                 tree exists, used to generate and check tests/golden/.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from dataclasses import dataclass, field
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "_build" / "liboracle.so"
REF_LIB = HERE / "_ref" / "libgms_ref.so"
# The reference's source tree: GMS_REFERENCE_SRC, else the project checked out
# beside this repository (../reference/src relative to the repository root).
REF_SRC = Path(os.environ.get("GMS_REFERENCE_SRC", str(HERE.parent.parent / "reference" / "src")))

DELTA, DIV, BITS, RANGE, MASK, EVEN_FLOAT = range(6)


class _CDesc(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int32), ("num_buckets", ctypes.c_uint32), ("shift", ctypes.c_uint32),
                ("param", ctypes.c_uint32), ("lower", ctypes.c_uint32), ("inverse_delta", ctypes.c_float),
                ("splitters", ctypes.c_void_p)]


@dataclass
class Desc:
    """Bucket identifier (same meaning as gms_bucket_desc; splitters on the host)."""

    kind: int
    num_buckets: int
    shift: int = 0
    param: int = 0
    lower: int = 0
    inverse_delta: float = 0.0
    splitters: np.ndarray | None = field(default=None, repr=False)

    def c(self) -> _CDesc:
        d = _CDesc(self.kind, self.num_buckets, self.shift, self.param, self.lower, self.inverse_delta, None)
        if self.splitters is not None:
            self._keep = np.ascontiguousarray(self.splitters, dtype=np.uint32)
            d.splitters = self._keep.ctypes.data
        return d


def build(with_ref: bool | None = None) -> None:
    """Compile liboracle.so, and libgms_ref.so when the reference tree is present."""
    subprocess.run(["make", "-s", "-C", str(HERE)], check=True)
    if with_ref is None:
        with_ref = (REF_SRC / "cpu_functions.h").exists()
    if with_ref:
        subprocess.run(["make", "-s", "-C", str(HERE), "ref", f"REF_SRC={REF_SRC}"], check=True)


_lib = None
_ref = None


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        if not LIB.exists():
            build(with_ref=False)
        _lib = ctypes.CDLL(str(LIB))
    return _lib


def ref_available() -> bool:
    return REF_LIB.exists()


def ref() -> ctypes.CDLL:
    global _ref
    if _ref is None:
        _ref = ctypes.CDLL(str(REF_LIB))
    return _ref


def _u32(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.uint32)


def _p(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


def buckets(keys, d: Desc) -> np.ndarray:
    keys = _u32(keys)
    cd = d.c()
    f = lib().oracle_bucket
    f.restype = ctypes.c_uint32
    return np.array([f(ctypes.byref(cd), ctypes.c_uint32(int(k))) for k in keys], dtype=np.uint32)


def multisplit(keys, d: Desc, values=None):
    """Stable multisplit -> (keys_out, values_out or None, bucket offsets)."""
    keys = _u32(keys)
    n = keys.size
    kout = np.empty(n, np.uint32)
    offs = np.empty(d.num_buckets, np.uint32)
    cd = d.c()
    if values is None:
        lib().oracle_multisplit_keys(_p(keys), _p(kout), ctypes.c_uint32(n), ctypes.byref(cd), _p(offs))
        return kout, None, offs
    values = _u32(values)
    vout = np.empty(n, np.uint32)
    lib().oracle_multisplit_pairs(_p(keys), _p(kout), _p(values), _p(vout), ctypes.c_uint32(n), ctypes.byref(cd),
                                  _p(offs))
    return kout, vout, offs


def multisplit_mt(keys, d: Desc, values=None, threads: int | None = None):
    """Multi-threaded restatement (CPU baseline); same output as multisplit()."""
    keys = _u32(keys)
    n = keys.size
    kout = np.empty(n, np.uint32)
    vout = np.empty(n, np.uint32) if values is not None else None
    values = _u32(values) if values is not None else None
    cd = d.c()
    lib().oracle_multisplit_mt(_p(keys), _p(kout), _p(values), _p(vout), ctypes.c_uint32(n), ctypes.byref(cd),
                               ctypes.c_int(threads or os.cpu_count() or 1))
    return kout, vout


def tile_counts(keys, d: Desc, tile: int) -> np.ndarray:
    """Bucket-major per-tile counts, shape (B, num_tiles)."""
    keys = _u32(keys)
    tiles = (keys.size + tile - 1) // tile
    out = np.empty(d.num_buckets * tiles, np.uint32)
    cd = d.c()
    lib().oracle_tile_counts(_p(keys), ctypes.c_uint32(keys.size), ctypes.byref(cd), ctypes.c_uint32(tile), _p(out))
    return out.reshape(d.num_buckets, tiles)


def histogram(keys, d: Desc) -> np.ndarray:
    keys = _u32(keys)
    hist = np.zeros(d.num_buckets, np.int32)
    cd = d.c()
    lib().oracle_histogram(_p(keys), ctypes.c_uint32(keys.size), ctypes.byref(cd), _p(hist))
    return hist


def sort(keys, values=None, digit_bits: int = 7):
    """Multisplit radix sort with the reference's schedule for `digit_bits` (4..8)."""
    keys = _u32(keys)
    n = keys.size
    kout, tk = np.empty(n, np.uint32), np.empty(n, np.uint32)
    vout = tv = None
    if values is not None:
        values = _u32(values)
        vout, tv = np.empty(n, np.uint32), np.empty(n, np.uint32)
    rc = lib().oracle_sort(_p(keys), _p(kout), _p(values), _p(vout), ctypes.c_uint32(n), _p(tk), _p(tv),
                           ctypes.c_int(digit_bits))
    if rc != 0:
        raise ValueError(f"unknown digit width {digit_bits}")
    return kout, vout


def sort_7bit(keys, values=None):
    return sort(keys, values, 7)


def sort_bits(keys, values=None, begin_bit: int = 0, end_bit: int = 32, digit_bits: int = 8):
    """Stable sort by key bits [begin_bit, end_bit) in digit_bits-wide multisplit passes."""
    keys = _u32(keys)
    n = keys.size
    kout, tk = np.empty(n, np.uint32), np.empty(n, np.uint32)
    vout = tv = None
    if values is not None:
        values = _u32(values)
        vout, tv = np.empty(n, np.uint32), np.empty(n, np.uint32)
    rc = lib().oracle_sort_bits(_p(keys), _p(kout), _p(values), _p(vout), ctypes.c_uint32(n), _p(tk), _p(tv),
                                ctypes.c_int(begin_bit), ctypes.c_int(end_bit), ctypes.c_int(digit_bits))
    if rc != 0:
        raise ValueError("invalid bit range or digit width")
    return kout, vout


def compaction(keys, d: Desc, values=None):
    """Two-bucket stable multisplit -> (keys_out, values_out, bucket-0 count)."""
    keys = _u32(keys)
    n = keys.size
    kout = np.empty(n, np.uint32)
    vout = np.empty(n, np.uint32) if values is not None else None
    values = _u32(values) if values is not None else None
    cd = d.c()
    f = lib().oracle_compaction
    f.restype = ctypes.c_uint32
    n0 = f(_p(keys), _p(kout), _p(values), _p(vout), ctypes.c_uint32(n), ctypes.byref(cd))
    return kout, vout, int(n0)


def uniform_u32(n: int, seed: int) -> np.ndarray:
    out = np.empty(n, np.uint32)
    lib().oracle_uniform_u32(_p(out), ctypes.c_uint64(n), ctypes.c_uint64(seed))
    return out


# ------------------------------------------------------------- 64-bit keys


class _CDesc64(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int32), ("num_buckets", ctypes.c_uint32), ("shift", ctypes.c_uint32),
                ("inverse_delta", ctypes.c_float), ("param", ctypes.c_uint64), ("lower", ctypes.c_uint64),
                ("splitters", ctypes.c_void_p)]


@dataclass
class Desc64:
    """Bucket identifier on 64-bit keys (same meaning as gms_bucket_desc64; splitters on the host)."""

    kind: int
    num_buckets: int
    shift: int = 0
    param: int = 0
    lower: int = 0
    inverse_delta: float = 0.0
    splitters: np.ndarray | None = field(default=None, repr=False)

    def c(self) -> _CDesc64:
        d = _CDesc64(self.kind, self.num_buckets, self.shift, self.inverse_delta, self.param, self.lower, None)
        if self.splitters is not None:
            self._keep = np.ascontiguousarray(self.splitters, dtype=np.uint64)
            d.splitters = self._keep.ctypes.data
        return d


def _u64(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.uint64)


def _values(values):
    """(contiguous array, element bytes) of a value array of 4- or 8-byte elements, or (None, 0)."""
    if values is None:
        return None, 0
    v = np.ascontiguousarray(values)
    if v.dtype.itemsize not in (4, 8):
        raise ValueError("values must have 4- or 8-byte elements")
    return v, v.dtype.itemsize


def buckets64(keys, d: Desc64) -> np.ndarray:
    keys = _u64(keys)
    cd = d.c()
    f = lib().oracle_bucket64
    f.restype = ctypes.c_uint32
    return np.array([f(ctypes.byref(cd), ctypes.c_uint64(int(k))) for k in keys], dtype=np.uint32)


def multisplit64(keys, d: Desc64, values=None):
    """Stable multisplit of 64-bit keys -> (keys_out, values_out or None, bucket offsets).
    Values are any 4- or 8-byte elements."""
    keys = _u64(keys)
    n = keys.size
    v, vb = _values(values)
    kout = np.empty(n, np.uint64)
    vout = np.empty_like(v) if v is not None else None
    offs = np.empty(d.num_buckets, np.uint32)
    cd = d.c()
    lib().oracle_multisplit64(_p(keys), _p(kout), _p(v), _p(vout), ctypes.c_int(vb), ctypes.c_uint32(n),
                              ctypes.byref(cd), _p(offs))
    return kout, vout, offs


def histogram64(keys, d: Desc64) -> np.ndarray:
    keys = _u64(keys)
    hist = np.zeros(d.num_buckets, np.int32)
    cd = d.c()
    lib().oracle_histogram64(_p(keys), ctypes.c_uint32(keys.size), ctypes.byref(cd), _p(hist))
    return hist


def sort_bits64(keys, values=None, begin_bit: int = 0, end_bit: int = 64, digit_bits: int = 8):
    """Stable sort of 64-bit keys by bits [begin_bit, end_bit) in digit_bits-wide passes."""
    keys = _u64(keys)
    n = keys.size
    v, vb = _values(values)
    kout, tk = np.empty(n, np.uint64), np.empty(n, np.uint64)
    vout = np.empty_like(v) if v is not None else None
    tv = np.empty_like(v) if v is not None else None
    rc = lib().oracle_sort_bits64(_p(keys), _p(kout), _p(v), _p(vout), ctypes.c_int(vb), ctypes.c_uint32(n), _p(tk),
                                  _p(tv), ctypes.c_int(begin_bit), ctypes.c_int(end_bit), ctypes.c_int(digit_bits))
    if rc != 0:
        raise ValueError("invalid bit range or digit width")
    return kout, vout


# ------------------------------------------------ the reference's own CPU code


def ref_multisplit(keys, d: Desc, values=None):
    """The reference's cpu_multisplit_general / _pairs_general with bucket ids from oracle_bucket."""
    keys = _u32(keys)
    n = keys.size
    kout = np.empty(n, np.uint32)
    vout = np.empty(n, np.uint32) if values is not None else None
    values = _u32(values) if values is not None else None
    cd = d.c()
    ref().ref_multisplit(_p(keys), _p(kout), _p(values), _p(vout), ctypes.c_uint32(n), ctypes.byref(cd))
    return kout, vout


def ref_multisplit_functor(keys, kind: int, num_buckets: int, param: int = 0, values=None):
    """The reference's CPU multisplit with reference-style functors: kind 0 top bits
    (key*B>>32), 1 key/param (delta_func), 2 (key>>param)&(B-1) (ms_bucket_sort)."""
    keys = _u32(keys)
    n = keys.size
    kout = np.empty(n, np.uint32)
    vout = np.empty(n, np.uint32) if values is not None else None
    values = _u32(values) if values is not None else None
    ref().ref_multisplit_functor(_p(keys), _p(kout), _p(values), _p(vout), ctypes.c_uint32(n), ctypes.c_int(kind),
                                 ctypes.c_uint32(num_buckets), ctypes.c_uint32(param))
    return kout, vout


def ref_sort(keys, values=None, digit_bits: int = 7):
    """The reference's digit schedule for `digit_bits` run on the reference's CPU multisplit."""
    keys = _u32(keys)
    n = keys.size
    kout, tk = np.empty(n, np.uint32), np.empty(n, np.uint32)
    vout = tv = None
    if values is not None:
        values = _u32(values)
        vout, tv = np.empty(n, np.uint32), np.empty(n, np.uint32)
    ref().ref_sort(_p(keys), _p(kout), _p(values), _p(vout), ctypes.c_uint32(n), _p(tk), _p(tv),
                   ctypes.c_int(digit_bits))
    return kout, vout


def ref_sort_7bit(keys, values=None):
    return ref_sort(keys, values, 7)
