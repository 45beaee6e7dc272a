"""Serving form: a continuous-batching request loop over the multisplit, 7-bit
sort, histogram and compaction operations (the native scheduler in
csrc/serve.cu, driven through the C ABI).

    server = Server(arena_bytes=64 << 30)          # device arena = HBM budget
    rid = server.submit("multisplit", keys, values, n, num_buckets=256,
                        identifier=delta_bucket())
    res = server.wait(rid)                          # Result: tensors in the arena
    server.release(rid)
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass

import torch

from . import _lib
from ._lib import BucketDesc, check
from .api import BucketIdentifier, _ptr, bits_bucket

OPS = {"multisplit": 0, "sort7": 1, "histogram": 2, "compaction": 3}


class GmsRequest(ctypes.Structure):
    _fields_ = [("op", ctypes.c_int32), ("d_key_in", ctypes.c_void_p), ("d_value_in", ctypes.c_void_p),
                ("n", ctypes.c_uint32), ("desc", BucketDesc)]


class GmsResult(ctypes.Structure):
    _fields_ = [("done", ctypes.c_int32), ("status", ctypes.c_int32), ("d_key_out", ctypes.c_void_p),
                ("d_value_out", ctypes.c_void_p), ("d_histogram", ctypes.c_void_p), ("num_bucket0", ctypes.c_uint32),
                ("rounds", ctypes.c_uint32), ("submit_s", ctypes.c_double), ("admit_s", ctypes.c_double),
                ("done_s", ctypes.c_double)]


class GmsServerStats(ctypes.Structure):
    _fields_ = [("submitted", ctypes.c_uint64), ("completed", ctypes.c_uint64), ("rounds", ctypes.c_uint64),
                ("launches", ctypes.c_uint64), ("keys", ctypes.c_uint64), ("arena_peak_bytes", ctypes.c_uint64),
                ("max_requests_in_round", ctypes.c_uint32)]


_SERVER_PROTOS = {
    "gms_server_create": ([ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p], ctypes.c_int32),
    "gms_server_submit": ([ctypes.c_void_p, ctypes.POINTER(GmsRequest), ctypes.POINTER(ctypes.c_uint64)],
                          ctypes.c_int32),
    "gms_server_poll": ([ctypes.c_void_p, ctypes.c_uint64, ctypes.POINTER(GmsResult)], ctypes.c_int32),
    "gms_server_wait": ([ctypes.c_void_p, ctypes.c_uint64, ctypes.POINTER(GmsResult)], ctypes.c_int32),
    "gms_server_take_completed": ([ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint32,
                                   ctypes.POINTER(ctypes.c_uint32)], ctypes.c_int32),
    "gms_server_release": ([ctypes.c_void_p, ctypes.c_uint64], ctypes.c_int32),
    "gms_server_drain": ([ctypes.c_void_p], ctypes.c_int32),
    "gms_server_get_stats": ([ctypes.c_void_p, ctypes.POINTER(GmsServerStats)], ctypes.c_int32),
    "gms_server_clock": ([ctypes.c_void_p], ctypes.c_double),
    "gms_server_destroy": ([ctypes.c_void_p], ctypes.c_int32),
}


def _lib_server():
    """The library with the server entry points typed to the structures above."""
    lib = _lib.load()
    if not getattr(lib, "_server_protos", False):
        for name, (args, res) in _SERVER_PROTOS.items():
            fn = getattr(lib, name)
            fn.argtypes = args
            fn.restype = res
        lib._server_protos = True
    return lib


@dataclass
class Result:
    status: int
    keys: torch.Tensor | None
    values: torch.Tensor | None
    histogram: torch.Tensor | None
    num_bucket0: int
    rounds: int
    submit_s: float
    admit_s: float
    done_s: float

    @property
    def latency_s(self) -> float:
        return self.done_s - self.submit_s


class Server:
    """Continuous-batching server over a device arena of `arena_bytes` (allocated
    here with torch, or pass `arena` = a CUDA uint8 tensor)."""

    def __init__(self, arena_bytes: int | None = None, arena: torch.Tensor | None = None):
        if arena is None:
            arena = torch.empty(int(arena_bytes), dtype=torch.uint8, device="cuda")
        self.arena = arena
        self._meta = {}
        h = ctypes.c_void_p()
        check(_lib_server().gms_server_create(arena.data_ptr(), arena.numel(), ctypes.byref(h)), "gms_server_create")
        self._h = h

    def clock(self) -> float:
        return _lib_server().gms_server_clock(self._h)

    def submit(self, op: str, keys, values, n: int, num_buckets: int = 2,
               identifier: BucketIdentifier | None = None) -> int:
        """Queue a request; returns its id.  keys/values: device tensors (values may be None)."""
        opc = OPS[op]
        ident = identifier if identifier is not None else bits_bucket(0)
        desc = ident.desc(num_buckets) if opc != OPS["sort7"] else BucketDesc()
        req = GmsRequest(opc, _ptr(keys), _ptr(values), int(n), desc)
        rid = ctypes.c_uint64()
        check(_lib_server().gms_server_submit(self._h, ctypes.byref(req), ctypes.byref(rid)), "gms_server_submit")
        self._meta[rid.value] = (op, int(n), values is not None, num_buckets, ident)
        return rid.value

    def _result(self, rid: int, r: GmsResult) -> Result:
        op, n, kv, nb, _ = self._meta[rid]

        def view(addr, count, dtype=torch.int32):
            if count == 0:
                return torch.empty(0, dtype=dtype, device="cuda")
            if not addr:
                return None
            off = addr - self.arena.data_ptr()
            return self.arena[off:off + 4 * count].view(dtype)

        hist = view(r.d_histogram, nb) if op == "histogram" else None
        return Result(r.status, view(r.d_key_out, n) if op != "histogram" else None,
                      view(r.d_value_out, n) if kv and op != "histogram" else None, hist, r.num_bucket0, r.rounds,
                      r.submit_s, r.admit_s, r.done_s)

    def poll(self, rid: int) -> Result | None:
        r = GmsResult()
        check(_lib_server().gms_server_poll(self._h, rid, ctypes.byref(r)), "gms_server_poll")
        return self._result(rid, r) if r.done else None

    def wait(self, rid: int) -> Result:
        r = GmsResult()
        check(_lib_server().gms_server_wait(self._h, rid, ctypes.byref(r)), "gms_server_wait")
        return self._result(rid, r)

    def take_completed(self, max_ids: int = 4096) -> list[int]:
        ids = (ctypes.c_uint64 * max_ids)()
        cnt = ctypes.c_uint32()
        check(_lib_server().gms_server_take_completed(self._h, ids, max_ids, ctypes.byref(cnt)),
              "gms_server_take_completed")
        return list(ids[:cnt.value])

    def release(self, rid: int) -> None:
        check(_lib_server().gms_server_release(self._h, rid), "gms_server_release")
        self._meta.pop(rid, None)

    def drain(self) -> None:
        check(_lib_server().gms_server_drain(self._h), "gms_server_drain")

    def stats(self) -> dict:
        s = GmsServerStats()
        check(_lib_server().gms_server_get_stats(self._h, ctypes.byref(s)), "gms_server_get_stats")
        return {k: getattr(s, k) for k, _ in GmsServerStats._fields_}

    def close(self) -> None:
        if self._h:
            _lib_server().gms_server_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
