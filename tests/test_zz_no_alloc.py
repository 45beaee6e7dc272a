"""The allocation-free key-value multisplit (gms_multisplit_key_value_noalloc).

It serves callers that cannot call cudaMalloc where they need a multisplit, so
its scratch is a fixed array in device memory owned by the library.  This file
sorts last on purpose: if it fails, a run that stops at the first failure has
already run every other test.  It passes alone in a fresh process and after the
other tests (the shared array keeps the previous call's contents, which every
call overwrites before reading).

Every case calls the entry point itself and compares its output with the
allocating entry point's (gms_multisplit_key_value) bit for bit, on two calls in
a row with different inputs.
"""
import ctypes

import pytest
import torch

import gpumultisplit_gb300 as gms
from gpumultisplit_gb300 import _lib, datagen

pytestmark = pytest.mark.gpu

LIMIT = 4 << 20  # GMS_NOALLOC_SCRATCH_BYTES
# The largest n at 256 buckets: 4093 tiles of 4096 pairs.  The count matrix
# (1 KiB per tile), the 256-byte header and the scan status words (8 bytes per
# 4096 counts, rounded up to 256 bytes) then fill 4,193,536 of the 4 MiB.
MAX_N_B256 = 4093 * 4096


def existing_entry_point(keys, vals, B, ident):
    n = keys.numel()
    ko, vo = torch.empty_like(keys), torch.empty_like(vals)
    ctx = gms.multisplit_context(B)
    gms.multisplit_allocate_key_value(n, ctx)
    gms.multisplit_key_value(keys, vals, ko, vo, n, ctx, ident)
    torch.cuda.synchronize()
    del ctx
    return ko, vo


def noalloc(lib, keys, vals, B, ident):
    n = keys.numel()
    ko, vo = torch.full_like(keys, -1), torch.full_like(vals, -1)
    desc = ident.desc(B)
    st = lib.gms_multisplit_key_value_noalloc(keys.data_ptr() if n else None, vals.data_ptr() if n else None,
                                              ko.data_ptr() if n else None, vo.data_ptr() if n else None, n,
                                              ctypes.byref(desc), torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    return st, ko, vo


def _ident(kind, B, seed):
    if kind == "delta":
        return gms.delta_bucket(), None
    spl = datagen.range_splitters(B, seed).cuda()
    return gms.range_bucket(spl), spl


@pytest.mark.parametrize("kind,B,n", [
    ("delta", 256, 1_000_003),
    ("delta", 8, 3_000_001),
    ("delta", 2, 4097),
    ("delta", 256, 8_000_000),          # past the old, too strict check (about 3.35 M)
    ("delta", 256, MAX_N_B256),         # the largest accepted n at 256 buckets
    ("range", 256, 8_388_608),          # costly identifier: no room for bucket bytes, evaluated in both stages
    ("range", 100, 200_003),            # costly identifier with room for its bucket bytes in the array
    ("delta", 1000, 100_003),           # two digit passes with ping-pong keys and values in the array
])
def test_noalloc_matches_existing_entry_point_twice(kind, B, n):
    from gpumultisplit_gb300 import build as gbuild

    gbuild.build()
    lib = gms.load()
    # two calls in a row with different inputs: the second must not see the first's state
    for call, seed in enumerate((11, 12)):
        ident, keep = _ident(kind, B, seed)
        keys = datagen.uniform_u32(n, seed + B, device="cuda")
        vals = datagen.index_values(n, "cuda")
        rk, rv = existing_entry_point(keys, vals, B, ident)
        st, gk, gv = noalloc(lib, keys, vals, B, ident)
        assert st == _lib.GMS_SUCCESS, (call, _lib.status_string(st))
        assert torch.equal(gk, rk), f"keys differ on call {call}"
        assert torch.equal(gv, rv), f"values differ on call {call}"
        del keep


@pytest.mark.parametrize("B,n", [(256, MAX_N_B256 + 1), (256, 20_000_000), (1000, 2_000_000)])
def test_noalloc_rejects_sizes_over_its_fixed_scratch(B, n):
    lib = gms.load()
    keys = torch.zeros(n, dtype=torch.int32, device="cuda")
    vals = torch.zeros(n, dtype=torch.int32, device="cuda")
    st, gk, gv = noalloc(lib, keys, vals, B, gms.delta_bucket())
    assert st == _lib.GMS_ERROR_SCRATCH_TOO_SMALL, _lib.status_string(st)
    assert bool((gk == -1).all()) and bool((gv == -1).all()), "a rejected call wrote its output"
