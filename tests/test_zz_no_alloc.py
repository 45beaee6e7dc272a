"""The allocation-free key-value multisplit (gms_multisplit_key_value_noalloc).

It serves callers that cannot call cudaMalloc where they need a multisplit, so
its scratch is a fixed array in device memory owned by the library.  This file
sorts last on purpose: if it fails, a run that stops at the first failure has
already run every other test.  It passes alone in a fresh process and after the
other tests (the shared array keeps the previous call's contents, which every
call overwrites before reading).
"""
import ctypes

import numpy as np
import pytest
import torch

import gpumultisplit_gb300 as gms
from gpumultisplit_gb300 import _lib, datagen

pytestmark = pytest.mark.gpu

LIMIT = 4 << 20  # GMS_NOALLOC_SCRATCH_BYTES


def existing_entry_point(keys, vals, B, ident):
    n = keys.numel()
    ko, vo = torch.empty_like(keys), torch.empty_like(vals)
    ctx = gms.multisplit_context(B)
    gms.multisplit_allocate_key_value(n, ctx)
    gms.multisplit_key_value(keys, vals, ko, vo, n, ctx, ident)
    torch.cuda.synchronize()
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


@pytest.mark.parametrize("B,n", [(256, 1_000_003), (8, 3_000_001), (2, 4097)])
def test_noalloc_matches_existing_entry_point_twice(B, n):
    from gpumultisplit_gb300 import build as gbuild

    gbuild.build()
    lib = gms.load()
    ident = gms.delta_bucket()
    # two calls in a row with different inputs: the second must not see the first's state
    for call, seed in enumerate((11, 12)):
        keys = datagen.uniform_u32(n, seed + B, device="cuda")
        vals = datagen.index_values(n, "cuda")
        rk, rv = existing_entry_point(keys, vals, B, ident)
        st, gk, gv = noalloc(lib, keys, vals, B, ident)
        assert st == _lib.GMS_SUCCESS, (call, _lib.status_string(st))
        assert torch.equal(gk, rk), f"keys differ on call {call}"
        assert torch.equal(gv, rv), f"values differ on call {call}"


def test_noalloc_rejects_sizes_over_its_fixed_scratch():
    lib = gms.load()
    need = ctypes.c_size_t()
    n = 20_000_000  # needs more than 4 MiB of count matrix at 256 buckets
    assert lib.gms_multisplit_scratch_bytes(n, 256, 1, ctypes.byref(need)) == 0 and need.value > LIMIT
    desc = gms.delta_bucket().desc(256)
    st = lib.gms_multisplit_key_value_noalloc(1 << 40, 2 << 40, 3 << 40, 4 << 40, n, ctypes.byref(desc), None)
    assert st == _lib.GMS_ERROR_SCRATCH_TOO_SMALL
    # and the range it accepts is exercised against the host-side limit: the
    # reported scratch size includes a byte per key that only costly
    # identifiers use, so a delta multisplit needs that much less
    def delta_bytes(m):
        assert lib.gms_multisplit_scratch_bytes(m, 256, 1, ctypes.byref(need)) == 0
        return need.value - (m + 255) // 256 * 256

    ok = max(m for m in (1 << 20, 1 << 23, 15_000_000) if delta_bytes(m) <= LIMIT)
    assert ok >= 1 << 23
