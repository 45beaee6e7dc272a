"""A bounded device wait that runs out, and the error the host reads afterwards.

The scan's decoupled look-back waits for its predecessor chunk to publish.  Here
the scan's ticket counter is left at 1 after the prescan, so the block that
draws ticket 1 waits on a chunk 0 that no block will ever scan: a flag that
nothing sets.  With the call's wait limit set to 2 ms in the scratch header the
wait gives up, the kernel records DEV_ERR_LOOKBACK_TIMEOUT, publishes anyway and
returns.  Nothing faults and nothing waits longer than the limit; the same
scratch then serves a normal call.
"""
import ctypes
import time

import numpy as np
import pytest
import torch

import gpumultisplit_gb300 as gms
from gpumultisplit_gb300 import _lib, datagen

pytestmark = pytest.mark.gpu

DEV_ERR_LOOKBACK_TIMEOUT = 2
# Header words (uint32) of the scratch: error, error_info, ticket, wait_limit_us.
TICKET, WAIT_LIMIT_US = 2, 3


def test_lookback_wait_runs_out_and_is_reported(gms_lib, oracle_mod):
    lib = gms_lib
    B = 256
    n = 17 * 4096  # 17 tiles x 256 buckets = 4352 counts: two scan chunks of 4096
    keys_h = datagen.as_u32(datagen.uniform_u32(n, 3))
    vals_h = np.arange(n, dtype=np.uint32)
    dk, dv = datagen.from_u32(keys_h, "cuda"), datagen.from_u32(vals_h, "cuda")
    ok, ov = torch.empty_like(dk), torch.empty_like(dv)
    ctx = gms.multisplit_context(B)
    gms.multisplit_allocate_key_value(n, ctx)
    desc = gms.delta_bucket().desc(B)
    scratch, nbytes = ctx.d_temp_storage.data_ptr(), ctx.temp_storage_bytes
    s = torch.cuda.current_stream().cuda_stream

    assert lib.gms_multisplit_prescan(dk.data_ptr(), n, ctypes.byref(desc), 1, scratch, nbytes, s) == 0
    torch.cuda.synchronize()
    hdr = ctx.d_temp_storage[:16].view(torch.int32)
    assert int(hdr[TICKET]) == 0 and int(hdr[WAIT_LIMIT_US]) == 0, "the prescan resets ticket and limit"
    hdr[TICKET] = 1           # chunk 0 is never drawn, so chunk 1 waits on it
    hdr[WAIT_LIMIT_US] = 2000  # 2 ms instead of the default 1 s
    torch.cuda.synchronize()

    t0 = time.perf_counter()
    assert lib.gms_multisplit_scan(n, ctypes.byref(desc), 1, scratch, nbytes, s) == 0  # the launch itself succeeds
    torch.cuda.synchronize()
    waited = time.perf_counter() - t0
    assert waited < 0.5, f"the scan took {waited:.3f} s: the 2 ms limit was not applied"

    code = ctypes.c_uint32()
    st = lib.gms_read_device_error(scratch, ctypes.byref(code), s)
    assert st == _lib.GMS_ERROR_DEVICE_TIMEOUT, _lib.status_string(st)
    assert code.value == DEV_ERR_LOOKBACK_TIMEOUT
    assert gms.read_device_error(ctx) == DEV_ERR_LOOKBACK_TIMEOUT

    # The context stays usable: the next call resets the header and is bit-exact.
    gms.multisplit_key_value(dk, dv, ok, ov, n, ctx, gms.delta_bucket())
    torch.cuda.synchronize()
    assert gms.read_device_error(ctx) == 0
    assert int(hdr[WAIT_LIMIT_US]) == 0
    rk, rv, _ = oracle_mod.multisplit(keys_h, oracle_mod.Desc(oracle_mod.DELTA, B), vals_h)
    np.testing.assert_array_equal(datagen.as_u32(ok), rk)
    np.testing.assert_array_equal(datagen.as_u32(ov), rv)
