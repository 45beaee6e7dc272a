"""Skewed warps above 32 buckets: a warp ranks its 512 keys (16 slots of 32)
with a per-warp count table, so these cases put exactly 255, 256, 300 and all
512 keys of one warp's range into one bucket, in the first and in later tiles
(8 warps x 16 keys per thread, 4096-key tiles), and make every warp of every
tile hold one or two buckets; every output is checked against the oracle."""
import numpy as np
import pytest
import torch

import gpumultisplit_gb300 as gms
from gpumultisplit_gb300 import datagen
from gpu_util import host, identifiers, to_dev

pytestmark = pytest.mark.gpu

WARP_KEYS = 512


def keys_with_runs(n, B, run, seed, where):
    """Uniform keys, except that `run` keys of the warp ranges listed in `where`
    (tile, warp) all fall into bucket 17 under delta bucketing."""
    rng = np.random.default_rng(seed)
    keys = rng.integers(0, 1 << 32, n, dtype=np.uint64).astype(np.uint32)
    lo = (17 << 32) // B
    for tile, warp in where:
        start = tile * 4096 + warp * WARP_KEYS
        idx = start + rng.choice(WARP_KEYS, size=run, replace=False)
        keys[idx] = np.uint32(lo + 5)
    return keys


@pytest.mark.parametrize("B", [64, 128, 256])
@pytest.mark.parametrize("run", [255, 256, 300, 512])
@pytest.mark.parametrize("kv", [True, False])
def test_one_bucket_runs_in_a_warp(gms_lib, oracle_mod, B, run, kv):
    n = 5 * 4096 + 1000
    keys = keys_with_runs(n, B, run, 40 + run, [(0, 0), (2, 5), (4, 7)])
    vals = np.arange(n, dtype=np.uint32)
    rk, rv, _ = oracle_mod.multisplit(keys, oracle_mod.Desc(oracle_mod.DELTA, B), vals if kv else None)
    dk, ok = to_dev(keys), torch.zeros(n, dtype=torch.int32, device="cuda")
    ctx = gms.multisplit_context(B)
    if kv:
        dv, ov = to_dev(vals), torch.zeros(n, dtype=torch.int32, device="cuda")
        gms.multisplit_allocate_key_value(n, ctx)
        gms.multisplit_key_value(dk, dv, ok, ov, n, ctx, gms.delta_bucket())
    else:
        gms.multisplit_allocate_key_only(n, ctx)
        gms.multisplit_key_only(dk, ok, n, ctx, gms.delta_bucket())
    torch.cuda.synchronize()
    assert gms.read_device_error(ctx) == 0
    np.testing.assert_array_equal(host(ok), rk)
    if kv:
        np.testing.assert_array_equal(host(ov), rv)


@pytest.mark.parametrize("B", [64, 256])
@pytest.mark.parametrize("kind", ["all_equal", "two_buckets", "range_skew"])
def test_skewed_tiles_every_warp_overflows(gms_lib, oracle_mod, B, kind):
    """Every warp of every tile overflows (all keys in one or two buckets), with
    delta and with range identifiers (the latter through the prescan's bucket bytes)."""
    n = 3 * 4096 + 123
    if kind == "all_equal":
        keys = np.full(n, 0x9E3779B9, np.uint32)
    elif kind == "two_buckets":
        keys = np.where(np.arange(n) % 5 == 0, 0x10, 0xF0000000).astype(np.uint32)
    else:
        keys = (np.random.default_rng(9).integers(0, 64, n) + 0x7FFFFF00).astype(np.uint32)
    vals = np.arange(n, dtype=np.uint32)
    o_kind = oracle_mod.RANGE if kind == "range_skew" else oracle_mod.DELTA
    ident, d, keep = identifiers(oracle_mod, o_kind, B, splitter_seed=3)
    rk, rv, _ = oracle_mod.multisplit(keys, d, vals)
    dk, dv = to_dev(keys), to_dev(vals)
    ok, ov = torch.zeros_like(dk), torch.zeros_like(dv)
    ctx = gms.multisplit_context(B)
    gms.multisplit_allocate_key_value(n, ctx)
    gms.multisplit_key_value(dk, dv, ok, ov, n, ctx, ident)
    torch.cuda.synchronize()
    assert gms.read_device_error(ctx) == 0
    np.testing.assert_array_equal(host(ok), rk)
    np.testing.assert_array_equal(host(ov), rv)
    del keep
