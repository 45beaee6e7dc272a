"""Full-size (2^28) checks through size-independent properties, evaluated on the
GPU: the output is a permutation of the input (values = index), keys sit in
ascending bucket order, equal-bucket keys keep input order, bucket sizes equal
the histogram, and the 7-bit sort is sorted and stable."""
import pytest
import torch

import gpumultisplit_gb300 as gms
from gpumultisplit_gb300 import datagen

pytestmark = [pytest.mark.gpu, pytest.mark.slow]

N = 1 << 28


def u64(t):
    return t.to(torch.int64) & 0xFFFFFFFF


def check_multisplit_properties(kin, vin, kout, vout, bucket_of, B):
    n = kin.numel()
    # permutation: every index appears once, and keys travelled with their values
    seen = torch.zeros(n, dtype=torch.int8, device="cuda")
    seen[vout.long()] = 1
    assert bool(seen.all())
    del seen
    assert torch.equal(kout, kin[vout.long()])
    b = bucket_of(u64(kout))
    assert bool((b[1:] >= b[:-1]).all()), "buckets not ascending"
    same = b[1:] == b[:-1]
    assert bool((vout[1:] > vout[:-1])[same].all()), "input order not kept inside a bucket"
    hist = torch.zeros(B, dtype=torch.int32, device="cuda")
    return b, hist


@pytest.mark.parametrize("dist", ["uniform", "zipf"])
def test_kv_multisplit_b256_full_size(gms_lib, dist):
    B = 256
    kin = (datagen.uniform_u32 if dist == "uniform" else datagen.zipf_u32)(N, 3, device="cuda")
    vin = datagen.index_values(N, "cuda")
    kout, vout = torch.empty_like(kin), torch.empty_like(vin)
    ctx = gms.multisplit_context(B)
    gms.multisplit_allocate_key_value(N, ctx)
    offs = gms.multisplit_key_value(kin, vin, kout, vout, N, ctx, gms.delta_bucket(), multisplit_offset=True)
    torch.cuda.synchronize()
    assert gms.read_device_error(ctx) == 0
    b, hist = check_multisplit_properties(kin, vin, kout, vout, lambda k: k >> 24, B)
    gms.multisplit_histogram(kin, N, hist, B, gms.delta_bucket())
    counts = torch.bincount(b, minlength=B).to(torch.int64)
    assert torch.equal(hist.to(torch.int64), counts)
    starts = torch.cumsum(counts, 0) - counts
    assert offs == [int(x) for x in starts.cpu()]


def test_kv_multisplit_range_b256_full_size(gms_lib):
    B = 256
    kin = datagen.uniform_u32(N, 4, device="cuda")
    vin = datagen.index_values(N, "cuda")
    spl = datagen.range_splitters(B, 5, "cuda")
    kout, vout = torch.empty_like(kin), torch.empty_like(vin)
    ctx = gms.multisplit_context(B)
    gms.multisplit_allocate_key_value(N, ctx)
    gms.multisplit_key_value(kin, vin, kout, vout, N, ctx, gms.range_bucket(spl))
    torch.cuda.synchronize()
    spl64 = u64(spl)
    check_multisplit_properties(kin, vin, kout, vout,
                                lambda k: torch.searchsorted(spl64, k, right=True) - 1, B)


@pytest.mark.parametrize("dist", ["uniform", "and4"])
def test_sort7_pairs_full_size(gms_lib, dist):
    kin = (datagen.uniform_u32 if dist == "uniform" else datagen.and4_u32)(N, 6, device="cuda")
    vin = datagen.index_values(N, "cuda")
    kout, vout = torch.empty_like(kin), torch.empty_like(vin)
    ctx = gms.ms_sort_context()
    gms.multisplit_sort_7bit_allocate_pairs(N, ctx)
    gms.multisplit_sort_7bit_pairs(kin, kout, vin, vout, N, ctx)
    torch.cuda.synchronize()
    k = u64(kout)
    assert bool((k[1:] >= k[:-1]).all()), "not sorted"
    assert torch.equal(kout, kin[vout.long()])
    same = k[1:] == k[:-1]
    assert bool((vout[1:] > vout[:-1])[same].all()), "not stable"
