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


def test_kv_multisplit_beyond_2p31(gms_lib):
    """n above 2^31 (32-bit index arithmetic, values that do not fit an int32)."""
    B = 256
    n = (1 << 31) + 4099
    kin = datagen.uniform_u32(n, 8, device="cuda")
    vin = datagen.index_values(n, "cuda")
    kout, vout = torch.empty_like(kin), torch.empty_like(vin)
    ctx = gms.multisplit_context(B)
    gms.multisplit_allocate_key_value(n, ctx)
    offs = gms.multisplit_key_value(kin, vin, kout, vout, n, ctx, gms.delta_bucket(), multisplit_offset=True)
    torch.cuda.synchronize()
    assert gms.read_device_error(ctx) == 0
    del ctx
    idx = u64(vout)
    seen = torch.zeros(n, dtype=torch.int8, device="cuda")
    seen[idx] = 1
    assert bool(seen.all()), "values are not a permutation of the indices"
    del seen
    assert torch.equal(kout, kin[idx]), "keys did not travel with their values"
    b = u64(kout) >> 24
    assert bool((b[1:] >= b[:-1]).all()), "buckets not ascending"
    assert bool((idx[1:] > idx[:-1])[b[1:] == b[:-1]].all()), "input order not kept inside a bucket"
    counts = torch.bincount(b, minlength=B)
    starts = torch.cumsum(counts, 0) - counts
    assert offs == [int(x) for x in starts.cpu()]


def test_u64_kv_multisplit_beyond_2p31(gms_lib):
    """64-bit keys and values, n above 2^31: element offsets past 2^34 bytes and
    32-bit positions near their top (buckets ascending, a stable permutation,
    offsets equal to the bucket starts)."""
    B = 256
    n = (1 << 31) + 4099
    kin = datagen.uniform_u64(n, 18, device="cuda")
    vin = torch.arange(n, dtype=torch.int64, device="cuda")
    kout, vout = torch.empty_like(kin), torch.empty_like(vin)
    ctx = gms.multisplit_context(B)
    gms.multisplit_wide_allocate(n, ctx, 8, 8)
    offs = gms.multisplit_wide(kin, kout, n, ctx, gms.delta_bucket(), vin, vout, multisplit_offset=True)
    torch.cuda.synchronize()
    assert gms.read_device_error(ctx) == 0
    del ctx, vin
    seen = torch.zeros(n, dtype=torch.int8, device="cuda")
    seen[vout] = 1
    assert bool(seen.all()), "values are not a permutation of the indices"
    del seen
    assert torch.equal(kout, kin[vout]), "keys did not travel with their values"
    del kin
    b = (kout >> 56) & 0xFF  # delta on 64-bit keys at B = 256: the top 8 bits
    assert bool((b[1:] >= b[:-1]).all()), "buckets not ascending"
    assert bool((vout[1:] > vout[:-1])[b[1:] == b[:-1]].all()), "input order not kept inside a bucket"
    counts = torch.bincount(b, minlength=B)
    starts = torch.cumsum(counts, 0) - counts
    assert offs == [int(x) for x in starts.cpu()]


def test_batched_scan_groups_beyond_2p32(gms_lib):
    """A batch whose keys add up to more than 2^32 is scanned in groups; every
    segment keeps the multisplit properties (key-only: ascending buckets, and
    per-bucket counts and key sums equal to the input's)."""
    sizes = [(1 << 31) + 5, 1000, (1 << 31) + 77]
    buckets = [8, 2, 256]
    segs, ins, outs = [], [], []
    for i, (n, B) in enumerate(zip(sizes, buckets)):
        kin = datagen.uniform_u32(n, 90 + i, device="cuda")
        kout = torch.empty_like(kin)
        segs.append(gms.Segment(kin, kout, n, B, gms.delta_bucket()))
        ins.append(kin)
        outs.append(kout)
    plan = gms.BatchedMultisplit(segs)
    plan.run(use_graph=False)
    torch.cuda.synchronize()
    assert plan.device_error() == 0
    plan.close()
    for kin, kout, B in zip(ins, outs, buckets):
        shift = 32 - (B.bit_length() - 1)
        bi, bo = u64(kin) >> shift, u64(kout) >> shift
        assert bool((bo[1:] >= bo[:-1]).all())
        assert torch.equal(torch.bincount(bi, minlength=B), torch.bincount(bo, minlength=B))
        si = torch.zeros(B, dtype=torch.int64, device="cuda").scatter_add_(0, bi, u64(kin))
        so = torch.zeros(B, dtype=torch.int64, device="cuda").scatter_add_(0, bo, u64(kout))
        assert torch.equal(si, so)
        del bi, bo


def test_largest_n(gms_lib):
    """n = 2^32 - 1, the largest size the 32-bit interface takes: a histogram
    and a key-only two-bucket multisplit (checked in chunks to bound memory)."""
    n = (1 << 32) - 1
    kin = datagen.uniform_u32(n, 12, device="cuda")
    hist = torch.zeros(2, dtype=torch.int32, device="cuda")
    gms.multisplit_histogram(kin, n, hist, 2, gms.delta_bucket())
    ones = sum(int((kin[s:s + (1 << 28)] < 0).sum()) for s in range(0, n, 1 << 28))  # top bit set
    # the bins are the reference's int counters: a bin above 2^31 - 1 holds its count mod 2^32
    h0, h1 = int(hist[0]) & 0xFFFFFFFF, int(hist[1]) & 0xFFFFFFFF
    assert h1 == ones and h0 + h1 == n
    kout = torch.empty_like(kin)
    ctx = gms.multisplit_context(2)
    gms.multisplit_allocate_key_only(n, ctx)
    offs = gms.multisplit_key_only(kin, kout, n, ctx, gms.delta_bucket(), multisplit_offset=True)
    torch.cuda.synchronize()
    assert gms.read_device_error(ctx) == 0
    assert offs == [0, n - ones]
    zeros = n - ones
    # bucket 0 (top bit clear) first, then bucket 1, and the same keys in each
    assert bool((kout[:zeros] >= 0).all()) and bool((kout[zeros:] < 0).all())
    si = so = 0
    for s in range(0, n, 1 << 28):
        si += int(u64(kin[s:s + (1 << 28)]).sum())
        so += int(u64(kout[s:s + (1 << 28)]).sum())
    assert si == so
