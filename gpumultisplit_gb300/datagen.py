"""Seeded synthetic inputs for the multisplit workloads.

All generators are counter-based (splitmix64 of seed + (i+1) * golden gamma,
the published SplitMix64 finaliser of Steele, Lea and Flood, "Fast splittable
pseudorandom number generators", OOPSLA 2014), so element i depends only on
(seed, i): the same arrays come out on the CPU and on the GPU, in any chunking.

Distributions (one per benchmark configuration):
  uniform_u32   keys uniform over [0, 2^32)
  uniform_u64   keys uniform over [0, 2^64) (64-bit keys)
  and4_u32      AND of 4 uniform draws (each bit set with p = 1/16)
  zipf_u32      Zipf(s) over `distinct` key values drawn uniformly over [0, 2^32)
  range_splitters  B sorted splitters, splitter[0] = 0, the rest uniform
  segment_sizes    log-uniform segment sizes
"""
from __future__ import annotations

import math

import numpy as np
import torch

GAMMA = 0x9E3779B97F4A7C15
M1 = 0xBF58476D1CE4E5B9
M2 = 0x94D049BB133111EB
MASK64 = (1 << 64) - 1


def _s64(x: int) -> int:
    """uint64 constant as the int64 with the same bits."""
    x &= MASK64
    return x - (1 << 64) if x >= (1 << 63) else x


def _srl(z: torch.Tensor, k: int) -> torch.Tensor:
    """Logical right shift of int64 bit patterns."""
    return (z >> k) & ((1 << (64 - k)) - 1)


def splitmix64(seed: int, start: int, count: int, device="cpu") -> torch.Tensor:
    """int64 tensor holding the uint64 bit patterns splitmix64(seed, i), i in [start, start+count)."""
    i = torch.arange(start + 1, start + 1 + count, dtype=torch.int64, device=device)
    z = i * _s64(GAMMA) + _s64(seed)
    z = (z ^ _srl(z, 30)) * _s64(M1)
    z = (z ^ _srl(z, 27)) * _s64(M2)
    return z ^ _srl(z, 31)


def _hi32(z: torch.Tensor) -> torch.Tensor:
    """Top 32 bits as int32 bit patterns."""
    return _srl(z, 32).to(torch.int32)


CHUNK = 1 << 24


def uniform_u32(n: int, seed: int, device="cpu") -> torch.Tensor:
    """n keys uniform over [0, 2^32), as an int32 tensor of uint32 bit patterns."""
    out = torch.empty(n, dtype=torch.int32, device=device)
    for s in range(0, n, CHUNK):
        c = min(CHUNK, n - s)
        out[s:s + c] = _hi32(splitmix64(seed, s, c, device))
    return out


def uniform_u64(n: int, seed: int, device="cpu") -> torch.Tensor:
    """n keys uniform over [0, 2^64): the full splitmix64 output, as an int64
    tensor of uint64 bit patterns."""
    out = torch.empty(n, dtype=torch.int64, device=device)
    for s in range(0, n, CHUNK):
        c = min(CHUNK, n - s)
        out[s:s + c] = splitmix64(seed, s, c, device)
    return out


def as_u64(t: torch.Tensor) -> np.ndarray:
    """Host numpy uint64 view of an int64 tensor."""
    return t.detach().cpu().numpy().view(np.uint64)


def from_u64(a: np.ndarray, device="cpu") -> torch.Tensor:
    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.uint64).view(np.int64)).to(device)


def and4_u32(n: int, seed: int, device="cpu") -> torch.Tensor:
    """AND of four independent uniform draws (reduced-entropy sort keys)."""
    out = uniform_u32(n, seed * 4 + 1, device)
    for k in (2, 3, 4):
        out &= uniform_u32(n, seed * 4 + k, device)
    return out


def index_values(n: int, device="cpu") -> torch.Tensor:
    """values = original index (pins value stability), as uint32 bit patterns in
    int32 (indices from 2^31 up wrap to negative int32 values)."""
    if n <= 1 << 31:
        return torch.arange(n, dtype=torch.int32, device=device)
    out = torch.empty(n, dtype=torch.int32, device=device)
    for s in range(0, n, CHUNK):
        e = min(n, s + CHUNK)
        out[s:e] = torch.arange(s, e, dtype=torch.int64, device=device).to(torch.int32)  # wraps mod 2^32
    return out


def uniform_unit(n: int, seed: int, device="cpu") -> torch.Tensor:
    """float64 uniforms in [0, 1) with 53 random bits."""
    out = torch.empty(n, dtype=torch.float64, device=device)
    for s in range(0, n, CHUNK):
        c = min(CHUNK, n - s)
        out[s:s + c] = _srl(splitmix64(seed, s, c, device), 11).to(torch.float64) * (2.0 ** -53)
    return out


def zipf_u32(n: int, seed: int, s: float = 1.1, distinct: int = 1 << 20, device="cpu") -> torch.Tensor:
    """Zipf(s)-distributed keys: rank r in [1, distinct] with P(r) ~ r^-s, mapped to
    `distinct` key values drawn uniformly over [0, 2^32) (seed ^ 0x5A5A)."""
    values = uniform_u32(distinct, seed ^ 0x5A5A, device)
    w = np.arange(1, distinct + 1, dtype=np.float64) ** (-s)
    cdf = np.cumsum(w)
    cdf /= cdf[-1]
    cdf_t = torch.from_numpy(cdf).to(device)
    out = torch.empty(n, dtype=torch.int32, device=device)
    for st in range(0, n, CHUNK):
        c = min(CHUNK, n - st)
        u = _srl(splitmix64(seed, st, c, device), 11).to(torch.float64) * (2.0 ** -53)
        idx = torch.searchsorted(cdf_t, u, right=True).clamp_(max=distinct - 1)
        out[st:st + c] = values[idx]
    return out


def range_splitters(num_buckets: int, seed: int, device="cpu") -> torch.Tensor:
    """num_buckets sorted splitters: 0 followed by num_buckets-1 sorted uniform draws."""
    draws = uniform_u32(num_buckets - 1, seed, "cpu").numpy().view(np.uint32)
    spl = np.concatenate([np.zeros(1, np.uint32), np.sort(draws)])
    return torch.from_numpy(spl.view(np.int32).copy()).to(device)


def segment_sizes(count: int, seed: int, lo: int = 1024, hi: int = 4194304) -> np.ndarray:
    """Log-uniform segment sizes in [lo, hi]."""
    u = uniform_unit(count, seed).numpy()
    return np.minimum(hi, np.floor(np.exp(math.log(lo) + u * (math.log(hi + 1) - math.log(lo))))).astype(np.int64)


def as_u32(t: torch.Tensor) -> np.ndarray:
    """Host numpy uint32 view of an int32 tensor."""
    return t.detach().cpu().numpy().view(np.uint32)


def from_u32(a: np.ndarray, device="cpu") -> torch.Tensor:
    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.uint32).view(np.int32)).to(device)


def batched_spec(count: int = 4096, seed: int = 7, buckets=(2, 8, 32, 256), kinds=("delta", "range"),
                 lo: int = 1024, hi: int = 4194304):
    """Segments of the batched workload: log-uniform sizes in [lo, hi] (seed), and
    per segment a bucket count and identifier kind drawn from `buckets` / `kinds`
    (seed + 1).  Returns (sizes, bucket counts, kinds) as numpy arrays / list."""
    sizes = segment_sizes(count, seed, lo, hi)
    u = uniform_unit(2 * count, seed + 1).numpy()
    b = np.array(buckets)[np.minimum((u[:count] * len(buckets)).astype(np.int64), len(buckets) - 1)]
    k = [kinds[min(int(x * len(kinds)), len(kinds) - 1)] for x in u[count:]]
    return sizes, b, k
