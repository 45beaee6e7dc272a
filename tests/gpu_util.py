"""Helpers shared by the GPU parity tests: identifiers for both sides (library
descriptor object and oracle descriptor) and device round trips."""
import numpy as np
import torch

import gpumultisplit_gb300 as gms
from gpumultisplit_gb300 import datagen

KIND_NAMES = {0: "delta", 1: "div", 2: "bits", 3: "range", 4: "mask", 5: "even_float"}


def identifiers(o, kind, B, splitter_seed=7, shift=None, param=None, lower=0, inverse_delta=None):
    """(library identifier, oracle Desc, keep-alive) for one identifier kind."""
    if kind == o.DELTA:
        return gms.delta_bucket(), o.Desc(o.DELTA, B), None
    if kind == o.DIV:
        p = param if param is not None else max(1, (1 << 32) // B + 12345)
        return gms.delta_func(p), o.Desc(o.DIV, B, param=p), None
    if kind == o.BITS:
        s = shift if shift is not None else 7
        return gms.bits_bucket(s), o.Desc(o.BITS, B, shift=s), None
    if kind == o.RANGE:
        spl = datagen.range_splitters(B, splitter_seed)
        d_spl = spl.cuda()
        return gms.range_bucket(d_spl), o.Desc(o.RANGE, B, splitters=datagen.as_u32(spl)), d_spl
    if kind == o.MASK:
        m = param if param is not None else 0x40
        return gms.mask_bucket(m), o.Desc(o.MASK, B, param=m), None
    if kind == o.EVEN_FLOAT:
        inv = inverse_delta if inverse_delta is not None else float(B) / 2**32
        return gms.even_float_bucket(lower, inv), o.Desc(o.EVEN_FLOAT, B, lower=lower, inverse_delta=inv), None
    raise ValueError(kind)


def to_dev(a: np.ndarray, pad_front: int = 0) -> torch.Tensor:
    """Device copy; with pad_front > 0 the returned view starts pad_front elements
    into its allocation (an address that is not 16-byte aligned)."""
    t = torch.zeros(a.size + pad_front, dtype=torch.int32, device="cuda")
    if a.size:
        t[pad_front:] = datagen.from_u32(a, "cuda")
    return t[pad_front:]


def host(t: torch.Tensor) -> np.ndarray:
    return datagen.as_u32(t)


def run_multisplit(keys: np.ndarray, B: int, ident, values: np.ndarray | None, misalign: int = 0,
                   want_offsets: bool = True):
    n = keys.size
    dk = to_dev(keys, misalign)
    ok = to_dev(np.zeros(n, np.uint32), misalign)
    ctx = gms.multisplit_context(B)
    if values is None:
        gms.multisplit_allocate_key_only(n, ctx)
        offs = gms.multisplit_key_only(dk, ok, n, ctx, ident, multisplit_offset=True if want_offsets else None)
        vo = None
    else:
        dv = to_dev(values, misalign)
        ov = to_dev(np.zeros(n, np.uint32), misalign)
        gms.multisplit_allocate_key_value(n, ctx)
        offs = gms.multisplit_key_value(dk, dv, ok, ov, n, ctx, ident,
                                        multisplit_offset=True if want_offsets else None)
        vo = host(ov)
    torch.cuda.synchronize()
    err = gms.read_device_error(ctx)
    return host(ok), vo, offs, err
