"""Multisplit of one input sharded across two CPU ranks (gloo): every rank
splits its own chunk (the oracle stands in for the per-rank GPU call), the
ranks allgather their bucket counts, and placing every rank's bucket runs at
the exchanged offsets reproduces the single-process stable multisplit."""
import os
import socket

import numpy as np
import pytest
import torch
import torch.multiprocessing as mp

WORLD = 2


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, port, n, cut, B, kind, out_dir):
    import torch.distributed as dist

    import oracle
    from gpumultisplit_gb300 import datagen, sharded

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=WORLD)
    try:
        keys = datagen.as_u32(datagen.zipf_u32(n, 9, distinct=1 << 12))
        vals = np.arange(n, dtype=np.uint32)
        spl = datagen.as_u32(datagen.range_splitters(B, 4)) if kind == oracle.RANGE else None
        d = oracle.Desc(kind, B, splitters=spl)
        lo, hi = (0, cut) if rank == 0 else (cut, n)
        ko, vo, starts = oracle.multisplit(keys[lo:hi], d, vals[lo:hi])
        counts = sharded.bucket_counts_from_offsets(starts.astype(np.int64), hi - lo)
        offsets, totals = sharded.global_bucket_offsets(counts)
        gk = torch.zeros(n, dtype=torch.int64)
        gv = torch.zeros(n, dtype=torch.int64)
        sharded.place_local_runs(torch.from_numpy(ko.astype(np.int64)), counts, offsets, gk)
        sharded.place_local_runs(torch.from_numpy(vo.astype(np.int64)), counts, offsets, gv)
        dist.all_reduce(gk)  # runs are disjoint, so the sum assembles the output
        dist.all_reduce(gv)
        if rank == 0:
            rk, rv, roffs = oracle.multisplit(keys, d, vals)
            np.save(os.path.join(out_dir, "ok.npy"), np.array([
                np.array_equal(gk.numpy().astype(np.uint32), rk),
                np.array_equal(gv.numpy().astype(np.uint32), rv),
                np.array_equal(totals.numpy(), np.diff(np.append(roffs.astype(np.int64), n))),
            ]))
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("n,cut,B,kind", [(100003, 40000, 256, 0), (50000, 50000, 32, 3), (30001, 0, 8, 0),
                                          (4097, 4097, 2, 3), (60001, 25000, 1000, 0), (40000, 10000, 12, 3)])
def test_sharded_offsets_reproduce_single_multisplit(oracle_mod, tmp_path, n, cut, B, kind):
    mp.start_processes(_worker, args=(_free_port(), n, cut, B, kind, str(tmp_path)), nprocs=WORLD,
                       start_method="spawn", join=True)
    ok = np.load(tmp_path / "ok.npy")
    assert ok.all(), ok


def test_counts_from_offsets():
    from gpumultisplit_gb300 import sharded

    assert sharded.bucket_counts_from_offsets([0, 3, 3, 7], 10).tolist() == [3, 0, 4, 3]
