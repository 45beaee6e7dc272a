"""Multisplit of one input sharded across ranks (host-side exchange logic).

Rank r holds input chunk r (chunks in rank order = input order).  Every rank
runs the stable multisplit of its own chunk on its own GPU, which gives its B
bucket counts; the only exchange is an allgather of those B counts.  An
exclusive scan of the (bucket, rank) count matrix in bucket-major order gives
each rank the global output offset of each of its bucket runs, and placing
the runs there reproduces the single-GPU stable multisplit exactly: within a
bucket, rank order is input order.

This is the exchange a multi-GPU deployment needs; moving the runs to the
rank that owns each output range is left to the caller's transport (peer
copies or an all-to-all), since every box this library is measured on holds
one GPU.  The functions take torch tensors and a torch.distributed group, so
they run with NCCL on GPUs and with gloo on CPU ranks.
"""
from __future__ import annotations

import torch


def bucket_counts_from_offsets(bucket_starts, n: int) -> torch.Tensor:
    """Counts per bucket from a local multisplit's bucket starts (the
    reference's h_offsets: start of every bucket in the local output)."""
    starts = torch.as_tensor(bucket_starts, dtype=torch.int64).flatten()
    ends = torch.cat([starts[1:], torch.tensor([n], dtype=torch.int64)])
    return ends - starts


def global_bucket_offsets(local_counts: torch.Tensor, group=None) -> tuple[torch.Tensor, torch.Tensor]:
    """Allgathers every rank's B counts and returns (offsets, totals):
    offsets[b] = where this rank's bucket-b run starts in the global output,
    totals[b] = keys of bucket b over all ranks."""
    import torch.distributed as dist

    counts = torch.as_tensor(local_counts, dtype=torch.int64).flatten().contiguous()
    world = dist.get_world_size(group)
    rank = dist.get_rank(group)
    gathered = [torch.empty_like(counts) for _ in range(world)]
    dist.all_gather(gathered, counts, group=group)
    matrix = torch.stack(gathered, dim=1)  # [B, world], bucket-major like the per-tile count matrix
    flat = matrix.flatten()
    excl = torch.cumsum(flat, 0) - flat
    offsets = excl.view_as(matrix)[:, rank].clone()
    return offsets, matrix.sum(dim=1)


def place_local_runs(local_out: torch.Tensor, local_counts: torch.Tensor, offsets: torch.Tensor,
                     global_out: torch.Tensor) -> None:
    """Copies each bucket run of this rank's local multisplit output to its
    global position (global_out is the full-size output, or a view of it that
    this rank may write)."""
    counts = torch.as_tensor(local_counts, dtype=torch.int64).flatten()
    starts = torch.cumsum(counts, 0) - counts
    for b in torch.nonzero(counts).flatten().tolist():
        c, s, o = int(counts[b]), int(starts[b]), int(offsets[b])
        global_out[o:o + c].copy_(local_out[s:s + c])
