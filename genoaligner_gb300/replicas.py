"""Replicas: one process per GPU, each aligning a contiguous share of a batch.

The path has no exchange step (pairs are independent), so N GPUs run N
independent replicas.  A batch is cut into N contiguous index ranges whose
predicted work (Smith-Waterman cells m*n, or WFA (d+1)^2 from a distance
estimate) is as even as contiguous ranges allow; each rank aligns its range
and rank 0 concatenates the per-rank results in request order.  No device
memory is shared and no collective touches the data path: the only
communication is the host-side gather of finished results.
"""
from __future__ import annotations

import numpy as np


def partition(weights, world: int) -> list[tuple[int, int]]:
    """Contiguous [lo, hi) ranges, one per rank, each close to sum(weights)/world.

    Cut k goes where the running weight first reaches k/world of the total, so
    no range holds more than the even share plus one item's weight.  Ranges may
    be empty (more ranks than items)."""
    w = np.asarray(weights, dtype=np.float64)
    n = int(w.shape[0])
    if world <= 0:
        raise ValueError("world must be >= 1")
    if n == 0:
        return [(0, 0)] * world
    if np.any(w < 0):
        raise ValueError("weights must be non-negative")
    cum = np.cumsum(w)
    total = float(cum[-1])
    cuts = [0]
    for k in range(1, world):
        target = total * k / world
        c = int(np.searchsorted(cum, target, side="left")) + 1 if total > 0 else (n * k) // world
        cuts.append(min(max(c, cuts[-1]), n))
    cuts.append(n)
    return [(cuts[k], cuts[k + 1]) for k in range(world)]


def sw_weights(text_len, pattern_len):
    """Predicted Smith-Waterman work of each pair: its cell count."""
    return np.asarray(text_len, np.int64) * np.asarray(pattern_len, np.int64)


def run_replicated(align_range, n: int, weights, rank: int, world: int, gather=None):
    """Run this rank's share and return the concatenated results on rank 0.

    align_range(lo, hi) aligns pairs [lo, hi) and returns a list of per-pair
    results.  gather(obj) -> list of every rank's obj (rank order) on rank 0,
    None elsewhere (torch.distributed.gather_object semantics); with world 1
    no gather is needed.  Rank 0 returns the n results in request order;
    other ranks return None."""
    ranges = partition(weights, world)
    lo, hi = ranges[rank]
    mine = align_range(lo, hi) if hi > lo else []
    if world == 1:
        return list(mine)
    parts = gather((lo, hi, list(mine)))
    if rank != 0:
        return None
    out = [None] * n
    for plo, phi, res in parts:
        if len(res) != phi - plo:
            raise RuntimeError(f"rank range [{plo}, {phi}) returned {len(res)} results")
        out[plo:phi] = res
    return out


def torch_gather(obj):
    """gather_object onto rank 0 over the default process group."""
    import torch.distributed as dist
    world = dist.get_world_size()
    dst = [None] * world if dist.get_rank() == 0 else None
    dist.gather_object(obj, dst, dst=0)
    return dst
