"""Sharding one round over several GPUs (one process per GPU).

Paths are independent, so a round of N paths splits into contiguous path-index
ranges, one per rank, with no exchange while tracking. Each rank tracks its range
with ``frg_config.path_offset`` set to the range's first global index: path i of the
range then draws from random stream ``path_offset + i``, exactly as path
``path_offset + i`` of the single-GPU round does, and every task keeps its global
index (tasks outside the range get 0 paths), so its gamma is the same too.

The round's one exchange is the merge of the roots into the collection (the
reference's SortingDeletingMerging, frgsupport.cu:10-215, called once per round at
frg.cu:440): ranks gather their roots and codes to rank 0, which merges the
concatenation in rank order, which is the single-GPU round's order.
"""
from __future__ import annotations

import numpy as np


def shard_range(n: int, rank: int, world: int) -> tuple[int, int]:
    """(first, count) of rank's contiguous share of n paths; shares differ by at most 1."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("need 0 <= rank < world")
    base, extra = divmod(int(n), world)
    first = rank * base + min(rank, extra)
    return first, base + (1 if rank < extra else 0)


def shard_paths_per_task(paths_per_task, first: int, count: int) -> np.ndarray:
    """Per-task path counts of the global index range [first, first + count)."""
    ppt = np.asarray(paths_per_task, dtype=np.int64)
    starts = np.concatenate([[0], np.cumsum(ppt)])
    lo = np.clip(starts[:-1], first, first + count)
    hi = np.clip(starts[1:], first, first + count)
    return (hi - lo).astype(np.int64)


def track_shard(tracker, fpm, paths_per_task, seed: int, rank: int, world: int, want_resid: bool = True):
    """Track rank's share of a round with ``tracker`` (a Tracker); returns (first, TrackResult).
    The tracker's path_offset is restored afterwards."""
    first, count = shard_range(int(np.sum(paths_per_task)), rank, world)
    cfg = tracker.config
    old = cfg.path_offset
    cfg.path_offset = first
    tracker.set_config(cfg)
    try:
        return first, tracker.track(fpm, shard_paths_per_task(paths_per_task, first, count), seed,
                                    want_resid=want_resid)
    finally:
        cfg.path_offset = old
        tracker.set_config(cfg)


def gather_merge(collection, roots, codes, group=None):
    """Gather every rank's (roots, codes) to rank 0 and merge them there, in rank order,
    into ``collection`` (a Collection). Returns the merged codes on rank 0 (duplicates
    marked 6, in the concatenated order), None elsewhere. Uses torch.distributed
    (gloo or NCCL) object gather; the arrays travel as numpy buffers."""
    import torch.distributed as dist

    rank = dist.get_rank(group)
    world = dist.get_world_size(group)
    mine = (np.ascontiguousarray(np.asarray(roots, np.complex128).reshape(-1, 21)),
            np.ascontiguousarray(np.asarray(codes, np.int32)))
    out = [None] * world if rank == 0 else None
    dist.gather_object(mine, out, dst=0, group=group)
    if rank != 0:
        return None
    all_roots = np.concatenate([r for r, _ in out])
    all_codes = np.concatenate([c for _, c in out])
    return collection.merge(all_roots, all_codes)
