"""Multi-GPU use: replicas over curve shards.

Curves are independent, so a catalogue is split into contiguous curve ranges, one per
process (one process per GPU), each rank runs the whole hot path on its own range, and
only the small per-curve results are gathered at the end (no collective on the data
path).  The reference scales out the same way with independent processes per
catalogue chunk (batch/makemocksh.py:12-26).
"""
from __future__ import annotations

import numpy as np


def shard_range(n_items: int, rank: int, world: int) -> tuple[int, int]:
    """Contiguous, balanced [start, stop) range of ``rank`` out of ``world``."""
    if world <= 0 or not 0 <= rank < world:
        raise ValueError("bad rank/world: %d/%d" % (rank, world))
    base, extra = divmod(int(n_items), world)
    start = rank * base + min(rank, extra)
    return start, start + base + (1 if rank < extra else 0)


def shard_columns(img: np.ndarray, rank: int, world: int) -> np.ndarray:
    """This rank's curves of a ``[n, nq]`` light-curve image (contiguous copy)."""
    a, b = shard_range(img.shape[1], rank, world)
    return np.ascontiguousarray(img[:, a:b])


def gather_rows(local: np.ndarray, rank: int, world: int, n_items: int, group=None):
    """Gather per-curve results (first axis = curves) onto rank 0 with
    ``torch.distributed.gather_object``; returns the concatenation on rank 0, None elsewhere."""
    import torch.distributed as dist
    parts = [None] * world if rank == 0 else None
    dist.gather_object(np.asarray(local), parts, dst=0, group=group)
    if rank != 0:
        return None
    out = np.concatenate(parts, axis=0)
    if out.shape[0] != n_items:
        raise RuntimeError("gathered %d rows, expected %d" % (out.shape[0], n_items))
    return out
