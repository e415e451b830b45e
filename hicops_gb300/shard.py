"""Spectrum sharding across ranks (one process per GPU).

Spectra are independent, so a batch is cut into contiguous per-rank shards
(the reference runs its MPI ranks over the whole batch and splits the
database instead, source/core/lbe_internal.cpp:75-103; splitting the queries
needs no exchange). Each rank searches its shard against its own replica of
the index; the only communication is the final gather of per-spectrum
results to rank 0, in global spectrum order (the reference's running
spectrumID, source/core/dslim_query.cpp:828).
"""
from __future__ import annotations

import numpy as np


def shard_bounds(nspec: int, rank: int, world: int) -> tuple[int, int]:
    """Contiguous [s0, s1) of rank `rank`; sizes differ by at most one."""
    base, extra = divmod(nspec, world)
    s0 = rank * base + min(rank, extra)
    return s0, s0 + base + (1 if rank < extra else 0)


def shard(q, rank: int, world: int):
    s0, s1 = shard_bounds(q.nspec, rank, world)
    return q.slice(s0, s1)


def sharded_query(index, q, dist=None, want_hist: bool = False):
    """Search this rank's shard; rank 0 returns the results of the whole batch.

    `index` is anything with ``query(batch, want_hist) -> (results, hist)``;
    `dist` is torch.distributed (or None for a single process).
    """
    if dist is None or not dist.is_initialized() or dist.get_world_size() == 1:
        return index.query(q, want_hist=want_hist)
    rank, world = dist.get_rank(), dist.get_world_size()
    res, hist = index.query(shard(q, rank, world), want_hist=want_hist)
    parts = [None] * world if rank == 0 else None
    dist.gather_object((res, hist), parts, dst=0)
    if rank != 0:
        return None, None
    r = np.concatenate([p[0] for p in parts])
    h = np.concatenate([p[1] for p in parts]) if want_hist else None
    return r, h
