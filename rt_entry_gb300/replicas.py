"""Multi-GPU query serving by replicas.

Queries are independent (the reference launches one block per query,
graph.cu:320), so N GPUs serve a batch as N replicas: every rank holds a full
index on its own GPU, searches a contiguous slice of the queries, and the
[nq_i x k] results are gathered.  That gather is the only exchange; there is
no collective on the data path.

The functions take a torch.distributed process group that is already
initialised (NCCL on GPUs; gloo works for the host-side logic) and a search
callable, so they serve any of the library's search entry points.
"""
from __future__ import annotations

from typing import Callable, Tuple

import numpy as np


def query_slice(nq: int, rank: int, world: int) -> Tuple[int, int]:
    """[start, end) of rank's contiguous share of nq queries (sizes differ by
    at most one, lower ranks take the extra)."""
    if world <= 0 or not 0 <= rank < world:
        raise ValueError("rank must be in [0, world)")
    base, extra = divmod(nq, world)
    start = rank * base + min(rank, extra)
    return start, start + base + (1 if rank < extra else 0)


def search_replicated(search: Callable[[np.ndarray], Tuple[np.ndarray, np.ndarray]],
                      queries: np.ndarray, rank: int, world: int, group=None):
    """Every rank searches its slice of `queries` with `search` (host arrays
    in, host (ids [m, k], dists [m, k]) out); returns the gathered results of
    all queries, in query order, on every rank."""
    import torch
    import torch.distributed as dist
    s, e = query_slice(len(queries), rank, world)
    ids, dists = search(np.ascontiguousarray(queries[s:e]))
    ids = np.asarray(ids, np.int32)
    dists = np.asarray(dists, np.float32)
    if world == 1:
        return ids, dists
    parts = [None] * world
    dist.all_gather_object(parts, (s, ids, dists), group=group)
    parts.sort(key=lambda p: p[0])
    return (np.concatenate([p[1] for p in parts]), np.concatenate([p[2] for p in parts]))


def max_over_ranks(seconds: float, device=None, group=None) -> float:
    """The slowest rank's time: what a replicated batch costs."""
    import torch
    import torch.distributed as dist
    if not dist.is_available() or not dist.is_initialized() or dist.get_world_size(group) == 1:
        return seconds
    t = torch.tensor([seconds], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX, group=group)
    return float(t.item())
