"""Replicas-only multi-GPU logic (rt_entry_gb300/replicas.py) on world_size 2
with the gloo backend on the CPU: query slicing, the result gather, and the
max-over-ranks time.  The search is a stand-in with the library's output
shape (ids [m, k], dists [m, k])."""
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp


def test_query_slices_cover_every_query_once():
    from rt_entry_gb300.replicas import query_slice
    for nq in (0, 1, 7, 10, 10000, 10001):
        for world in (1, 2, 3, 8):
            spans = [query_slice(nq, r, world) for r in range(world)]
            assert spans[0][0] == 0 and spans[-1][1] == nq
            assert all(a[1] == b[0] for a, b in zip(spans, spans[1:]))
            sizes = [e - s for s, e in spans]
            assert max(sizes) - min(sizes) <= 1
    with pytest.raises(ValueError):
        query_slice(10, 2, 2)


def _fake_search(q):
    # stand-in for Index.search: ids and dists that depend on each query
    k = 4
    s = q.sum(1, keepdims=True)
    return (np.arange(k)[None, :] + s.astype(np.int32)).astype(np.int32), \
        (s + np.arange(k)[None, :]).astype(np.float32)


def _worker(rank, world, port, queries, out):
    import torch.distributed as dist
    from rt_entry_gb300.replicas import max_over_ranks, search_replicated
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        ids, dists = search_replicated(_fake_search, queries, rank, world)
        t = max_over_ranks(0.25 * (rank + 1))
        out.put((rank, ids, dists, t))
    finally:
        dist.destroy_process_group()


def test_replicated_search_gathers_in_query_order_gloo():
    world = 2
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    queries = np.random.default_rng(0).integers(0, 50, (11, 3)).astype(np.float32)
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_worker, args=(r, world, port, queries, q)) for r in range(world)]
    for p in procs:
        p.start()
    res = [q.get(timeout=120) for _ in range(world)]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    want_ids, want_d = _fake_search(queries)
    for rank, ids, dists, t in res:
        assert np.array_equal(ids, want_ids) and np.array_equal(dists, want_d)
        assert t == pytest.approx(0.5)  # the slower rank's time
