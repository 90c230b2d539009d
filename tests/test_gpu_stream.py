"""Uneven query streams: CUDA-graph replay of the query path (rte_batcher)
and the parameter autotuner."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _index(n=8000, nq=1500, seed=41):
    import rt_entry_gb300 as r
    from rt_entry_gb300 import datasets as ds
    mix = ds.mixture_config(2)
    base = mix.sample(n, seed)
    q = mix.sample(nq, seed + 1)
    graph = ds.knn_graph(base, 64)
    idx = r.Index.from_arrays(base, graph).build_pca().build_kdtree(32, 0.2)
    return idx, base, q


@pytest.mark.parametrize("prec", [0, 1])
def test_batcher_equals_direct_search_for_every_batch_size(lib, cuda, prec):
    import torch

    import rt_entry_gb300 as r
    idx, base, q = _index()
    p = r.default_params(beam=64, k=10, precision=prec, rerank=int(prec > 0))
    want, wd = idx.search(q, params=p)
    b = idx.batcher(1024, params=p)
    assert b.k == 10
    qt = torch.from_numpy(q).cuda()
    for s, e in [(0, 1), (1, 3), (3, 131), (131, 1024), (1024, 1500), (0, 7)]:
        ids, dd = b.search(q[s:e])                      # host in, host out
        assert np.array_equal(ids, want[s:e]) and np.array_equal(dd, wd[s:e]), (s, e)
        ti, td = b.search(qt[s:e])                      # device in, device out
        assert np.array_equal(ti.cpu().numpy(), want[s:e]), (s, e)
    with pytest.raises(r.RteError):
        b.search(q[:1025])
    b.close()


def test_batcher_teams_follow_the_live_batch_size(lib, cuda):
    """The replayed search picks its team size on the device from the live
    batch: up to 8 warps per query for a small batch, one (a team of one)
    when the batch fills the resident warps.  Every size equals the direct
    search."""
    import rt_entry_gb300 as r
    idx, base, q = _index(nq=6000, seed=43)
    p = r.default_params(beam=32, k=10)
    want, wd = idx.search(q, params=r.default_params(beam=32, k=10, team_warps=1))
    b = idx.batcher(6000, params=p)
    for s, e in [(0, 6000), (0, 100), (100, 3100), (3100, 3101)]:
        ids, dd = b.search(q[s:e])
        assert np.array_equal(ids, want[s:e]) and np.array_equal(dd, wd[s:e]), (s, e)
    b.close()


def test_learned_batcher_equals_direct_search(lib, cuda):
    """Learned entries through the CUDA graph (projection with the head's
    input, fused head, subtree location, kd-tree location on a parallel
    branch, search) against rte_search's learned path, batch by batch: the
    head's tile split and every kernel read the live batch size from device
    memory."""
    import torch

    import rt_entry_gb300 as r
    from rt_entry_gb300 import datasets as ds
    idx, base, q = _index()
    idx.train_learned(ds.mixture_config(2).sample(20000, 77))
    for beam, prec in [(16, 1), (32, 0)]:
        p = r.default_params(beam=beam, k=10, precision=prec, rerank=int(prec > 0),
                             entry_mode=r.ENTRY_LEARNED)
        b = idx.batcher(1024, params=p)
        qt = torch.from_numpy(q).cuda()
        for s, e in [(0, 1), (1, 3), (3, 131), (131, 1024), (1024, 1500), (0, 7)]:
            want, wd = idx.search(q[s:e], params=p)
            ids, dd = b.search(q[s:e])
            assert np.array_equal(ids, want) and np.array_equal(dd, wd), (beam, s, e)
            ti, _ = b.search(qt[s:e])
            assert np.array_equal(ti.cpu().numpy(), want), (beam, s, e)
        b.close()


def test_large_batches_drop_the_two_warp_floor(lib, cuda):
    """FP32 rows with small pools get two warps per query only while a batch
    is at most three times the resident warps (4,864 on 152 SMs): 16,000
    queries run one warp per query, chosen on the host by rte_search and on
    the device by the batcher's graph, with the results of one warp per
    query; a 4,000-query batch through the same graph keeps the floor."""
    import rt_entry_gb300 as r
    idx, base, q = _index(nq=16000, seed=49)
    want, wd = idx.search(q, params=r.default_params(beam=16, k=10, team_warps=1))
    got, gd = idx.search(q, params=r.default_params(beam=16, k=10))
    assert np.array_equal(got, want) and np.array_equal(gd, wd)
    b = idx.batcher(16000, params=r.default_params(beam=16, k=10))
    for s, e in [(0, 16000), (0, 4000)]:
        ids, dd = b.search(q[s:e])
        assert np.array_equal(ids, want[s:e]) and np.array_equal(dd, wd[s:e]), (s, e)
    b.close()


def test_batchers_take_large_batches_in_leaf_order(lib, cuda):
    """A live batch of more queries than the resident warps (at most 4,864 on
    152 SMs) runs the graph's sort kernel and takes its queries in entry-leaf
    order, by the kd-tree leaf or, with learned entries, by the kd-tree leaf
    computed beside the model; a small batch through the same graph skips
    the order.  Every batch equals the direct search, which orders large
    batches the same way and is checked against the oracle."""
    import rt_entry_gb300 as r
    from rt_entry_gb300 import datasets as ds
    idx, base, q = _index(nq=12000, seed=47)
    idx.train_learned(ds.mixture_config(2).sample(20000, 79))
    for mode in (r.ENTRY_KDTREE, r.ENTRY_LEARNED):
        p = r.default_params(beam=16, k=10, precision=r.PREC_BF16, rerank=1, entry_mode=mode)
        b = idx.batcher(12000, params=p)
        for s, e in [(0, 12000), (0, 50), (50, 9050)]:
            want, wd = idx.search(q[s:e], params=p)
            ids, dd = b.search(q[s:e])
            assert np.array_equal(ids, want) and np.array_equal(dd, wd), (mode, s, e)
        b.close()


def test_autotune_meets_the_recall_target(lib, cuda):
    import rt_entry_gb300 as r
    from rt_entry_gb300 import datasets as ds
    idx, base, q = _index()
    gt = ds.ground_truth(base, q[:600], 10)
    p, rep = idx.autotune(q[:600], gt, k=10, target_recall=0.9)
    assert rep["evaluated"] >= 10
    assert rep["met_target"] == 1 and rep["recall"] >= 0.9
    ids, _ = idx.search(q[:600], params=p)
    assert ds.recall_at(ids, gt, 10) == pytest.approx(rep["recall"], abs=1e-6)
    assert p.beam in (16, 32, 64, 128, 256) and p.bloom_words in (512, 2048, 8192)
