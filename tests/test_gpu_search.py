"""GPU parity: the CUDA query path against the oracle and the reference's
own kernel, through the C ABI.

Bars: ids bit-exact and distances bit-exact against the oracle (the kernel
and the oracle run the same FP32 operations in the same order); the
reference kernel returns ids only, so against it ids are compared; PCA and
projection within FP64 tolerances stated per test.
"""
import os
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLD = os.path.join(ROOT, "tests", "golden")
sys.path.insert(0, GOLD)
import make_search_golden as golden  # noqa: E402


def _index(base, graph, leaf=32, expand=0.2, pca=False):
    import rt_entry_gb300 as r
    idx = r.Index.from_arrays(base, graph)
    if pca:
        idx.build_pca()
    idx.build_kdtree(leaf, expand)
    return idx


def _mixture(n, nq, d, integer, seed, k=12, spread=45.0):
    rng = np.random.Generator(np.random.Philox(seed))
    cent = rng.uniform(40, 215, (k, d))
    x = cent[rng.integers(0, k, n + nq)] + spread * rng.standard_normal((n + nq, d))
    x = np.clip(x, 0, 255)
    x = np.rint(x) if integer else x
    x = x.astype(np.float32)
    return x[:n], x[n:]


@pytest.mark.parametrize("case", [c[0] for c in golden.CASES])
def test_search_matches_reference_kernel_and_oracle(lib, orc, cuda, case):
    c = golden.load_case(case)
    L = int(c["beam"])
    idx = _index(c["base"], c["graph"], int(c["leaf"]), float(c["expand_ratio"]))
    _, _, pids = idx.kdtree()
    assert np.array_equal(pids, c["leaf_pids"])
    hits = idx.locate(c["queries"])
    assert np.array_equal(hits, c["hits"])
    ids, d = idx.search_projected(c["queries"], beam=L, k=L, max_iter=int(c["max_iter"]),
                                  entry_mode=int(c["algo"]))
    oids, od = orc.search(c["base"], c["queries"], c["graph"], L=L, k=L,
                          max_iter=int(c["max_iter"]), entry_mode=int(c["algo"]),
                          leaf_pids=c["leaf_pids"], hits=c["hits"])
    assert np.array_equal(ids, oids), f"{(ids != oids).any(1).sum()} queries differ from the oracle"
    assert np.array_equal(d, od)
    if "ref_ids_scrub" in c:  # reference with its bloom filter starting empty
        assert np.array_equal(ids, c["ref_ids_scrub"]), "differs from the reference kernel"
    elif "ref_ids" in c:
        assert np.array_equal(ids, c["ref_ids"]), "differs from the reference kernel"


SWEEP = [
    # d, integer, degree, beam, width, bloom words, hashes, entry mode, max_iter
    (32, True, 32, 32, 1, 512, 3, 1, 100),
    (64, False, 64, 64, 1, 512, 3, 1, 100),
    (96, True, 32, 128, 2, 512, 3, 1, 100),
    (128, True, 64, 64, 1, 2048, 3, 1, 100),
    (128, False, 64, 128, 2, 4096, 2, 1, 60),
    (128, True, 32, 256, 4, 8192, 3, 1, 100),
    (96, False, 32, 64, 1, 512, 3, 0, 100),
    (128, True, 64, 32, 1, 32, 5, 1, 100),      # tiny filter: many false positives
    (128, False, 64, 64, 1, 512, 3, 1, 7),      # stops at max_iter
    (128, True, 32, 64, 2, 1024, 1, 0, 100),
    (128, True, 64, 16, 1, 512, 3, 1, 100),     # beam 16: half-warp pool
    (32, False, 32, 16, 1, 512, 3, 0, 100),
    (128, False, 32, 16, 2, 1024, 3, 1, 100),
    (64, True, 32, 16, 1, 32, 4, 1, 5),
    (960, False, 64, 64, 1, 512, 3, 1, 100),    # 960 dims: 30 chunks of 32 per row
    (960, False, 32, 16, 2, 1024, 3, 0, 60),
    # kernels built for any chunk count: dimensions without a specialised
    # kernel (remainders of 1, 2 and 3 chunks past the 4-chunk slabs), and a
    # specialised count whose (beam, batch) pair was not built (960, width 1
    # over degree 32)
    (160, True, 32, 64, 1, 512, 3, 1, 100),
    (256, False, 64, 32, 1, 512, 3, 1, 100),
    (416, True, 32, 128, 2, 1024, 3, 1, 100),
    (736, False, 64, 16, 1, 512, 3, 0, 100),
    (1000, False, 32, 64, 1, 512, 3, 1, 60),
    (960, True, 32, 32, 1, 512, 3, 1, 100),
    # degree-16 graphs: a 16-slot batch (width 1), two lists per batch
    # register (width 2 and 4), with 16- to 64-slot pools
    (128, True, 16, 64, 1, 512, 3, 1, 100),
    (128, False, 16, 16, 1, 512, 3, 1, 100),
    (64, True, 16, 32, 2, 1024, 3, 1, 100),
    (96, False, 16, 128, 4, 2048, 3, 0, 100),
    (320, False, 16, 32, 1, 512, 3, 1, 100),
]


@pytest.mark.parametrize("d,integer,R,L,W,bw,nh,mode,mi", SWEEP)
def test_search_matches_oracle_sweep(lib, orc, cuda, d, integer, R, L, W, bw, nh, mode, mi):
    from rt_entry_gb300 import datasets as ds
    base, q = _mixture(3000, 300, d, integer, seed=d * 1000 + L + W + bw + mode + mi)
    graph = ds.knn_graph(base, R)
    idx = _index(base, graph, 24, 0.2)
    _, _, pids = idx.kdtree()
    hits = idx.locate(q)
    kw = dict(beam=L, k=L, search_width=W, bloom_words=bw, bloom_hashes=nh, entry_mode=mode,
              max_iter=mi)
    ids, dd = idx.search_projected(q, **kw)
    oids, od, ocnt = orc.search(base, q, graph, L=L, k=L, search_width=W, bloom_words=bw,
                                bloom_hashes=nh, entry_mode=mode, max_iter=mi, leaf_pids=pids,
                                hits=hits, with_counters=True)
    assert np.array_equal(ids, oids), f"{(ids != oids).any(1).sum()} queries differ"
    assert np.array_equal(dd, od)
    cnt = idx.counters(q, **kw)
    assert np.array_equal(cnt, ocnt[:, :4])
    # run twice: bytes identical
    ids2, dd2 = idx.search_projected(q, **kw)
    assert np.array_equal(ids, ids2) and np.array_equal(dd, dd2)


# A main-loop batch with 1..8 distances below the pool's largest, pairwise
# distinct, is merged by rank; ties, NaN or more candidates take the
# reference's sort-and-merge network.  "dup" repeats every row of the base's
# second half from its first half (exact ties between candidates), "real" has
# real-valued rows (distinct distances).
MERGE_CASES = [
    # d, degree, beam, width, data
    (128, 64, 16, 1, "dup"),
    (128, 64, 32, 1, "real"),
    (128, 64, 64, 2, "dup"),
    (128, 32, 128, 1, "real"),
    (128, 16, 16, 1, "real"),   # 16-slot batch
    (64, 16, 64, 2, "dup"),
    (160, 32, 32, 1, "dup"),    # kernel built for any chunk count
    (32, 32, 256, 2, "real"),
]


@pytest.mark.parametrize("d,R,L,W,kind", MERGE_CASES)
def test_merge_by_rank_and_network_match_oracle(lib, orc, cuda, d, R, L, W, kind):
    from rt_entry_gb300 import datasets as ds
    base, q = _mixture(3000, 300, d, kind == "dup", seed=7 * d + L + W + R)
    if kind == "dup":
        rng = np.random.Generator(np.random.Philox(d + L))
        base[1500:] = base[rng.integers(0, 1500, 1500)]
    graph = ds.knn_graph(base, R)
    idx = _index(base, graph, 24, 0.2)
    _, _, pids = idx.kdtree()
    hits = idx.locate(q)
    ids, dd = idx.search_projected(q, beam=L, k=L, search_width=W)
    oids, od, ocnt = orc.search(base, q, graph, L=L, k=L, search_width=W, leaf_pids=pids, hits=hits,
                                with_counters=True)
    merges, idle, few = ocnt[:, 4].sum(), ocnt[:, 5].sum(), ocnt[:, 6].sum()
    assert few > 0 and merges - idle - few > 0, "both merge paths must occur"
    assert np.array_equal(ids, oids), f"{(ids != oids).any(1).sum()} queries differ"
    assert np.array_equal(dd, od)


# Teams: 2, 4 or 8 warps share each query's distance evaluations.  Every
# distance path (tensor-core BF16, FP32 rows in registers, rows of any chunk
# count, 960 dims, degree 16, the rerank) gives the single warp's results bit
# for bit, and the FP32 ones the oracle's.
TEAM_CASES = [
    # d, integer, degree, beam, width, precision, rerank, entry mode
    (128, True, 64, 32, 1, 0, 0, 1),
    (128, True, 64, 16, 1, 1, 1, 1),
    (96, False, 32, 64, 2, 0, 0, 0),
    (160, True, 32, 64, 1, 0, 0, 1),
    (160, False, 32, 32, 1, 1, 1, 1),
    (960, False, 64, 32, 1, 2, 1, 1),
    (128, True, 16, 32, 1, 0, 0, 1),
    (64, True, 32, 256, 4, 0, 0, 1),
]


@pytest.mark.parametrize("d,integer,R,L,W,prec,rr,mode", TEAM_CASES)
def test_teams_match_single_warp_and_oracle(lib, orc, cuda, d, integer, R, L, W, prec, rr, mode):
    import rt_entry_gb300 as r
    from rt_entry_gb300 import datasets as ds
    base, q = _mixture(2500, 120, d, integer, seed=3 * d + L + W + prec)
    graph = ds.knn_graph(base, R)
    idx = _index(base, graph, 24, 0.2)
    kw = dict(beam=L, k=L, search_width=W, precision=prec, rerank=rr, entry_mode=mode)
    ids1, d1 = idx.search_projected(q, params=r.default_params(team_warps=1, **kw))
    c1 = idx.counters(q, params=r.default_params(team_warps=1, **kw))
    for team in (2, 4, 8):
        p = r.default_params(team_warps=team, **kw)
        ids, dd = idx.search_projected(q, params=p)
        assert np.array_equal(ids, ids1) and np.array_equal(dd, d1), team
        assert np.array_equal(idx.counters(q, params=p), c1), team
    if prec == 0:
        _, _, pids = idx.kdtree()
        oids, od = orc.search(base, q, graph, L=L, k=L, search_width=W, entry_mode=mode, leaf_pids=pids,
                              hits=idx.locate(q))
        assert np.array_equal(ids1, oids) and np.array_equal(d1, od)


# Helping in the tail: one warp per query (team_warps = 1); warps left
# without a query share the distance phases of their block's searching
# warps.  A batch of 37 queries leaves idle warps in a block from the start;
# 700 gives a tail.  Integer data: bit-exact with the oracle.
@pytest.mark.parametrize("d,prec,rerank,W,R", [(128, 1, 1, 1, 64), (128, 1, 0, 2, 64), (160, 0, 0, 1, 64),
                                              (160, 1, 1, 1, 64), (128, 1, 1, 1, 16), (160, 0, 0, 2, 16)])
@pytest.mark.parametrize("nq", [37, 700])
def test_tail_helping_matches_oracle(lib, orc, cuda, d, prec, rerank, W, R, nq):
    from rt_entry_gb300 import datasets as ds
    base, q = _mixture(3000, nq, d, True, seed=d + prec + rerank + nq + R)
    graph = ds.knn_graph(base, R)
    idx = _index(base, graph, 32, 0.2)
    _, _, pids = idx.kdtree()
    hits = idx.locate(q)
    kw = dict(beam=32, k=32, search_width=W, precision=prec, rerank=rerank, team_warps=1)
    ids, dd = idx.search_projected(q, **kw)
    low = idx.search_base_lowp(prec) if prec else base
    oids, od, ocnt = orc.search(low, q, graph, L=32, k=32, search_width=W, leaf_pids=pids, hits=hits,
                                rerank_base=base if rerank else None, with_counters=True)
    assert np.array_equal(ids, oids), f"{(ids != oids).any(1).sum()} queries differ"
    assert np.array_equal(dd, od)
    assert np.array_equal(idx.counters(q, **kw), ocnt[:, :4])


# Batches larger than the resident warps (at most 4,864 on 152 SMs at these
# shapes) are taken in entry-leaf order: the results stay those of the
# oracle, which takes the queries one by one in index order.  Both single
# leaves and the first of several leaves per query order the batch.
@pytest.mark.parametrize("prec,rerank,H", [(0, 0, 1), (1, 1, 1), (0, 0, 2)])
def test_leaf_ordered_large_batches_match_oracle(lib, orc, cuda, prec, rerank, H):
    from rt_entry_gb300 import datasets as ds
    base, q = _mixture(4000, 20000, 128, True, seed=90 + prec + H)
    graph = ds.knn_graph(base, 64)
    idx = _index(base, graph, 32, 0.2)
    _, _, pids = idx.kdtree()
    kw = dict(beam=32, k=10, precision=prec, rerank=rerank, max_hits=H)
    ids, dd = idx.search_projected(q, **kw)
    low = idx.search_base_lowp(prec) if prec else base
    hits = idx.locate(q, max_hits=H)
    if H > 1:
        oids, od, ocnt = orc.search_multi(low, q, graph, L=32, k=10, hits_multi=hits, leaf_pids=pids,
                                          with_counters=True)
    else:
        oids, od, ocnt = orc.search(low, q, graph, L=32, k=10, leaf_pids=pids, hits=hits,
                                    rerank_base=base if rerank else None, with_counters=True)
    assert np.array_equal(ids, oids), f"{(ids != oids).any(1).sum()} queries differ"
    assert np.array_equal(dd, od)
    assert np.array_equal(idx.counters(q, **kw), ocnt[:, :4])


def test_automatic_teams_on_small_batches(lib, cuda):
    """team_warps = 0 spreads a small batch over up to 8 warps per query (and
    a large one over one): same results as one warp per query, for batches
    from 1 query to more than the resident warps."""
    import rt_entry_gb300 as r
    from rt_entry_gb300 import datasets as ds
    base, q = _mixture(3000, 6000, 128, True, seed=77)
    idx = _index(base, ds.knn_graph(base, 64), 24, 0.2)
    for nq in (1, 37, 600, 6000):
        for prec in (0, 1):
            kw = dict(beam=32, k=10, precision=prec, rerank=prec)
            a = idx.search_projected(q[:nq], params=r.default_params(team_warps=0, **kw))
            b = idx.search_projected(q[:nq], params=r.default_params(team_warps=1, **kw))
            assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1]), (nq, prec)


def test_team_parameter_errors(lib, cuda):
    import rt_entry_gb300 as r
    from rt_entry_gb300 import datasets as ds
    base, q = _mixture(2000, 10, 64, True, seed=5)
    idx = _index(base, ds.knn_graph(base, 32), 24, 0.2)
    for bad in (dict(team_warps=3), dict(team_warps=16), dict(team_warps=-1),
                dict(team_warps=8, warps_per_block=4)):
        with pytest.raises(r.RteError) as e:
            idx.search_projected(q, params=r.default_params(beam=32, k=10, **bad))
        assert "team_warps" in str(e.value)


def test_topk_prefix_and_host_device_io(lib, orc, cuda):
    import torch
    from rt_entry_gb300 import datasets as ds
    base, q = _mixture(2500, 200, 128, True, seed=77)
    graph = ds.knn_graph(base, 64)
    idx = _index(base, graph, 32, 0.2)
    full, fd = idx.search_projected(q, beam=64, k=64)
    top, td = idx.search_projected(q, beam=64, k=10)
    assert np.array_equal(top, full[:, :10]) and np.array_equal(td, fd[:, :10])
    # device tensors in, device tensors out; same bytes
    qt = torch.from_numpy(q).cuda()
    it, dt = idx.search_projected(qt, beam=64, k=10)
    assert it.is_cuda and np.array_equal(it.cpu().numpy(), top)
    s = torch.cuda.Stream()
    it2, _ = idx.search_projected(qt, beam=64, k=10, stream=s)
    s.synchronize()
    assert np.array_equal(it2.cpu().numpy(), top)
    # host queries and outputs: pageable outputs come back by copy,
    # page-locked ones are written by the kernels through their device address
    hi, hd = idx.search(q, beam=64, k=10)
    assert np.array_equal(hi, top) and np.array_equal(hd, td)
    pi = torch.full((q.shape[0], 10), -7, dtype=torch.int32).pin_memory()
    pd = torch.full((q.shape[0], 10), float("nan"), dtype=torch.float32).pin_memory()
    idx.search(torch.from_numpy(q).pin_memory(), beam=64, k=10, out_ids=pi, out_dists=pd, stream=s)
    assert np.array_equal(pi.numpy(), top) and np.array_equal(pd.numpy(), td)
    # only the ids page-locked, the distances pageable
    pi.fill_(-7)
    nd = np.full((q.shape[0], 10), np.nan, np.float32)
    idx.search(q, beam=64, k=10, out_ids=pi, out_dists=nd)
    assert np.array_equal(pi.numpy(), top) and np.array_equal(nd, td)


def test_pca_against_fp64_and_reference_golden(lib, cuda):
    import rt_entry_gb300 as r
    z = np.load(os.path.join(GOLD, "pca_ref.npz"))
    x = z["x"].astype(np.float32)
    g = np.zeros((x.shape[0], 32), np.int32)
    idx = r.Index.from_arrays(x, g).build_pca()
    mean, rot, ev = idx.pca()
    assert np.allclose(mean, z["mean"], rtol=0, atol=1e-4)
    assert np.allclose(ev, z["eigvals"], rtol=1e-9, atol=1e-9 * ev[0])
    ref = z["eigvecs"]
    sign = np.sign((ref * rot).sum(0))
    sep = np.minimum(np.abs(np.diff(ev, prepend=np.inf)), np.abs(np.diff(ev, append=-np.inf)))
    ok = sep > 1e-6 * ev[0]
    assert np.abs(ref[:, ok] * sign[ok] - rot[:, ok]).max() < 1e-6
    # projected base vs the reference's (Eigen FP64, rounded to float)
    pb = idx.search_base()
    refp = z["projected"] * sign[None, :]
    scale = np.abs(refp).max()
    assert np.abs(pb[:, ok] - refp[:, ok]).max() <= 1e-5 * scale
    # query projection vs FP64
    q = x[:500] + 0.5
    qp = idx.project(q)
    exact = (q.astype(np.float64) - z["mean"]) @ rot.astype(np.float64)
    assert np.abs(qp - exact).max() <= 1e-5 * np.abs(exact).max()


@pytest.mark.parametrize("d,keep,nq", [(128, 128, 10000), (960, 960, 300), (100, 100, 777),
                                        (96, 3, 500), (128, 48, 1000)])
def test_tensor_core_projection_matches_fp64(lib, cuda, d, keep, nq):
    """The projection (x - mean) V on the tensor cores (TF32, three-term
    split, FP32 accumulation): queries and the projected base within 1e-5 of
    the largest coordinate of an FP64 product of the same FP32 mean and
    rotation, for one to four column blocks and K not a multiple of 32.  A
    misaligned query buffer takes the FP32 FMA kernel, which must agree to
    the same tolerance."""
    import torch

    import rt_entry_gb300 as r
    rng = np.random.default_rng(d + keep)
    base = (rng.standard_normal((2000, d)) * 3.0 + rng.uniform(0, 50, d)).astype(np.float32)
    q = (rng.standard_normal((nq, d)) * 3.0 + rng.uniform(0, 50, d)).astype(np.float32)
    idx = r.Index.from_arrays(base, np.zeros((2000, 32), np.int32)).build_pca(keep)
    mean, rot, _ = idx.pca()
    V = rot.astype(np.float64)[:, :keep]
    exact = (q.astype(np.float64) - mean.astype(np.float64)) @ V
    tol = 1e-5 * np.abs(exact).max()
    qd = torch.from_numpy(q).cuda()
    qp = idx.project(qd).cpu().numpy()
    assert np.abs(qp - exact).max() <= tol
    flat = torch.empty(nq * d + 1, dtype=torch.float32, device="cuda")
    qm = flat[1:].view(nq, d)  # 4 bytes off the 16-byte alignment TMA needs
    qm.copy_(qd)
    qp_fma = idx.project(qm).cpu().numpy()
    assert np.abs(qp_fma - exact).max() <= tol
    pb = idx.search_base()
    pexact = (base.astype(np.float64) - mean.astype(np.float64)) @ V
    assert np.abs(pb - pexact).max() <= 1e-5 * np.abs(pexact).max()


def test_pca_keep_dims_and_kdtree_consistency(lib, orc, cuda):
    import rt_entry_gb300 as r
    from rt_entry_gb300 import datasets as ds
    base, q = _mixture(4000, 100, 96, False, seed=5)
    graph = ds.knn_graph(base, 32)
    idx = r.Index.from_arrays(base, graph).build_pca(keep_dims=64).build_kdtree(32, 0.2)
    assert idx.info.search_dim == 64
    pb = idx.search_base()
    t, e, p = idx.kdtree()
    b, pp = orc.kdtree_build(pb[:, :3], 32)
    assert np.array_equal(t, b) and np.array_equal(p, pp)
    assert np.array_equal(e, orc.expand_boxes(b, 0.2))
    qp = idx.project(q)
    assert qp.shape == (100, 64)
    ids, dd = idx.search(q, beam=64, k=64)
    oids, od = orc.search(pb, qp, graph, L=64, k=64, leaf_pids=p, hits=orc.locate(e, qp))
    assert np.array_equal(ids, oids) and np.array_equal(dd, od)


def test_locate_matches_oracle_including_faces(lib, orc, cuda):
    import rt_entry_gb300 as r
    from rt_entry_gb300 import datasets as ds
    base, _ = _mixture(5000, 1, 32, False, seed=9)
    idx = _index(base, ds.knn_graph(base, 32), 16, 0.2)
    t, e, p = idx.kdtree()
    rng = np.random.default_rng(0)
    lo, hi = e[:, :3].min(0), e[:, 3:].max(0)
    pts = np.zeros((20000, 32), np.float32)
    pts[:, :3] = rng.uniform(lo - 5, hi + 5, (20000, 3))
    # points exactly on box faces and corners
    pick = rng.integers(0, e.shape[0], 3000)
    pts[:3000, 0] = e[pick, 0]
    pts[3000:6000, 1] = e[pick, 4]
    pts[6000:9000, :3] = e[pick, 3:6]
    got = idx.locate(pts)
    want = orc.locate(e, pts)
    assert np.array_equal(got, want)
    assert (want == 0).any()  # misses fall back to leaf 0


def test_two_dimensional_space_locates_and_searches(lib, orc, cuda):
    """A search space of fewer than three dimensions: the kd-tree is built on
    the coordinates padded with zeros, and point location reads only the
    coordinates the space has (the oracle is given the padded points)."""
    import rt_entry_gb300 as r
    from rt_entry_gb300 import datasets as ds
    rng = np.random.default_rng(21)
    base = rng.uniform(0, 200, (3000, 2)).astype(np.float32)
    q = rng.uniform(-10, 210, (400, 2)).astype(np.float32)
    graph = ds.knn_graph(base, 32)
    idx = r.Index.from_arrays(base, graph).build_kdtree(32, 0.2)
    pad = lambda a: np.pad(a, ((0, 0), (0, 1)))
    t, e, p = idx.kdtree()
    b, pp = orc.kdtree_build(pad(idx.search_base()), 32)
    assert np.array_equal(t, b) and np.array_equal(p, pp)
    hits = orc.locate(e, pad(q))
    assert np.array_equal(idx.locate(q), hits)
    ids, dd = idx.search(q, beam=32, k=32)
    oids, od = orc.search(idx.search_base(), q, graph, L=32, k=32, leaf_pids=p, hits=hits)
    assert np.array_equal(ids, oids) and np.array_equal(dd, od)


@pytest.mark.parametrize("L", [64, 16])
@pytest.mark.parametrize("prec", [1, 2])
@pytest.mark.parametrize("rerank", [0, 1])
def test_low_precision_paths_match_oracle(lib, orc, cuda, prec, rerank, L):
    """BF16 (d <= 128) forms its dot products on the tensor cores, which is
    bit-exact with the oracle when every term is exact: integer-valued data.
    FP8 runs the oracle's own operations, on any data."""
    from rt_entry_gb300 import datasets as ds
    base, q = _mixture(3000, 200, 128, prec == 1, seed=31 + prec)
    graph = ds.knn_graph(base, 64)
    idx = _index(base, graph, 32, 0.2)
    _, _, pids = idx.kdtree()
    hits = idx.locate(q)
    low = idx.search_base_lowp(prec)
    if prec == 1:
        bits = base.view(np.uint32).astype(np.uint64)
        rne = ((bits + 0x7FFF + ((bits >> 16) & 1)) >> 16 << 16).astype(np.uint32)
        assert np.array_equal(low, rne.view(np.float32))
    else:
        rel = np.abs(low - base) / np.maximum(np.abs(base).max(1, keepdims=True), 1e-9)
        assert rel.max() <= 2 ** -4 + 1e-6  # E4M3: 3 mantissa bits, scale = max|x|/448
    ids, dd = idx.search_projected(q, beam=L, k=L, precision=prec, rerank=rerank)
    oids, od = orc.search(low, q, graph, L=L, k=L, leaf_pids=pids, hits=hits,
                          rerank_base=base if rerank else None)
    assert np.array_equal(ids, oids), f"{(ids != oids).any(1).sum()} queries differ"
    assert np.array_equal(dd, od)


@pytest.mark.parametrize("d,R,L,W", [(96, 32, 128, 4), (96, 32, 256, 4), (128, 64, 64, 2), (128, 64, 256, 4)])
@pytest.mark.parametrize("prec", [1, 2])
def test_low_precision_wide_batches_match_oracle(lib, orc, cuda, d, R, L, W, prec):
    """Batches of 4 and 8 registers (width 4 over degree 32, widths 2 and 4
    over degree 64) on the tensor-core BF16 and the FP8 kernels, with the
    FP32 rerank: integer data, bit-exact with the oracle."""
    from rt_entry_gb300 import datasets as ds
    base, q = _mixture(3000, 150, d, True, seed=d + R + L + W + prec)
    graph = ds.knn_graph(base, R)
    idx = _index(base, graph, 32, 0.2)
    _, _, pids = idx.kdtree()
    hits = idx.locate(q)
    low = idx.search_base_lowp(prec)
    ids, dd = idx.search_projected(q, beam=L, k=L, search_width=W, precision=prec, rerank=1)
    oids, od = orc.search(low, q, graph, L=L, k=L, search_width=W, leaf_pids=pids, hits=hits,
                          rerank_base=base)
    assert np.array_equal(ids, oids), f"{(ids != oids).any(1).sum()} queries differ"
    assert np.array_equal(dd, od)


@pytest.mark.parametrize("L,W", [(16, 1), (64, 1), (32, 4)])
@pytest.mark.parametrize("prec", [1, 2])
def test_low_precision_paths_on_degree16_graph_match_oracle(lib, orc, cuda, prec, L, W):
    """The BF16 tensor-core and FP8 paths over a degree-16 graph (a 16-slot
    batch at width 1, four lists in two batch registers at width 4), with
    the FP32 rerank: bit-exact against the oracle on the dequantised base
    (integer-valued data keeps every BF16 term exact)."""
    from rt_entry_gb300 import datasets as ds
    base, q = _mixture(3000, 200, 128, True, seed=161 + prec + L)
    graph = ds.knn_graph(base, 16)
    idx = _index(base, graph, 32, 0.2)
    _, _, pids = idx.kdtree()
    hits = idx.locate(q)
    low = idx.search_base_lowp(prec)
    ids, dd = idx.search_projected(q, beam=L, k=L, search_width=W, precision=prec, rerank=1)
    oids, od = orc.search(low, q, graph, L=L, k=L, search_width=W, leaf_pids=pids, hits=hits,
                          rerank_base=base)
    assert np.array_equal(ids, oids), f"{(ids != oids).any(1).sum()} queries differ"
    assert np.array_equal(dd, od)


@pytest.mark.parametrize("d", [128, 96])
def test_bf16_tensor_core_distances_on_real_valued_data(lib, orc, cuda, d):
    """Real-valued data: the BF16 distance is |p|^2 + |q|^2 - 2 p.q with the
    query rounded to BF16 and FP32 sums, so it differs from the oracle's
    sum of (p - q)^2 by roundings.  Bars: every returned distance within
    1e-5 of the squared-norm scale of the same formula in FP64; top-10
    agreement with the oracle >= 0.98; after the FP32 rerank, distances of
    the returned ids within FP32 rounding of FP64 and sorted; recall within
    0.01 of the FP32 search."""
    import rt_entry_gb300 as r
    from rt_entry_gb300 import datasets as ds
    base, q = _mixture(3000, 200, d, False, seed=77 + d)
    graph = ds.knn_graph(base, 64)
    idx = _index(base, graph, 32, 0.2)
    _, _, pids = idx.kdtree()
    hits = idx.locate(q)
    low = idx.search_base_lowp(1).astype(np.float64)
    qb = (r.bf16_bits(q).astype(np.uint32) << 16).view(np.float32).astype(np.float64)
    ids, dd = idx.search_projected(q, beam=64, k=64, precision=1, rerank=0)
    ref = ((low[ids] - qb[:, None, :]) ** 2).sum(-1)
    scale = (low ** 2).sum(1).max() + (qb ** 2).sum(1).max()
    assert np.abs(dd - ref).max() <= 1e-5 * scale
    oids, _ = orc.search(idx.search_base_lowp(1), q, graph, L=64, k=64, leaf_pids=pids, hits=hits)
    agree = np.mean([len(set(a[:10]) & set(b[:10])) / 10 for a, b in zip(ids, oids)])
    assert agree >= 0.98, agree
    ids2, dd2 = idx.search_projected(q, beam=64, k=64, precision=1, rerank=1)
    exact = ((base[ids2].astype(np.float64) - q[:, None, :]) ** 2).sum(-1)
    assert np.allclose(dd2, exact, rtol=1e-5)
    assert (np.diff(dd2, axis=1) >= 0).all()
    fp32_ids, _ = orc.search(base, q, graph, L=64, k=64, leaf_pids=pids, hits=hits)
    gt = ds.ground_truth(base, q, 10)
    rec_b = ds.recall_at(ids2, gt, 10)
    rec_f = ds.recall_at(fp32_ids, gt, 10)
    assert rec_b >= rec_f - 0.01, (rec_b, rec_f)


@pytest.mark.parametrize("d", [960, 200, 288])
@pytest.mark.parametrize("prec", [1, 2])
def test_high_dim_precisions_match_oracle(lib, orc, cuda, prec, d):
    """Above 128 dims the BF16 and FP8 paths run the scalar distance code
    (960: the 30-chunk kernel; 200 and 288: the kernels built for any chunk
    count), so both are bit-exact against the oracle on the dequantised
    base, before and after the FP32 rerank, on real-valued data."""
    from rt_entry_gb300 import datasets as ds
    base, q = _mixture(2500, 120, d, False, seed=d + prec)
    graph = ds.knn_graph(base, 64)
    idx = _index(base, graph, 32, 0.2)
    _, _, pids = idx.kdtree()
    hits = idx.locate(q)
    low = idx.search_base_lowp(prec)
    for rerank in (0, 1):
        ids, dd = idx.search_projected(q, beam=64, k=64, precision=prec, rerank=rerank)
        oids, od = orc.search(low, q, graph, L=64, k=64, leaf_pids=pids, hits=hits,
                              rerank_base=base if rerank else None)
        assert np.array_equal(ids, oids), (rerank, f"{(ids != oids).any(1).sum()} queries differ")
        assert np.array_equal(dd, od)


@pytest.mark.parametrize("L", [16, 64])
def test_truncated_pca_search_with_full_rerank(lib, orc, cuda, L):
    """Search in 48 of 128 PCA dims, then rerank the final pool exactly
    against the original rows (rerank 2, the reference's REORDER): bit-exact
    against the oracle's search in the projected space followed by its
    full-dimension rerank, and recall no worse than without the rerank."""
    import rt_entry_gb300 as r
    from rt_entry_gb300 import datasets as ds
    base, q = _mixture(3000, 150, 128, False, seed=55 + L)
    graph = ds.knn_graph(base, 64)
    idx = r.Index.from_arrays(base, graph).build_pca(48).build_kdtree(32, 0.2)
    assert idx.info.search_dim == 48
    qp = idx.project(q)
    _, _, pids = idx.kdtree()
    hits = idx.locate(qp)
    ids, dd = idx.search(q, beam=L, k=10, rerank=2)
    pool, _ = orc.search(idx.search_base(), qp, graph, L=L, k=L, leaf_pids=pids, hits=hits)
    oids, od = orc.rerank_full(base, q, pool, 10)
    assert np.array_equal(ids, oids), f"{(ids != oids).any(1).sum()} queries differ"
    assert np.array_equal(dd, od)
    gt = ds.ground_truth(base, q, 10)
    ids0, _ = idx.search(q, beam=L, k=10)
    assert ds.recall_at(ids, gt, 10) >= ds.recall_at(ids0, gt, 10)
    with pytest.raises(r.RteError):
        idx.search_projected(qp, beam=L, k=10, rerank=2)  # needs the original queries


@pytest.mark.parametrize("H,L", [(2, 16), (4, 64), (3, 32)])
def test_multi_leaf_entries_match_oracle(lib, orc, cuda, H, L):
    """Kd-tree entries from the first H containing leaves (the reference's
    disabled multi-hit entry): the leaves equal the oracle's H smallest
    containing indices, and the search is bit-exact against the oracle."""
    import rt_entry_gb300 as r
    from rt_entry_gb300 import datasets as ds
    base, q = _mixture(3000, 200, 128, True, seed=70 + H + L)
    graph = ds.knn_graph(base, 64)
    idx = _index(base, graph, 32, 0.2)
    _, boxes, pids = idx.kdtree()
    hm = idx.locate(q, max_hits=H)
    assert np.array_equal(hm, orc.locate_multi(boxes, q[:, :3], H))
    assert np.array_equal(hm[:, 0], idx.locate(q))
    ids, dd = idx.search_projected(q, beam=L, k=L, max_hits=H)
    oids, od = orc.search_multi(base, q, graph, L=L, k=L, hits_multi=hm, leaf_pids=pids)
    assert np.array_equal(ids, oids), f"{(ids != oids).any(1).sum()} queries differ"
    assert np.array_equal(dd, od)
    # caller-given leaves, host and device, give the same result
    ids2, _ = idx.search_projected(q, hits=hm, beam=L, k=L, max_hits=H)
    assert np.array_equal(ids2, ids)
    with pytest.raises(r.RteError):
        idx.search_projected(q, beam=L, k=L, max_hits=H, entry_mode=r.ENTRY_RANDOM)


def test_parameter_errors(lib, cuda):
    import rt_entry_gb300 as r
    from rt_entry_gb300 import datasets as ds
    base, q = _mixture(1000, 10, 32, True, seed=3)
    idx = r.Index.from_arrays(base, ds.knn_graph(base, 32))
    with pytest.raises(r.RteError) as e:
        idx.search_projected(q, beam=64, k=10)  # kd-tree entries before the kd-tree
    assert e.value.status == r.RTE_ESTATE
    idx.build_kdtree(32, 0.2)
    for kw in (dict(beam=64, k=65), dict(beam=8, k=4), dict(beam=16, k=17), dict(beam=512, k=10),
               dict(beam=64, k=10, bloom_words=1000), dict(beam=64, k=10, bloom_hashes=11),
               dict(beam=64, k=10, search_width=3), dict(beam=64, k=10, precision=7),
               dict(beam=64, k=10, max_iter=-1)):
        with pytest.raises(r.RteError) as e:
            idx.search_projected(q, **kw)
        assert e.value.status == r.RTE_EINVAL, kw
    # graphs below degree 16 have no kernel (a list must fill half a warp)
    idx8 = r.Index.from_arrays(base, ds.knn_graph(base, 8)).build_kdtree(32, 0.2)
    with pytest.raises(r.RteError) as e:
        idx8.search_projected(q, beam=64, k=10)
    assert e.value.status == r.RTE_EINVAL and "degree" in str(e.value)
    # empty batch is fine
    ids, dd = idx.search_projected(q[:0], beam=64, k=10)
    assert ids.shape == (0, 10)
    # out-of-range caller hits fall back to leaf 0 instead of reading out of bounds
    bad = np.full(len(q), 10 ** 6, np.int32)
    ids1, _ = idx.search_projected(q, hits=bad, beam=64, k=10)
    ids0, _ = idx.search_projected(q, hits=np.zeros(len(q), np.int32), beam=64, k=10)
    assert np.array_equal(ids1, ids0)


def test_save_load_roundtrip(lib, cuda, tmp_path):
    import rt_entry_gb300 as r
    from rt_entry_gb300 import datasets as ds
    base, q = _mixture(3000, 100, 64, True, seed=12)
    graph = ds.knn_graph(base, 32)
    idx = r.Index.from_arrays(base, graph).build_pca().build_kdtree(32, 0.2)
    ids, dd = idx.search(q, beam=64, k=10)
    idx.save(str(tmp_path / "ix"))
    assert (tmp_path / "ix" / "32_0.aabbs").exists() and (tmp_path / "ix" / "O.fbin").exists()
    idx2 = r.Index.load_dir(str(tmp_path / "ix"))
    ids2, dd2 = idx2.search(q, beam=64, k=10)
    assert np.array_equal(ids, ids2) and np.array_equal(dd, dd2)


def test_load_reference_data_directory(lib, orc, cuda, tmp_path):
    """An index opened from a data directory the reference's own code wrote
    (mean.fbin and O.fbin by PCA::save_mean_rotation, pca_base.fbin by
    PCA::save_result, 32_0.aabbs from its Kdtree): the search space is
    pca_base.fbin as stored, the kd-tree equals the file's leaves, and the
    search is bit-exact against the oracle on those inputs.  The same holds
    for a directory this library saved, which reopens into an index with
    identical results.  A leaf file of another base is rejected."""
    import rt_entry_gb300 as r
    sys.path.insert(0, GOLD)
    import make_refdir_golden as refdir
    d = str(tmp_path / "ref")
    os.mkdir(d)
    q, leaf = refdir.materialise(d)
    idx = r.Index.load_reference(d, os.path.join(d, "base.bvecs"), os.path.join(d, "graph.int32"),
                                 leaf_size=leaf, expand_ratio=0.2)
    info = idx.info
    assert info.has_pca and info.has_kdtree and info.degree == refdir.R
    pb = r.read_vectors(os.path.join(d, "pca_base.fbin"))
    assert np.array_equal(idx.search_base(), pb)
    tight, expanded, pids = idx.kdtree()
    raw = open(os.path.join(d, f"{leaf}_0.aabbs"), "rb").read()
    nl = int(np.frombuffer(raw[:4], np.int32)[0])
    assert nl == info.n_leaves
    assert np.array_equal(tight, np.frombuffer(raw[8:8 + 24 * nl], np.float32).reshape(nl, 6))
    assert np.array_equal(pids, np.frombuffer(raw[8 + 24 * nl:], np.int32).reshape(nl, leaf))
    mean = r.read_vectors(os.path.join(d, "mean.fbin"))[0].astype(np.float64)
    O = r.read_vectors(os.path.join(d, "O.fbin")).astype(np.float64)
    qp = idx.project(q)
    exact = (q.astype(np.float64) - mean) @ O
    assert np.abs(qp - exact).max() <= 1e-5 * np.abs(exact).max()
    graph = np.fromfile(os.path.join(d, "graph.int32"), np.int32).reshape(-1, refdir.R)
    ids, dd = idx.search(q, beam=64, k=64)
    oids, od = orc.search(pb, qp, graph, L=64, k=64, leaf_pids=pids, hits=orc.locate(expanded, qp))
    assert np.array_equal(ids, oids) and np.array_equal(dd, od)
    # a directory this library saved (the same layouts) reopens identically
    own = r.Index.from_arrays(r.read_vectors(os.path.join(d, "base.fvecs")), graph).build_pca()
    own.build_kdtree(leaf, 0.2)
    s = str(tmp_path / "own")
    own.save(s)
    again = r.Index.load_reference(s, os.path.join(s, "base.fbin"), os.path.join(s, "graph.ibin"),
                                   leaf_size=leaf, expand_ratio=0.2)
    ids1, dd1 = own.search(q, beam=64, k=10)
    ids2, dd2 = again.search(q, beam=64, k=10)
    assert np.array_equal(ids1, ids2) and np.array_equal(dd1, dd2)
    # the leaves of another base: rejected
    import shutil
    shutil.copy(os.path.join(d, f"{leaf}_0.aabbs"), os.path.join(s, f"{leaf}_0.aabbs"))
    os.remove(os.path.join(s, "pca_base.fbin"))
    with pytest.raises(r.RteError) as e:
        r.Index.load_reference(s, os.path.join(s, "base.fbin"), os.path.join(s, "graph.ibin"),
                               leaf_size=leaf, expand_ratio=0.2)
    assert e.value.status == r.RTE_EIO and "aabbs" in str(e.value)


def test_reduced_precision_copies_made_on_use_and_released(lib, cuda):
    """An index holds only its FP32 search space and the raw base until a
    BF16 or FP8 search needs more; copies made on first use, made ahead by
    rte_index_prepare, or made again after rte_index_release all give the
    same results.  Releasing the raw base turns the calls that read it into
    RTE_ESTATE and leaves the search working."""
    import rt_entry_gb300 as r
    from rt_entry_gb300 import datasets as ds
    base, q = _mixture(3000, 100, 128, True, seed=77)
    graph = ds.knn_graph(base, 32)
    idx = _index(base, graph)
    i0 = idx.info
    assert not i0.has_bf16 and not i0.has_fp8
    ids32, d32 = idx.search_projected(q, beam=64, k=10)
    assert idx.info.device_bytes == i0.device_bytes
    ids16, d16 = idx.search_projected(q, beam=64, k=10, precision=r.PREC_BF16, rerank=1)
    i1 = idx.info
    assert i1.has_bf16 and not i1.has_fp8 and i1.device_bytes > i0.device_bytes
    ahead = _index(base, graph).prepare(r.COPY_BF16 | r.COPY_FP8)
    assert ahead.info.has_bf16 and ahead.info.has_fp8
    got = ahead.search_projected(q, beam=64, k=10, precision=r.PREC_BF16, rerank=1)
    assert np.array_equal(got[0], ids16) and np.array_equal(got[1], d16)
    fp8 = ahead.search_projected(q, beam=64, k=10, precision=r.PREC_FP8, rerank=1)
    mine = idx.search_projected(q, beam=64, k=10, precision=r.PREC_FP8, rerank=1)
    assert np.array_equal(mine[0], fp8[0]) and np.array_equal(mine[1], fp8[1])
    idx.release(r.COPY_BF16 | r.COPY_FP8)
    assert not idx.info.has_bf16 and not idx.info.has_fp8
    again = idx.search_projected(q, beam=64, k=10, precision=r.PREC_BF16, rerank=1)
    assert np.array_equal(again[0], ids16) and np.array_equal(again[1], d16)
    idx.release(r.COPY_RAW)
    assert idx.info.device_bytes < i1.device_bytes
    for call in (lambda: idx.build_pca(), lambda: idx.search(q, beam=64, k=10, rerank=2)):
        with pytest.raises(r.RteError) as e:
            call()
        assert e.value.status == r.RTE_ESTATE
    ids, dd = idx.search_projected(q, beam=64, k=10)
    assert np.array_equal(ids, ids32) and np.array_equal(dd, d32)
