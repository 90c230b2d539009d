"""Learned entry on the GPU: tensor-core GEMM, MLP gradients against the CPU
oracle (oracle/mlp_ref.py), training, and the learned-entry search against
the search oracle."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_tensor_core_gemm_matches_fp64(lib, cuda):
    import rt_entry_gb300 as r
    rng = np.random.default_rng(0)
    # resident (K <= 256) and streamed A blocks; several column tiles per CTA
    # (two accumulators in turn) in the last two shapes
    for M, N, K in [(128, 128, 64), (100, 70, 96), (513, 257, 264), (256, 4096, 256),
                    (2000, 2048, 320), (10000, 4096, 256)]:
        a = rng.standard_normal((M, K)).astype(np.float32)
        b = rng.standard_normal((N, K)).astype(np.float32)
        ab, bb = r.bf16_bits(a), r.bf16_bits(b)
        af = (ab.astype(np.uint32) << 16).view(np.float32).astype(np.float64)
        bf = (bb.astype(np.uint32) << 16).view(np.float32).astype(np.float64)
        ref = af @ bf.T
        c = r.gemm_bf16(ab, bb)
        # exact BF16 products, FP32 accumulation: error ~ K * 2^-24 of the terms
        assert np.abs(c - ref).max() <= 1e-5 * np.abs(ref).max(), (M, N, K)


def test_tensor_core_bias_argmax_matches_fp64(lib, cuda):
    """The fused bias + row-argmax epilogue of the head's last layer: 128 x
    256 tiles for wide outputs (resident and streamed A), 128 x 128 for
    narrow ones.  The chosen column's value must be the FP64 maximum within
    the FP32 accumulation error, and equal columns must resolve to the
    first one."""
    import rt_entry_gb300 as r
    rng = np.random.default_rng(5)
    for M, N, K in [(10000, 4096, 256), (3000, 2048, 320), (700, 1030, 128), (500, 300, 64)]:
        a = rng.standard_normal((M, K)).astype(np.float32)
        b = rng.standard_normal((N, K)).astype(np.float32)
        bias = rng.standard_normal(N).astype(np.float32)
        ab, bb = r.bf16_bits(a), r.bf16_bits(b)
        af = (ab.astype(np.uint32) << 16).view(np.float32).astype(np.float64)
        bf = (bb.astype(np.uint32) << 16).view(np.float32).astype(np.float64)
        logits = af @ bf.T + bias
        cols = r.gemm_bf16_bias_argmax(ab, bb, bias)
        assert ((cols >= 0) & (cols < N)).all(), (M, N, K)
        best = logits.max(1)
        got = logits[np.arange(M), cols]
        assert (best - got).max() <= 1e-5 * np.abs(logits).max(), (M, N, K)
        assert (cols == logits.argmax(1)).mean() > 0.999, (M, N, K)
    # ties: duplicated columns of B -> the first index wins
    M, N, K = 256, 1536, 64
    a = rng.standard_normal((M, K)).astype(np.float32)
    b = rng.standard_normal((N, K)).astype(np.float32)
    b[N // 2:] = b[: N // 2]
    cols = r.gemm_bf16_bias_argmax(r.bf16_bits(a), r.bf16_bits(b), np.zeros(N, np.float32))
    assert (cols < N // 2).all()


def test_fused_head_equals_layer_by_layer(lib, cuda):
    """The learned head in one kernel (h1, h2 kept in shared memory) against
    the three layer-by-layer GEMMs: the same columns for every row, over
    shapes with partial row blocks, a batch smaller than one block, narrow
    and wide last layers, H = 64 .. 256 and inputs not a multiple of 64
    wide.  The chosen column is also the FP64 maximum of the same BF16
    network within the accumulation error of the last layer."""
    import torch
    import rt_entry_gb300 as r
    g = torch.Generator(device="cpu").manual_seed(11)
    for M, dp, H, N in [(10000, 128, 256, 4096), (3001, 96, 256, 1000), (77, 128, 128, 300),
                        (1500, 256, 64, 100), (640, 40, 192, 2304)]:
        x = torch.randn(M, dp, generator=g).mul(2).bfloat16().cuda()
        w1 = torch.randn(H, dp, generator=g).mul(dp ** -0.5).bfloat16().cuda()
        w2 = torch.randn(H, H, generator=g).mul(H ** -0.5).bfloat16().cuda()
        w3 = torch.randn(N, H, generator=g).mul(H ** -0.5).bfloat16().cuda()
        b1, b2, b3 = (torch.randn(n, generator=g).mul(0.1).cuda() for n in (H, H, N))
        fused = r.mlp_head_argmax(x, w1, b1, w2, b2, w3, b3, path=0)
        ref = r.mlp_head_argmax(x, w1, b1, w2, b2, w3, b3, path=1)
        torch.cuda.synchronize()
        assert torch.equal(fused, ref), (M, dp, H, N, int((fused != ref).sum()))
        # FP64 check of the last layer on the GEMM path's own BF16 h2
        h1 = torch.relu(x.double() @ w1.double().T + b1.double()).bfloat16().double()
        h2 = torch.relu(h1 @ w2.double().T + b2.double()).bfloat16().double()
        logits = h2 @ w3.double().T + b3.double()
        best = logits.max(1).values
        got = logits.gather(1, fused.long()[:, None])[:, 0]
        # rows whose BF16 h2 differs from the FP64-rounded one are excluded
        # by the tolerance only where rounding flips change the maximum
        frac = ((best - got) <= 1e-4 * logits.abs().max()).double().mean().item()
        assert frac > 0.99, (M, dp, H, N, frac)
    with pytest.raises(RuntimeError):  # H not a multiple of 64: the fused form refuses it
        x = torch.zeros(128, 64, dtype=torch.bfloat16, device="cuda")
        w = torch.zeros(72, 64, dtype=torch.bfloat16, device="cuda")
        w2 = torch.zeros(72, 72, dtype=torch.bfloat16, device="cuda")
        b = torch.zeros(72, device="cuda")
        r.mlp_head_argmax(x, w, b, w2, b, w2, b, path=0)


def test_mlp_gradients_match_oracle(lib, cuda):
    import rt_entry_gb300 as r
    from oracle import mlp_ref
    rng = np.random.default_rng(1)
    M, d, H, C = 256, 100, 64, 300
    X = rng.standard_normal((M, d)).astype(np.float32)
    y = rng.integers(0, C, M).astype(np.int32)
    W1 = (rng.standard_normal((H, d)) / np.sqrt(d)).astype(np.float32)
    b1 = (rng.standard_normal(H) * 0.1).astype(np.float32)
    W2 = (rng.standard_normal((H, H)) / np.sqrt(H)).astype(np.float32)
    b2 = (rng.standard_normal(H) * 0.1).astype(np.float32)
    W3 = (rng.standard_normal((C, H)) / np.sqrt(H)).astype(np.float32)
    b3 = (rng.standard_normal(C) * 0.1).astype(np.float32)
    g, loss = r.mlp_grad_check(X, y, W1, b1, W2, b2, W3, b3)
    lref, gref = mlp_ref.loss_and_grads(X, y, W1, b1, W2, b2, W3, b3, bf=True)
    assert np.allclose(loss, lref, rtol=2e-3, atol=2e-3)
    # BF16 roundings of intermediates may flip by one BF16 ulp where FP32 and
    # FP64 accumulation differ; the tolerance is a relative Frobenius norm
    for name in ("W1", "b1", "W2", "b2", "W3", "b3"):
        err = np.linalg.norm(g[name] - gref[name]) / max(np.linalg.norm(gref[name]), 1e-30)
        assert err < 1e-2, (name, err)


def test_learned_entry_trains_and_searches(lib, orc, cuda):
    import rt_entry_gb300 as r
    from rt_entry_gb300 import datasets as ds
    # one mixture (flat clusters, centres on a subspace) for base, queries
    # and training queries, at a small size
    mix = ds.mixture_config(2)
    base = mix.sample(20000, ds.SEED_BASE)
    q = mix.sample(800, ds.SEED_QUERY)
    train = mix.sample(16384, ds.SEED_TRAIN)
    graph = ds.knn_graph(base, 32)
    gt = ds.ground_truth(base, q, 10)
    idx = r.Index.from_arrays(base, graph).build_pca().build_kdtree(32, 0.2)
    rep = idx.train_learned(train, hidden=128, epochs=12, batch=4096, lr=3e-3, label_beam=64,
                            max_classes=256)
    assert 128 < rep["classes"] <= 256
    assert rep["last_loss"] < 0.6 * rep["first_loss"], rep
    qp = idx.project(q)
    learned = idx.learned_leaves(qp)
    kd = idx.locate(qp)
    assert learned.shape == kd.shape and ((learned >= 0) & (learned < idx.info.n_leaves)).all()
    # the predictions spread over the tree (labels come from every leaf)
    assert len(np.unique(learned)) > 100
    # the learned search is bit-exact with the oracle given the same two leaves
    pb = idx.search_base()
    _, _, pids = idx.kdtree()
    ids, dd = idx.search_projected(qp, beam=64, k=64, entry_mode=r.ENTRY_LEARNED)
    oids, od = orc.search(pb, qp, graph, L=64, k=64, entry_mode=2, leaf_pids=pids, hits=learned,
                          hits2=kd)
    assert np.array_equal(ids, oids), f"{(ids != oids).any(1).sum()} queries differ"
    assert np.array_equal(dd, od)
    # raw queries (the projection also writes the model's BF16 input) give
    # the same learned search as projected ones (a separate cast)
    ir, dr = idx.search(q, beam=64, k=64, entry_mode=r.ENTRY_LEARNED)
    assert np.array_equal(ir, ids) and np.array_equal(dr, dd)
    # beam 16: both whole leaves as entries
    ids, dd = idx.search_projected(qp, beam=16, k=16, entry_mode=r.ENTRY_LEARNED)
    oids, od = orc.search(pb, qp, graph, L=16, k=16, entry_mode=2, leaf_pids=pids, hits=learned,
                          hits2=kd)
    assert np.array_equal(ids, oids), f"{(ids != oids).any(1).sum()} queries differ"
    assert np.array_equal(dd, od)
    # 12,000 queries at two warps each outnumber the resident warps: the
    # batch is taken in kd-tree-leaf order, ordered on the side stream beside
    # the model, and the results are still the oracle's
    qb = mix.sample(12000, ds.SEED_QUERY + 5)
    ib, db = idx.search(qb, beam=16, k=16, entry_mode=r.ENTRY_LEARNED)
    qbp = idx.project(qb)
    oids, od = orc.search(pb, qbp, graph, L=16, k=16, entry_mode=2, leaf_pids=pids,
                          hits=idx.learned_leaves(qbp), hits2=idx.locate(qbp))
    assert np.array_equal(ib, oids), f"{(ib != oids).any(1).sum()} queries differ"
    assert np.array_equal(db, od)
    # the model's leaf alone, without the kd-tree leaf, is a usable entry
    # (a model mapped to the wrong leaves scores near zero here)
    rk, _ = idx.search(q, beam=32, k=10)
    rec_kd = ds.recall_at(rk, gt, 10)
    ro, _ = idx.search_projected(qp, hits=learned, beam=32, k=10, entry_mode=r.ENTRY_KDTREE)
    rec_o = ds.recall_at(ro, gt, 10)
    assert rec_o >= 0.85, (rec_o, rec_kd)


def _gain(idx, q, gt, beam):
    """Recall@10 and mean expanded nodes per query at one beam: kd-tree
    entries, learned entries (model leaf + kd-tree leaf), and the model's
    leaf alone as the only entry leaf."""
    import rt_entry_gb300 as r
    from rt_entry_gb300 import datasets as ds
    qp = idx.project(q)
    kd = idx.locate(qp)
    learned = idx.learned_leaves(qp)
    p_kd = r.default_params(beam=beam, k=10)
    p_l = r.default_params(beam=beam, k=10, entry_mode=r.ENTRY_LEARNED)
    out = {}
    ids, _ = idx.search_projected(qp, hits=kd, params=p_kd)
    out["rec_kd"] = ds.recall_at(ids, gt, 10)
    out["hops_kd"] = float(idx.counters(qp, hits=kd, params=p_kd)[:, 1].mean())
    ids, _ = idx.search_projected(qp, hits=learned, params=p_l)
    out["rec_l"] = ds.recall_at(ids, gt, 10)
    out["hops_l"] = float(idx.counters(qp, hits=learned, params=p_l)[:, 1].mean())
    ids, _ = idx.search_projected(qp, hits=learned, params=p_kd)
    out["rec_model_leaf"] = ds.recall_at(ids, gt, 10)
    return out, learned


def test_learned_entry_gains_over_the_kdtree_entry(lib, cuda):
    """What the trained network gains, on the config-2 mixture (flat
    clusters, integer values) at beam 16, k = 10: recall@10 rises by at least
    0.03 over kd-tree entries and the search expands fewer nodes; the model's
    leaf alone beats a random leaf and the same leaves shuffled across
    queries.  A model trained with a learning rate of 1e-9 (its weights stay
    at their random start) must fail the same gain bar, so the bar measures
    the training."""
    import rt_entry_gb300 as r
    from rt_entry_gb300 import datasets as ds
    mix = ds.mixture_config(2)
    base = mix.sample(400_000, ds.SEED_BASE)
    q = mix.sample(2000, ds.SEED_QUERY)
    train = mix.sample(262_144, ds.SEED_TRAIN)
    graph = ds.knn_graph(base, 64)
    gt = ds.ground_truth(base, q, 10)
    rng = np.random.default_rng(5)

    idx = r.Index.from_arrays(base, graph).build_pca().build_kdtree(32, 0.2)
    idx.train_learned(train, epochs=6)
    g, learned = _gain(idx, q, gt, 16)
    n_leaves = idx.info.n_leaves
    qp = idx.project(q)
    p_kd = r.default_params(beam=16, k=10)
    ids, _ = idx.search_projected(qp, hits=rng.integers(0, n_leaves, len(q)).astype(np.int32), params=p_kd)
    rec_random_leaf = ds.recall_at(ids, gt, 10)
    ids, _ = idx.search_projected(qp, hits=rng.permutation(learned), params=p_kd)
    rec_shuffled = ds.recall_at(ids, gt, 10)
    print("trained", g, "random leaf", rec_random_leaf, "shuffled", rec_shuffled)
    assert g["rec_l"] - g["rec_kd"] >= 0.03, g
    assert g["hops_l"] < g["hops_kd"], g
    assert g["rec_model_leaf"] > rec_random_leaf + 0.2, (g, rec_random_leaf)
    assert g["rec_model_leaf"] > rec_shuffled + 0.2, (g, rec_shuffled)

    # negative control: the same pipeline with an untrained model
    idx0 = r.Index.from_arrays(base, graph).build_pca().build_kdtree(32, 0.2)
    idx0.train_learned(train, epochs=1, lr=1e-9)
    g0, _ = _gain(idx0, q, gt, 16)
    print("untrained", g0)
    assert g0["rec_l"] - g0["rec_kd"] < 0.03, g0
    assert g0["rec_model_leaf"] < g["rec_model_leaf"] - 0.2, (g0, g)


def test_bounded_waits_run_out_and_the_device_stays_usable(lib, cuda):
    """Every pipeline wait of the tensor-core kernels is bounded.  With the
    limit lowered to one try_wait round the waits run out at once: the GEMM
    and the fused head return RTE_ETIMEOUT (their kernels let the copies and
    MMAs in flight finish, free their tensor memory and exit), and with the
    default restored the same calls in the same process give the right
    results again."""
    import torch

    import rt_entry_gb300 as r
    rng = np.random.default_rng(9)
    a = r.bf16_bits(rng.standard_normal((1024, 256)).astype(np.float32))
    b = r.bf16_bits(rng.standard_normal((512, 256)).astype(np.float32))
    want = r.gemm_bf16(a, b)
    M, dp, H, N = 512, 128, 128, 1024

    def dev_bf16(shape):
        return torch.from_numpy(r.bf16_bits(rng.standard_normal(shape).astype(np.float32) * 0.1)
                                .view(np.int16)).cuda()

    x, w1, w2, w3 = dev_bf16((M, dp)), dev_bf16((H, dp)), dev_bf16((H, H)), dev_bf16((N, H))
    b1, b2, b3 = (torch.zeros(n, dtype=torch.float32, device="cuda") for n in (H, H, N))
    cols_want = r.mlp_head_argmax(x, w1, b1, w2, b2, w3, b3)
    torch.cuda.synchronize()
    lib.rte_set_wait_limit(1)
    try:
        with pytest.raises(r.RteError) as e:
            r.gemm_bf16(a, b)
        assert e.value.status == r.RTE_ETIMEOUT, e.value
        with pytest.raises(r.RteError) as e:
            r.mlp_head_argmax(x, w1, b1, w2, b2, w3, b3)
            torch.cuda.synchronize()
        assert e.value.status == r.RTE_ETIMEOUT, e.value
    finally:
        lib.rte_set_wait_limit(0)
    torch.cuda.synchronize()
    assert np.array_equal(r.gemm_bf16(a, b), want)
    cols = r.mlp_head_argmax(x, w1, b1, w2, b2, w3, b3)
    assert torch.equal(cols, cols_want)
