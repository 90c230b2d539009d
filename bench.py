"""Benchmark of the query path (projection -> entry -> beam search).

Workload (config 2): 1M x 128-d integer-valued base (256 flat Gaussian
clusters whose centres lie on an 8-d subspace, rounded and clipped to
0..255), 10k queries, exact degree-64 kNN graph, PCA-128, kd-tree leaves of
32 points expanded by 0.2, k = 10, recall@10 against FP64 brute force.

Two arms of this library are compared, each at its fastest (beam, search
width) whose recall@10 >= 0.95:
  plain FP32     kd-tree entries, FP32 distances (the reference's method)
  learned + BF16 MLP-proposed entries (trained on 1M queries labelled by the
                 plain search), BF16 distances, exact FP32 rerank
`value` is the learned + BF16 QPS (the headline); the plain FP32 arm is in
`plain_fp32`.  A step = one pass of the query path over the 10k queries with
the queries in HBM; L2 is flushed before every timed step; CUDA events on
the launching stream.  `e2e` = the same through rte_search with pinned host
queries and host outputs.  `roofline` = the plain FP32 search kernel alone
(algorithmic bytes from its counters / event time); `roofline_headline`
the same for the headline configuration.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

--impl reference: the reference's search logic restated on the host cores
(the oracle port, OpenMP over queries) on the same workload.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "QPS@recall10>=0.95, 1 GB300: learned+BF16 vs plain FP32; HBM GB/s % of peak"
SWEEP = ((16, 1), (32, 1), (64, 1), (64, 2), (128, 2), (128, 4), (256, 4))
RECALL_TARGET = 0.95
LEAF, EXPAND, K_TOP = 32, 0.2, 10
N_TRAIN = 1_000_000
WORKLOAD = ("config2: 1M x 128 int-valued flat-cluster mixture (256 clusters, centres on an "
            "8-d subspace), 10k queries, degree-64 exact kNN graph, PCA-128, kd-tree leaf 32, k=10")


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.p = None
        self.path = os.path.join("/tmp", f"rte_clocks_{os.getpid()}.csv")

    def __enter__(self):
        try:
            self.f = open(self.path, "w")
            self.p = subprocess.Popen(["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.Q}",
                                       "--format=csv,noheader,nounits", "-lms", "100"],
                                      stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.p = None
        return self

    def __exit__(self, *a):
        if self.p:
            self.p.terminate()
            try:
                self.p.wait(5)
            except Exception:
                self.p.kill()
            self.f.close()

    def summary(self):
        if not self.p:
            return None
        rows = []
        for line in open(self.path):
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                rows.append((float(parts[1]), float(parts[2]), parts[5:9]))
            except ValueError:
                continue
        if not rows:
            return None
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({n for _, _, fl in rows for n, v in zip(names, fl) if v.lower() == "active"})
        return {"sm_mhz": statistics.median(r[0] for r in rows), "sm_max_mhz": max(r[1] for r in rows),
                "reasons": reasons, "samples": len(rows)}


def algorithmic_bytes(cnt, d, L, R, k, elem_bytes=4, rerank=False, scale_bytes=0):
    """Sum over queries of B(q) = 4d + 4L + s*d*E + 4R*X + s*d*D + 8k (+ 4dL rerank)."""
    E, X, D = cnt[:, 0].astype(np.float64), cnt[:, 1], cnt[:, 2]
    b = 4 * d + 4 * L + (elem_bytes * d + scale_bytes) * (E + D) + 4 * R * X + 8 * k
    if rerank:
        b = b + 4 * d * L
    return float(b.sum())


def run_reference(args, w, setup_s):
    """The reference's search logic on the host cores: the oracle port (the
    reference has no CPU search; its GraphSearchKernel is restated in oracle/)."""
    import oracle
    from rt_entry_gb300 import datasets as ds
    t0 = time.time()
    x = w.base.astype(np.float64)
    mean = x.mean(0)
    xc = x - mean
    cov = xc.T @ xc / (x.shape[0] - 1)
    _, vec = np.linalg.eigh(cov)
    vec = vec[:, ::-1].copy()
    pb = (xc @ vec).astype(np.float32)
    del x, xc
    boxes, pids = oracle.kdtree_build(pb[:, :3], LEAF)
    ebox = oracle.expand_boxes(boxes, EXPAND)
    prep = time.time() - t0
    nthreads = os.cpu_count() or 1
    qp_all = ((w.queries.astype(np.float64) - mean) @ vec).astype(np.float32)
    hits_all = oracle.locate(ebox, qp_all, nthreads)
    sample = np.arange(min(2000, len(w.queries)))
    beam, width = SWEEP[-1]
    for L, W in SWEEP:
        ids, _ = oracle.search(pb, qp_all[sample], w.graph, L=L, k=K_TOP, search_width=W,
                               leaf_pids=pids, hits=hits_all[sample], n_threads=nthreads)
        if ds.recall_at(ids, w.gt[sample], K_TOP) >= RECALL_TARGET:
            beam, width = L, W
            break
    per_step = min(len(w.queries), 2000)
    times, rec = [], []
    for step in range(args.warmup + args.steps):
        s = (step * per_step) % len(w.queries)
        qs = w.queries[s:s + per_step]
        t1 = time.perf_counter()
        qpp = ((qs.astype(np.float64) - mean) @ vec).astype(np.float32)
        h = oracle.locate(ebox, qpp, nthreads)
        ids, _ = oracle.search(pb, qpp, w.graph, L=beam, k=K_TOP, search_width=width,
                               leaf_pids=pids, hits=h, n_threads=nthreads)
        t2 = time.perf_counter()
        if step >= args.warmup:
            times.append(t2 - t1)
            rec.append(ds.recall_at(ids, w.gt[s:s + per_step], K_TOP))
    qps = per_step * len(times) / sum(times)
    out = {"metric": METRIC, "impl": "reference", "value": qps, "unit": "queries/s",
           "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
           "ms_per_step": 1000 * sum(times) / len(times), "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
           "config": {"workload": WORKLOAD, "beam": beam, "search_width": width,
                      "queries_per_step": per_step, "recall_at_10": float(np.mean(rec)),
                      "setup_s": round(setup_s + prep, 1)},
           "cpu_baseline": {"value": qps, "unit": "queries/s", "cores": nthreads, "kind": "port",
                            "sample": f"{per_step} queries per step: projection (numpy FP64), "
                                      f"brute-force point location, oracle search; OpenMP over queries"},
           "e2e": {"value": qps, "unit": "queries/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out), flush=True)


def truncated_pca_bench(w, r, ds, torch, stream, flush, dev, keep=64, steps=5):
    """Search in the first `keep` PCA dims of the same base and graph, then
    (rerank 2) rerank the final pool exactly against the original 128-dim
    rows, as the reference's REORDER does on the host: FP32, kd-tree entries,
    k = 10.  Device-resident queries, L2 flushed before each step."""
    idx = r.Index.from_arrays(w.base, w.graph, device=dev.index or 0).build_pca(keep)
    idx.build_kdtree(LEAF, EXPAND)
    qd = torch.from_numpy(w.queries).to(dev)
    nq = qd.shape[0]
    ids = torch.empty((nq, K_TOP), dtype=torch.int32, device=dev)
    dd = torch.empty((nq, K_TOP), dtype=torch.float32, device=dev)
    res = []
    for L in (32, 64):
        for rr in (0, 2):
            p = r.default_params(beam=L, k=K_TOP, rerank=rr)
            idx.search(qd, params=p, stream=stream, out_ids=ids, out_dists=dd)
            torch.cuda.synchronize(dev)
            rec = ds.recall_at(ids.cpu().numpy(), w.gt, K_TOP)
            ts = []
            for _ in range(steps):
                flush.zero_()
                a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                a.record(stream)
                idx.search(qd, params=p, stream=stream, out_ids=ids, out_dists=dd)
                b.record(stream)
                torch.cuda.synchronize(dev)
                ts.append(a.elapsed_time(b))
            ms = statistics.median(ts)
            res.append({"beam": L, "rerank": rr, "recall": round(rec, 4), "ms": round(ms, 3),
                        "qps": nq / (ms / 1000.0)})
    idx.close()
    return {"search_dims": keep, "of_dims": int(w.base.shape[1]), "sweep": res,
            "path": "FP32 search in the truncated PCA space; rerank 2 = exact FP32 rerank "
                    "of the final pool against the original rows"}


def stream_bench(idx, r, ds, torch, stream, entry_mode, n_batches=2000, max_batch=8192):
    """Config 5: uneven batches (sizes floor(exp(U[0, ln 8192])), k in
    {1, 10, 100}) over the config-2 index.  Per k: parameters autotuned for
    recall@k >= 0.95 on 2000 held-out queries, then one CUDA-graph batcher
    (capacity 8192) replays the whole query path for every batch.  Latency is
    wall time per batch: pinned host queries in, host results out.
    entry_mode: learned entries (the head in the graph) or kd-tree entries."""
    mix = ds.mixture_config(2)
    pool = mix.sample(65536, ds.SEED_STREAM)
    tune_q = mix.sample(2000, ds.SEED_STREAM + 1)
    sizes, ks = ds.stream_batches(n_batches, max_batch)
    base = idx.search_base()  # search space == PCA coordinates; GT is rotation-invariant
    tune_gt = ds.ground_truth(base, idx.project(tune_q), 100)
    batchers, tuned = {}, {}
    for k in sorted(set(int(x) for x in ks)):
        p, rep = idx.autotune(tune_q, tune_gt, k=k, target_recall=RECALL_TARGET,
                              precision=r.PREC_BF16, rerank=1, entry_mode=entry_mode)
        batchers[k] = idx.batcher(max_batch, params=p)
        tuned[k] = {"beam": p.beam, "search_width": p.search_width, "bloom_words": p.bloom_words,
                    "warps_per_block": p.warps_per_block, **{kk: rep[kk] for kk in ("recall", "met_target")}}
    qh = torch.from_numpy(pool).pin_memory()
    outs = {k: (torch.empty((max_batch, k), dtype=torch.int32).pin_memory(),
                torch.empty((max_batch, k), dtype=torch.float32).pin_memory()) for k in batchers}
    for k, b in batchers.items():  # warm-up
        b.search(qh[:max_batch], out_ids=outs[k][0], out_dists=outs[k][1], stream=stream)
    lat, pos, total = [], 0, 0
    t_all = time.perf_counter()
    for n, k in zip(sizes, ks):
        n, k = int(n), int(k)
        if pos + n > len(pool):
            pos = 0
        t1 = time.perf_counter()
        batchers[k].search(qh[pos:pos + n], out_ids=outs[k][0][:n], out_dists=outs[k][1][:n],
                           stream=stream)
        lat.append(time.perf_counter() - t1)
        pos += n
        total += n
    wall = time.perf_counter() - t_all
    for b in batchers.values():
        b.close()
    lat_ms = np.array(lat) * 1000.0
    return {"batches": n_batches, "queries": total, "qps": total / wall,
            "p50_ms": float(np.percentile(lat_ms, 50)), "p99_ms": float(np.percentile(lat_ms, 99)),
            "tuned": {str(k): v for k, v in tuned.items()},
            "path": "rte_batcher (one CUDA graph per k), BF16 distances + FP32 rerank, "
                    + ("learned entries" if entry_mode == r.ENTRY_LEARNED else "kd-tree entries")}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=("ours", "reference"))
    ap.add_argument("--no-stream", action="store_true", help="skip the uneven-stream measurement")
    args = ap.parse_args()
    args.warmup = max(3, args.warmup)

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    from rt_entry_gb300 import datasets as ds
    if args.impl == "reference":
        if rank != 0:
            return
        import torch
        dev = f"cuda:{local}" if torch.cuda.is_available() else None
        t0 = time.time()
        w = ds.make_config(2, device=dev, fast_graph=False)  # no kernel of this library here
        run_reference(args, w, time.time() - t0)
        return

    import torch
    torch.cuda.set_device(local)
    dist = None
    if world > 1:  # replicas: every rank searches its own copy of the workload
        import torch.distributed as dist
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        dist.init_process_group("nccl", rank=rank, world_size=world)
    import rt_entry_gb300 as r
    from rt_entry_gb300 import build as rbuild
    rbuild.build()
    dev = torch.device(f"cuda:{local}")

    t0 = time.time()
    w = ds.make_config(2, device=str(dev))
    setup_s = time.time() - t0
    t0 = time.time()
    idx = r.Index.from_arrays(w.base, w.graph, device=local).build_pca().build_kdtree(LEAF, EXPAND)
    build_s = time.time() - t0
    t0 = time.time()
    train_rep = idx.train_learned(ds.training_queries(2, N_TRAIN))
    train_s = time.time() - t0
    nq, d = w.queries.shape
    R = w.graph.shape[1]
    qd = torch.from_numpy(w.queries).to(dev)
    stream = torch.cuda.current_stream(dev)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    out_ids = torch.empty((nq, K_TOP), dtype=torch.int32, device=dev)
    out_d = torch.empty((nq, K_TOP), dtype=torch.float32, device=dev)

    def timed(params, steps, warmup):
        for _ in range(warmup):
            idx.search(qd, params=params, stream=stream, out_ids=out_ids, out_dists=out_d)
        torch.cuda.synchronize(dev)
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
              for _ in range(steps)]
        for i in range(steps):
            flush.zero_()
            ev[i][0].record(stream)
            idx.search(qd, params=params, stream=stream, out_ids=out_ids, out_dists=out_d)
            ev[i][1].record(stream)
        torch.cuda.synchronize(dev)
        return [a.elapsed_time(b) for a, b in ev]

    def log(msg):
        print(f"[bench] {msg}", file=sys.stderr, flush=True)

    log(f"setup {setup_s:.1f}s, index {build_s:.1f}s, learned {train_s:.1f}s {train_rep}")

    def sweep(**kw):
        res = []
        for L, W in SWEEP:
            p = r.default_params(beam=L, k=K_TOP, search_width=W, **kw)
            idx.search(qd, params=p, stream=stream, out_ids=out_ids, out_dists=out_d)
            torch.cuda.synchronize(dev)
            rec = ds.recall_at(out_ids.cpu().numpy(), w.gt, K_TOP)
            ms = statistics.median(timed(p, 3, 1))
            res.append({"beam": L, "width": W, "recall": round(rec, 4), "ms": round(ms, 3)})
            log(f"{kw} {res[-1]}")
        ok = [x for x in res if x["recall"] >= RECALL_TARGET]
        best = min(ok, key=lambda x: x["ms"]) if ok else max(res, key=lambda x: x["recall"])
        return best, res

    plain_best, plain_sweep = sweep(entry_mode=r.ENTRY_KDTREE)
    head_kw = dict(entry_mode=r.ENTRY_LEARNED, precision=r.PREC_BF16, rerank=1)
    head_best, head_sweep = sweep(**head_kw)
    p_plain = r.default_params(beam=plain_best["beam"], k=K_TOP, search_width=plain_best["width"])
    p_head = r.default_params(beam=head_best["beam"], k=K_TOP, search_width=head_best["width"],
                              **head_kw)

    # ---- timed: the headline arm, with clocks sampled ----
    if dist:
        dist.barrier()
    with ClockSampler(local) as clk:
        torch.cuda.nvtx.range_push("rte_timed")  # lets a profiler select the timed region
        head_ms = timed(p_head, args.steps, args.warmup)
        torch.cuda.nvtx.range_pop()
    head_ids = out_ids.cpu().numpy()
    from rt_entry_gb300.replicas import max_over_ranks
    total_s = max_over_ranks(sum(head_ms) / 1000.0, device=dev)  # the slowest replica
    value = nq * args.steps * world / total_s
    head_recall = ds.recall_at(head_ids, w.gt, K_TOP)
    torch.cuda.nvtx.range_push("rte_timed_plain")
    plain_ms = timed(p_plain, args.steps, args.warmup)
    torch.cuda.nvtx.range_pop()
    plain_ids = out_ids.cpu().numpy()
    plain_qps = nq * len(plain_ms) / (sum(plain_ms) / 1000.0)
    plain_recall = ds.recall_at(plain_ids, w.gt, K_TOP)

    # ---- search kernels alone: rooflines ----
    hbm, hbm_kind = peaks()
    qp = idx.project(qd)
    hits = idx.locate(qp)

    # DRAM bytes (read + write) of one launch of the search kernel on this
    # workload, from the ncu captures summarised in profiles/ (files
    # search_kernel_f32_config2_beam32_nq10000.md and
    # search_kernel_bf16_learned_config2_beam16_nq10000.md).  Only a
    # configuration that was captured gets a traffic figure.
    traffic_profiled = {(0, 32): 6.216e9 + 4.6e6, (1, 16): 1.224e9 + 4.4e6}

    def kernel_roofline(params, hits_in, elem_bytes, rerank, scale_bytes=0):
        kev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
               for _ in range(args.steps)]
        for i in range(args.steps + args.warmup):
            flush.zero_()
            j = i - args.warmup
            if j >= 0:
                kev[j][0].record(stream)
            idx.search_projected(qp, hits=hits_in, params=params, stream=stream)
            if j >= 0:
                kev[j][1].record(stream)
        torch.cuda.synchronize(dev)
        kms = statistics.mean(a.elapsed_time(b) for a, b in kev)
        cnt = idx.counters(qp, hits=hits_in, params=params)
        alg = algorithmic_bytes(cnt, d, params.beam, R, K_TOP, elem_bytes, rerank, scale_bytes)
        ach = alg / (kms / 1000.0) / 1e9
        return {"bound": "hbm", "achieved": ach, "peak": hbm, "unit": "GB/s", "frac": ach / hbm,
                "traffic": traffic_profiled.get((params.precision, params.beam)),
                "kernel": "search_kernel", "kernel_ms": kms,
                "alg_bytes_per_launch": alg, "peak_kind": hbm_kind,
                "mean_dist_evals": float(cnt[:, 2].mean()), "mean_expanded": float(cnt[:, 1].mean())}

    roof_plain = kernel_roofline(p_plain, hits, 4, False)
    learned_hits = idx.learned_leaves(qp)
    roof_head = kernel_roofline(p_head, learned_hits, 2, True)
    roof_head["note"] = "includes the kd-tree locate launch of the second entry leaf"

    # ---- end to end through the public API with pinned host buffers ----
    qh = torch.from_numpy(w.queries).pin_memory()
    ih = torch.empty((nq, K_TOP), dtype=torch.int32).pin_memory()
    dh = torch.empty((nq, K_TOP), dtype=torch.float32).pin_memory()
    for _ in range(args.warmup):
        idx.search(qh, params=p_head, out_ids=ih, out_dists=dh, stream=stream)
    e2e_t = []
    for _ in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize(dev)
        t1 = time.perf_counter()
        idx.search(qh, params=p_head, out_ids=ih, out_dists=dh, stream=stream)
        e2e_t.append(time.perf_counter() - t1)
    e2e = nq * world * len(e2e_t) / sum(e2e_t)
    assert np.array_equal(ih.numpy(), head_ids)

    # ---- CPU baseline: the oracle port of the plain search on the host cores ----
    cpu = None
    if rank == 0:
        import oracle
        pb = idx.search_base()
        _, _, pids = idx.kdtree()
        qpn, hn = qp.cpu().numpy(), hits.cpu().numpy()
        nthreads = os.cpu_count() or 1
        oracle.search(pb, qpn[:64], w.graph, L=p_plain.beam, k=K_TOP, search_width=p_plain.search_width,
                      leaf_pids=pids, hits=hn[:64])
        t1 = time.perf_counter()
        oids, _ = oracle.search(pb, qpn, w.graph, L=p_plain.beam, k=K_TOP,
                                search_width=p_plain.search_width, leaf_pids=pids, hits=hn,
                                n_threads=nthreads)
        cpu_s = time.perf_counter() - t1
        cpu = {"value": nq / cpu_s, "unit": "queries/s", "cores": nthreads, "kind": "port",
               "sample": f"all {nq} queries, plain FP32 search stage (beam {p_plain.beam}, width "
                         f"{p_plain.search_width}) on the same projected queries, hits and graph; "
                         f"OpenMP over queries"}
        assert np.array_equal(oids, plain_ids), "GPU result differs from the oracle"

    stream_res = stream_kd = None
    if rank == 0 and not args.no_stream:
        stream_res = stream_bench(idx, r, ds, torch, stream, r.ENTRY_LEARNED)
        log(f"stream {stream_res}")
        stream_kd = stream_bench(idx, r, ds, torch, stream, r.ENTRY_KDTREE)
        log(f"stream (kd-tree entries) {stream_kd}")
    # kd-tree entries from several containing leaves (the reference's
    # disabled multi-hit entry), FP32: informational
    multi_res = []
    if rank == 0:
        for H in (2, 4):
            for L in (16, 32):
                p = r.default_params(beam=L, k=K_TOP, max_hits=H)
                idx.search(qd, params=p, stream=stream, out_ids=out_ids, out_dists=out_d)
                torch.cuda.synchronize(dev)
                rec = ds.recall_at(out_ids.cpu().numpy(), w.gt, K_TOP)
                ms = statistics.median(timed(p, 5, 1))
                multi_res.append({"max_hits": H, "beam": L, "recall": round(rec, 4), "ms": round(ms, 3)})
        log(f"multi-leaf {multi_res}")
    trunc_res = None
    if rank == 0:
        trunc_res = truncated_pca_bench(w, r, ds, torch, stream, flush, dev)
        log(f"truncated pca {trunc_res}")

    if rank == 0:
        out = {"metric": METRIC, "value": value, "unit": "queries/s", "n_gpus": world,
               "steps": args.steps, "warmup": args.warmup,
               "ms_per_step": 1000 * total_s / args.steps, "higher_is_better": True,
               "scaling": "weak", "vs_baseline": None, "dtype": "bf16+f32rerank", "data": "synthetic",
               "config": {"workload": WORKLOAD, "arm": "learned entry + BF16 distances + FP32 rerank",
                          "beam": p_head.beam, "search_width": p_head.search_width,
                          "recall_at_10": round(head_recall, 4), "sweep": head_sweep,
                          "parallelism": f"replicas{world}",
                          "l2": "flushed (256 MB write) before every timed step",
                          "setup_s": round(setup_s, 1), "index_build_s": round(build_s, 1),
                          "learned": {"train_s": round(train_s, 1), "n_train": N_TRAIN, **train_rep}},
               "plain_fp32": {"value": plain_qps, "unit": "queries/s", "beam": p_plain.beam,
                              "search_width": p_plain.search_width,
                              "recall_at_10": round(plain_recall, 4), "sweep": plain_sweep,
                              "speedup_of_headline": value / plain_qps},
               "stream": stream_res,
               "stream_kdtree": stream_kd,
               "truncated_pca": trunc_res,
               "multi_leaf_kdtree": multi_res or None,
               "roofline": roof_plain,
               "roofline_headline": roof_head,
               "cpu_baseline": cpu,
               "e2e": {"value": e2e, "unit": "queries/s",
                       "h2d_bytes_per_step": int(nq * d * 4),
                       "d2h_bytes_per_step": int(nq * K_TOP * 8)},
               # per timed step of the headline arm: project_rows, locate_points (side
               # stream), mlp_head_kernel, locate_in_subtree_wide, search_kernel
               "gpu_launches": 5 * args.steps,
               "clocks": clk.summary()}
        print(json.dumps(out), flush=True)
    if dist:
        dist.barrier()
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
