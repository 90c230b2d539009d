"""Recall loss and distance error of the reduced-precision search paths,
and what the learned entry gains, per workload config.

    python -m rt_entry_gb300.precision_report [--configs 1 2 3 4] [--n4 1000000]
    python -m rt_entry_gb300.precision_report --learned [--configs 1 2 4]

For each workload config (datasets.make_config; config 4 at --n4 base vectors
instead of 10M, whose exact graph would take minutes to build), this builds
the index (full-dimension PCA, kd-tree leaf 32, expand 0.2) and searches
with kd-tree entries at the config's beam, k = 10, in FP32, BF16 and FP8
(per-row scale), each without and with the exact FP32 rerank of the final
beam.  It prints one JSON line per config with
  * recall@10 against the FP64 brute-force ground truth,
  * the relative error |d - d64| / d64 of every returned distance against
    the FP64 distance of the same (query, id) pair in the searched space
    (median, p99, max), before any rerank.
"""
from __future__ import annotations

import argparse
import json
import time

import numpy as np
import torch

import rt_entry_gb300 as r
from rt_entry_gb300 import build as rbuild
from rt_entry_gb300 import datasets as ds

BEAM = {1: 64, 2: 64, 3: 64, 4: 64}


def rel_errors(base_s, q_s, ids, dists):
    """|d - d64| / d64 over all returned (query, id) pairs with d64 > 0."""
    b = torch.from_numpy(base_s).cuda()
    q = torch.from_numpy(q_s).cuda().double()
    iv = torch.from_numpy(ids.astype(np.int64)).cuda()
    ok = iv < b.shape[0]
    ivc = torch.where(ok, iv, torch.zeros_like(iv))
    exact = ((b[ivc].double() - q[:, None, :]) ** 2).sum(-1)
    d = torch.from_numpy(dists).cuda().double()
    m = ok & (exact > 0)
    e = ((d - exact).abs() / exact)[m].cpu().numpy()
    return {"median": float(np.median(e)), "p99": float(np.percentile(e, 99)), "max": float(e.max())}


def report(cfg: int, n: int | None):
    t0 = time.time()
    w = ds.make_config(cfg, n=n, gt_k=10, device="cuda")
    idx = r.Index.from_arrays(w.base, w.graph).build_pca().build_kdtree(32, 0.2)
    qp = idx.project(torch.from_numpy(w.queries).cuda())
    base_s = idx.search_base()
    q_s = qp.cpu().numpy()
    out = {"config": cfg, "n": int(w.base.shape[0]), "d": int(w.base.shape[1]),
           "nq": int(w.queries.shape[0]), "degree": int(w.graph.shape[1]), "beam": BEAM[cfg], "k": 10}
    for prec, name in ((0, "fp32"), (1, "bf16"), (2, "fp8")):
        for rerank in ((0,) if prec == 0 else (0, 1)):
            ids, dd = idx.search(w.queries, beam=BEAM[cfg], k=10, precision=prec, rerank=rerank)
            key = name + ("+rerank" if rerank else "")
            out[key] = {"recall_at_10": round(ds.recall_at(ids, w.gt, 10), 4)}
            if not rerank:
                out[key]["dist_rel_error"] = rel_errors(base_s, q_s, ids, dd)
    out["seconds"] = round(time.time() - t0, 1)
    idx.close()
    return out


def learned_gain(cfg: int, n: int | None, n_train: int = 1_000_000):
    """Recall@10 and time per 10k queries (FP32, k = 10) of kd-tree entries,
    kd-tree entries from 4 leaves, and learned entries (the model trained on
    n_train queries of the config's mixture), at beams 16, 32 and 64."""
    t0 = time.time()
    w = ds.make_config(cfg, n=n, gt_k=10, device="cuda")
    idx = r.Index.from_arrays(w.base, w.graph).build_pca().build_kdtree(32, 0.2)
    rep = idx.train_learned(ds.training_queries(cfg, n_train))
    qd = torch.from_numpy(w.queries).cuda()
    out = {"config": cfg, "n": int(w.base.shape[0]), "d": int(w.base.shape[1]),
           "nq": int(w.queries.shape[0]), "train": {k: rep[k] for k in ("classes", "last_loss", "train_ms")}}
    for L in (16, 32, 64):
        for name, kw in (("kdtree", {}), ("kdtree_4_leaves", {"max_hits": 4}),
                         ("learned", {"entry_mode": r.ENTRY_LEARNED})):
            p = r.default_params(beam=L, k=10, **kw)
            ids, _ = idx.search(qd, params=p)
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            for _ in range(5):
                idx.search(qd, params=p)
            e1.record()
            torch.cuda.synchronize()
            ms = e0.elapsed_time(e1) / 5 * 10000 / len(w.queries)
            out[f"{name}_L{L}"] = {"recall_at_10": round(ds.recall_at(ids.cpu().numpy(), w.gt, 10), 4),
                                   "ms_per_10k": round(ms, 3)}
    out["seconds"] = round(time.time() - t0, 1)
    idx.close()
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--configs", type=int, nargs="+", default=[1, 2, 3, 4])
    ap.add_argument("--n4", type=int, default=1_000_000)
    ap.add_argument("--learned", action="store_true", help="the learned-entry gain instead")
    a = ap.parse_args()
    rbuild.build()
    for cfg in a.configs:
        f = learned_gain if a.learned else report
        print(json.dumps(f(cfg, a.n4 if cfg == 4 else None)), flush=True)


if __name__ == "__main__":
    main()
