"""Recall loss and distance error of the reduced-precision search paths.

    python -m rt_entry_gb300.precision_report [--configs 1 2 3 4] [--n4 1000000]

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


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--configs", type=int, nargs="+", default=[1, 2, 3, 4])
    ap.add_argument("--n4", type=int, default=1_000_000)
    a = ap.parse_args()
    rbuild.build()
    for cfg in a.configs:
        print(json.dumps(report(cfg, a.n4 if cfg == 4 else None)), flush=True)


if __name__ == "__main__":
    main()
