"""Synthetic workloads, exact kNN graphs and FP64 ground truth.

The reference measures on SIFT/DEEP/GIST/COCO files that are not available
here; seeded synthetic data with their shapes and value ranges stands in.
Every generator uses numpy's counter-based Philox bit generator with fixed
seeds (base 1001, queries 2002, training queries 3003, stream 4004).

Graphs: degree-R exact kNN of every base vector (itself excluded), ordered by
(distance, id).  Ground truth: FP64 brute force, ordered by (distance, id).
Both run on a CUDA device through torch when one is present (plumbing for
fixtures, not the measured path) and in numpy otherwise (small sizes).
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

SEED_BASE, SEED_QUERY, SEED_TRAIN, SEED_STREAM = 1001, 2002, 3003, 4004


def _rng(seed):
    return np.random.Generator(np.random.Philox(seed))


@dataclass
class Mixture:
    """Isotropic Gaussian mixture: equal weights, per-cluster centres."""
    centers: np.ndarray
    sigma: float
    post: str = "none"          # "none" | "round_clip255" | "unit" | "minmax"
    lo: np.ndarray | None = field(default=None)
    hi: np.ndarray | None = field(default=None)

    def sample(self, n: int, seed: int, chunk: int = 1 << 18) -> np.ndarray:
        rng = _rng(seed)
        k, d = self.centers.shape
        out = np.empty((n, d), np.float32)
        for s in range(0, n, chunk):
            e = min(n, s + chunk)
            lab = rng.integers(0, k, e - s)
            x = self.centers[lab] + np.float32(self.sigma) * rng.standard_normal((e - s, d), np.float32)
            out[s:e] = self._post(x)
        return out

    def _post(self, x):
        if self.post == "round_clip255":
            return np.rint(np.clip(x, 0, 255)).astype(np.float32)
        if self.post == "unit":
            nrm = np.linalg.norm(x, axis=1, keepdims=True)
            return (x / np.maximum(nrm, 1e-12)).astype(np.float32)
        if self.post == "minmax":
            return ((x - self.lo) / (self.hi - self.lo)).astype(np.float32)
        return x.astype(np.float32)


@dataclass
class SubspaceMixture:
    """Gaussian mixture whose clusters are flat: cluster k is centre_k +
    bases_k z + noise with z ~ N(0, s^2 I_rank); the centres themselves lie on
    a low-dimensional subspace, so neighbouring clusters overlap and the kNN
    graph stays connected (a low intrinsic dimension, as SIFT-like data has)."""
    centers: np.ndarray   # [K, d]
    bases: np.ndarray     # [K, d, rank], orthonormal columns
    s: float
    noise: float
    post: str = "round_clip255"

    def sample(self, n: int, seed: int, chunk: int = 1 << 17) -> np.ndarray:
        rng = _rng(seed)
        K, d = self.centers.shape
        rank = self.bases.shape[2]
        out = np.empty((n, d), np.float32)
        for s0 in range(0, n, chunk):
            e = min(n, s0 + chunk)
            m = e - s0
            lab = rng.integers(0, K, m)
            z = rng.standard_normal((m, rank), np.float32) * np.float32(self.s)
            x = self.centers[lab] + np.einsum("mdr,mr->md", self.bases[lab], z)
            x += np.float32(self.noise) * rng.standard_normal((m, d), np.float32)
            out[s0:e] = np.rint(np.clip(x, 0, 255)) if self.post == "round_clip255" else x
        return out


@dataclass
class Workload:
    name: str
    base: np.ndarray
    queries: np.ndarray
    degree: int
    leaf_size: int = 32
    expand_ratio: float = 0.2
    k: int = 10
    beam: int = 64
    mixture: Mixture | None = None
    graph: np.ndarray | None = None
    gt: np.ndarray | None = None


def mixture_config(cfg: int, d: int | None = None) -> Mixture:
    """Mixture of configuration `cfg` (1..4)."""
    rng = _rng(SEED_BASE + 17 * cfg)
    if cfg == 1:   # 64 components, centres U[0,100]^d, sigma 5
        d = d or 128
        return Mixture(rng.uniform(0, 100, (64, d)).astype(np.float32), 5.0)
    if cfg == 2:   # 256 flat clusters, integer values 0..255 (SIFT-like bvecs)
        d = d or 128
        K, cdim, rank = 256, 8, 16
        B = np.linalg.qr(rng.standard_normal((d, cdim)))[0]
        cent = 128.0 + (rng.standard_normal((K, cdim)) * 50.0) @ B.T
        bases = np.stack([np.linalg.qr(rng.standard_normal((d, rank)))[0] for _ in range(K)])
        return SubspaceMixture(cent.astype(np.float32), bases.astype(np.float32), 25.0, 6.0)
    if cfg == 3:   # 128 clusters, N(0,1) per dim around N(0,1) centres, min-max to [0,1]
        d = d or 960
        return Mixture(rng.standard_normal((128, d), np.float32), 1.0, "minmax")
    if cfg == 4:   # 1024 clusters on the unit sphere (angular, DEEP-like)
        d = d or 96
        return Mixture(rng.standard_normal((1024, d), np.float32), 0.35, "unit")
    raise ValueError(cfg)


def make_config(cfg: int, n: int | None = None, nq: int | None = None, d: int | None = None,
                with_graph: bool = True, with_gt: bool = True, gt_k: int = 100,
                device: str | None = None, fast_graph: bool = True) -> Workload:
    """Config 1..4 at its published size (or the given n / nq / d).  With
    fast_graph the kNN graph comes from this library's GPU builder (the same
    exact graph as knn_graph)."""
    sizes = {1: (100_000, 10_000, 32), 2: (1_000_000, 10_000, 64), 3: (1_000_000, 1_000, 64),
             4: (10_000_000, 10_000, 32)}
    n0, nq0, R = sizes[cfg]
    n = n or n0
    nq = nq or nq0
    mix = mixture_config(cfg, d)
    if mix.post == "minmax":
        raw = Mixture(mix.centers, mix.sigma).sample(n, SEED_BASE)
        mix.lo = raw.min(axis=0)
        mix.hi = np.maximum(raw.max(axis=0), mix.lo + 1e-6)
        base = mix._post(raw)
        q = mix._post(Mixture(mix.centers, mix.sigma).sample(nq, SEED_QUERY))
    else:
        base = mix.sample(n, SEED_BASE)
        q = mix.sample(nq, SEED_QUERY)
    w = Workload(f"config{cfg}", base, q, R, mixture=mix)
    if with_graph:
        w.graph = (knn_graph_fast if fast_graph else knn_graph)(base, R, device=device)
    if with_gt:
        w.gt = ground_truth(base, q, min(gt_k, n), device=device)
    return w


def training_queries(cfg: int, n: int, d: int | None = None) -> np.ndarray:
    """Queries for training the learned entry: the config's mixture, seed 3003."""
    mix = mixture_config(cfg, d)
    if getattr(mix, "post", None) == "minmax":
        raise ValueError("training queries are defined for configs 1, 2 and 4")
    return mix.sample(n, SEED_TRAIN)


def _torch_device(device):
    try:
        import torch
    except ImportError:
        return None, None
    if device is None:
        device = "cuda" if torch.cuda.is_available() else None
    if device is None:
        return torch, None
    return torch, torch.device(device)


def _sort_by_dist_then_id(d, i):
    """Rows of (dist, id) candidates -> lexicographic order (numpy)."""
    o = np.lexsort((i, d), axis=-1)
    return np.take_along_axis(d, o, -1), np.take_along_axis(i, o, -1)


def knn_graph_fast(base: np.ndarray, R: int, device: str | None = None) -> np.ndarray:
    """The same exact graph as knn_graph, built by this library's GPU builder
    (rte_knn_graph) when a CUDA device is given, else by knn_graph."""
    torch, dev = _torch_device(device)
    if dev is None or dev.type != "cuda":
        return knn_graph(base, R, device=device)
    from rt_entry_gb300 import knn_graph as rte_knn_graph
    return np.asarray(rte_knn_graph(np.ascontiguousarray(base, np.float32), R,
                                    device=dev.index or 0))


def _exact_row(base, i, cols, R):
    """Row i's R nearest of the candidate columns by exact FP64 (distance, id),
    self excluded."""
    cols = cols[cols != i]
    dd = ((base[cols].astype(np.float64) - base[i].astype(np.float64)) ** 2).sum(-1)
    o = np.lexsort((cols, dd))
    return cols[o[:R]]


def _boundary_rows(D, kth, tol, kk):
    """Rows (of a block of approximate distances D) where more than kk
    columns lie within 2*tol of the kk-th smallest: ties or near-ties that
    cross the candidate cut, which those rows settle over every such column.
    Elsewhere every column whose exact distance can reach the R-th (R <= kk)
    is among the kk kept: its approximate distance is at most the R-th's
    approximate distance plus 2*tol."""
    return np.nonzero((D <= (kth + 2 * tol)[:, None]).sum(1) > kk)[0]


def knn_graph(base: np.ndarray, R: int, device: str | None = None, chunk: int = 4096) -> np.ndarray:
    """Degree-R kNN graph (self excluded), rows ordered by (FP64 dist, id).
    Candidates come from approximate distances |x|^2 + |y|^2 - 2 x.y, then
    an FP64 rerank.  On the host (FP64) the result is exact: rows whose
    candidate cut falls within the FP64 error bound of other columns are
    redone over all of them.  On a device (FP32) the candidates are the
    R + 8 smallest, and only runs of exactly equal FP32 distances at the cut
    (duplicated rows) are widened; this library's rte_knn_graph is the
    certified exact builder on the GPU."""
    n, d = base.shape
    if n <= R:
        raise ValueError("need more than R base vectors")
    torch, dev = _torch_device(device)
    extra = 8
    kk = R + extra
    out = np.empty((n, R), np.int32)
    if dev is not None:
        prev = torch.backends.cuda.matmul.allow_tf32
        torch.backends.cuda.matmul.allow_tf32 = False
        try:
            X = torch.from_numpy(base).to(dev)
            nrm64 = (X.double() ** 2).sum(1)
            nrm_d = nrm64.float()
            for s in range(0, n, chunk):
                e = min(n, s + chunk)
                D = nrm_d[s:e, None] + nrm_d[None, :] - 2.0 * (X[s:e] @ X.T)
                D[torch.arange(e - s, device=dev), torch.arange(s, e, device=dev)] = float("inf")
                dv, iv = torch.topk(D, kk, dim=1, largest=False)
                # exact FP64 distances of the candidates, then (dist, id) order
                cand = X[iv.reshape(-1)].reshape(e - s, kk, -1).double()
                dd = ((cand - X[s:e, None, :].double()) ** 2).sum(-1)
                dd_np, iv_np = _sort_by_dist_then_id(dd.cpu().numpy(), iv.cpu().numpy())
                out[s:e] = iv_np[:, :R]
                # rows whose cut falls inside a run of equal FP32 distances
                # (duplicated rows): redone over the whole run.  Near-ties
                # are left to the R + 8 candidates, as a bound of the FP32
                # error would pull in most rows of a dense base.
                thr = dv[:, -1]
                cnt = (D <= thr[:, None]).sum(1)
                over = (cnt > kk).nonzero().flatten()
                if over.numel():  # redo those rows over every column below the cut
                    kb = int(cnt[over].max())
                    step = max(1, min(256, (1 << 30) // (kb * d * 8)))
                    for o0 in range(0, over.numel(), step):
                        sub = over[o0:o0 + step]
                        _, ivb = torch.topk(D[sub], kb, dim=1, largest=False)
                        xb = X[ivb.reshape(-1)].reshape(sub.numel(), kb, -1).double()
                        ddb = ((xb - X[s + sub, None, :].double()) ** 2).sum(-1)
                        _, ivb = _gpu_sort_dist_id(ddb, ivb)
                        out[(s + sub).cpu().numpy()] = ivb[:, :R].cpu().numpy()
        finally:
            torch.backends.cuda.matmul.allow_tf32 = prev
        return out
    X64 = base.astype(np.float64)
    nrm = (X64 ** 2).sum(1)
    nmax = float(nrm.max())
    for s in range(0, n, 1024):
        e = min(n, s + 1024)
        D = nrm[s:e, None] + nrm[None, :] - 2.0 * (X64[s:e] @ X64.T)
        D[np.arange(e - s), np.arange(s, e)] = np.inf
        iv = np.argpartition(D, kk, axis=1)[:, :kk]
        cand = X64[iv]
        dd = ((cand - X64[s:e, None, :]) ** 2).sum(-1)
        _, iv2 = _sort_by_dist_then_id(dd, iv)
        out[s:e] = iv2[:, :R]
        # FP64 products and sums: error below (d + 2) 2^-50 (|x|^2 + |y|^2)
        tol = (d + 2) * 2.0 ** -50 * (nrm[s:e] + nmax)
        kth = np.take_along_axis(D, iv, 1).max(1)
        for r in _boundary_rows(D, kth, tol, kk):
            cols = np.nonzero(D[r] <= kth[r] + 2 * tol[r])[0]
            out[s + r] = _exact_row(base, s + r, cols, R)
    return out


def _gpu_sort_dist_id(dd, ids):
    """Rows of (FP64 distance, id) on the device -> lexicographic order."""
    import torch
    o = torch.argsort(ids, dim=1, stable=True)
    dd, ids = torch.gather(dd, 1, o), torch.gather(ids, 1, o)
    o = torch.argsort(dd, dim=1, stable=True)
    return torch.gather(dd, 1, o), torch.gather(ids, 1, o)


def knn_graph_partitioned(base: np.ndarray, R: int, device: str = "cuda", part_size: int = 2048,
                          probes: int = 8, lloyd_iters: int = 2, seed: int = 7) -> np.ndarray:
    """A degree-R kNN graph for bases too large for the exact builder (10M rows).

    The base is split into ~n/part_size parts by nearest centroid (centroids
    start as a seeded sample of base rows, then `lloyd_iters` mean updates).
    Each row's neighbours are searched among the rows of the `probes` parts
    whose centroids are nearest its own part's centroid: candidates by FP32
    distances, the best R + 8 re-measured in FP64 and ordered by (distance,
    id), self excluded.  Rows whose true neighbours lie outside the probed
    parts get near neighbours instead, so the graph is approximate;
    graph_edge_recall() measures how close it is on a sample."""
    import torch
    dev = torch.device(device)
    X = torch.from_numpy(np.ascontiguousarray(base, np.float32)).to(dev)
    n, d = X.shape
    n_parts = max(1, min(n // max(1, part_size), 65536))
    probes = min(probes, n_parts)
    rng = _rng(seed)
    cent = X[torch.from_numpy(np.sort(rng.choice(n, n_parts, replace=False))).to(dev)].clone()
    prev = torch.backends.cuda.matmul.allow_tf32
    torch.backends.cuda.matmul.allow_tf32 = False
    try:
        xn = (X * X).sum(1)
        assign = torch.empty(n, dtype=torch.int64, device=dev)
        for it in range(lloyd_iters + 1):
            cn = (cent * cent).sum(1)
            for s in range(0, n, 1 << 18):
                e = min(n, s + (1 << 18))
                assign[s:e] = torch.argmin(cn[None, :] - 2.0 * (X[s:e] @ cent.T), dim=1)
            if it == lloyd_iters:
                break
            sums = torch.zeros_like(cent).index_add_(0, assign, X)
            cnt = torch.bincount(assign, minlength=n_parts).to(X.dtype)
            keep = cnt > 0
            cent[keep] = sums[keep] / cnt[keep, None]
        order = torch.argsort(assign, stable=True)
        counts = torch.bincount(assign, minlength=n_parts)
        offs = torch.zeros(n_parts + 1, dtype=torch.int64, device=dev)
        offs[1:] = torch.cumsum(counts, 0)
        cn = (cent * cent).sum(1)
        probe = torch.topk(cn[:, None] + cn[None, :] - 2.0 * (cent @ cent.T), probes, dim=1,
                           largest=False).indices
        offs_h, probe_h = offs.cpu().numpy(), probe.cpu().numpy()
        out = torch.empty((n, R), dtype=torch.int32, device=dev)
        kk = R + 8
        for p in range(n_parts):
            qi = order[offs_h[p]:offs_h[p + 1]]
            if qi.numel() == 0:
                continue
            ci = torch.cat([order[offs_h[c]:offs_h[c + 1]] for c in probe_h[p]])
            C = X[ci]
            for s in range(0, qi.numel(), 4096):
                qs = qi[s:s + 4096]
                D = xn[qs, None] + xn[None, ci] - 2.0 * (X[qs] @ C.T)
                D[qs[:, None] == ci[None, :]] = float("inf")
                k_here = min(kk, ci.numel() - 1)
                iv = torch.topk(D, k_here, dim=1, largest=False).indices
                cand = ci[iv]
                dd = ((X[cand].double() - X[qs, None, :].double()) ** 2).sum(-1)
                dd, cand = _gpu_sort_dist_id(dd, cand)
                row = torch.full((qs.numel(), R), n, dtype=torch.int64, device=dev)
                m = min(R, k_here)
                row[:, :m] = cand[:, :m]
                out[qs] = row.to(torch.int32)
    finally:
        torch.backends.cuda.matmul.allow_tf32 = prev
    return out.cpu().numpy()


def graph_edge_recall(base: np.ndarray, graph: np.ndarray, sample: int = 2000, seed: int = 11,
                      device: str | None = None) -> float:
    """Fraction of the true R nearest neighbours (FP64, self excluded) that a
    graph lists, over a seeded sample of rows."""
    n, R = graph.shape
    rows = np.sort(_rng(seed).choice(n, min(sample, n), replace=False))
    gt = ground_truth(base, base[rows], R + 1, device=device)
    hit = 0
    for r, g, t in zip(rows, graph[rows], gt):
        t = t[t != r][:R]
        hit += len(np.intersect1d(g, t))
    return hit / (len(rows) * R)


def ground_truth(base: np.ndarray, queries: np.ndarray, k: int = 100, device: str | None = None,
                 chunk: int = 1024) -> np.ndarray:
    """FP64 brute-force k nearest base ids per query, ordered by (dist, id).

    Bases above 4M rows preselect k + 64 candidates per query by FP32
    distances and measure those in FP64 (a full FP64 pass over 10M rows
    takes tens of seconds); the FP32 error is far below the distance gap of
    64 ranks."""
    torch, dev = _torch_device(device)
    if dev is not None and base.shape[0] > 4_000_000:
        return _ground_truth_preselect(base, queries, k, torch, dev)
    nq = queries.shape[0]
    out = np.empty((nq, k), np.int32)
    extra = 16
    kk = min(base.shape[0], k + extra)
    if dev is not None:
        X = torch.from_numpy(base).to(dev).double()
        nrm = (X ** 2).sum(1)
        Q = torch.from_numpy(queries).to(dev).double()
        for s in range(0, nq, chunk):
            e = min(nq, s + chunk)
            q = Q[s:e]
            D = (q ** 2).sum(1)[:, None] + nrm[None, :] - 2.0 * (q @ X.T)
            _, iv = torch.topk(D, kk, dim=1, largest=False)
            cand = X[iv.reshape(-1)].reshape(e - s, kk, -1)
            dd = ((cand - q[:, None, :]) ** 2).sum(-1)
            _, iv_np = _sort_by_dist_then_id(dd.cpu().numpy(), iv.cpu().numpy())
            out[s:e] = iv_np[:, :k]
        return out
    X = base.astype(np.float64)
    nrm = (X ** 2).sum(1)
    for s in range(0, nq, 256):
        e = min(nq, s + 256)
        q = queries[s:e].astype(np.float64)
        D = (q ** 2).sum(1)[:, None] + nrm[None, :] - 2.0 * (q @ X.T)
        iv = np.argpartition(D, kk - 1, axis=1)[:, :kk] if kk < base.shape[0] else np.tile(
            np.arange(base.shape[0]), (e - s, 1))
        dd = ((X[iv] - q[:, None, :]) ** 2).sum(-1)
        _, iv = _sort_by_dist_then_id(dd, iv)
        out[s:e] = iv[:, :k]
    return out


def _ground_truth_preselect(base, queries, k, torch, dev, chunk=128):
    prev = torch.backends.cuda.matmul.allow_tf32
    torch.backends.cuda.matmul.allow_tf32 = False
    try:
        X = torch.from_numpy(np.ascontiguousarray(base, np.float32)).to(dev)
        xn = (X * X).sum(1)
        Q = torch.from_numpy(np.ascontiguousarray(queries, np.float32)).to(dev)
        out = np.empty((Q.shape[0], k), np.int32)
        kk = min(X.shape[0], k + 64)
        for s in range(0, Q.shape[0], chunk):
            q = Q[s:s + chunk]
            iv = torch.topk(xn[None, :] - 2.0 * (q @ X.T), kk, dim=1, largest=False).indices
            dd = ((X[iv].double() - q[:, None, :].double()) ** 2).sum(-1)
            _, iv = _gpu_sort_dist_id(dd, iv)
            out[s:s + chunk] = iv[:, :k].cpu().numpy()
    finally:
        torch.backends.cuda.matmul.allow_tf32 = prev
    return out


def recall_at(ids: np.ndarray, gt: np.ndarray, k: int = 10) -> float:
    """k@k recall: fraction of the true top-k found among the returned top-k."""
    ids = np.asarray(ids)[:, :k]
    gt = np.asarray(gt)[:, :k]
    hit = 0
    for a, b in zip(ids, gt):
        hit += len(np.intersect1d(a, b, assume_unique=False))
    return hit / (gt.shape[0] * k)


def recall_reference_style(ids: np.ndarray, gt: np.ndarray, k: int = 10) -> float:
    """The reference's recall@k: true top-k ids found anywhere in the returned
    list (graph_helper.cu:64-80), which with topk = beam is k@beam."""
    hit = 0
    for a, b in zip(np.asarray(ids), np.asarray(gt)[:, :k]):
        hit += np.isin(b, a).sum()
    return hit / (gt.shape[0] * k)


def stream_batches(n_batches: int = 2000, max_batch: int = 8192, seed: int = SEED_STREAM):
    """Config-5 batch plan: sizes floor(exp(U[0, ln max_batch])), k in {1,10,100}."""
    rng = _rng(seed)
    sizes = np.floor(np.exp(rng.uniform(0, math.log(max_batch), n_batches))).astype(np.int64)
    sizes = np.maximum(sizes, 1)
    ks = rng.choice(np.array([1, 10, 100]), n_batches)
    return sizes, ks
