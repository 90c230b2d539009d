"""ORACLE -- CPU restatement of rt_entry's query path (test infrastructure).

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline
leg may import this package.  It is the oracle, never the thing measured or
shipped: the product (``rt_entry_gb300``) has no dependency on it.

``build()`` compiles ``search_ref.cpp`` and ``kdtree_ref.cpp`` (plain C++,
OpenMP, ``-ffp-contract=off``) into ``oracle/_build/liboracle.so``.
``build_reference()`` runs ``oracle/ref/Makefile`` when the reference tree is
present (this machine only), producing the reference's own kd-tree and PCA as
executables and its search kernel as sm_103a cubins in ``oracle/_ref/``.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from concurrent.futures import ThreadPoolExecutor

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
REF_OUT = os.path.join(HERE, "_ref")
# The reference's source tree: $RTE_REFERENCE_TREE, else a directory named
# `reference` beside this repository.  It exists only where fixtures are made.
REFERENCE_TREE = os.environ.get("RTE_REFERENCE_TREE") or os.path.join(
    os.path.dirname(os.path.dirname(HERE)), "reference")
LIB = os.path.join(BUILD, "liboracle.so")
REF_LAUNCH_LIB = os.path.join(BUILD, "liboracle_refgpu.so")
MAX_DIST = np.float32(536870912.0)

_lib = None


def _run(cmd):
    subprocess.run(cmd, check=True)


def build(force: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    srcs = [os.path.join(HERE, f) for f in ("search_ref.cpp", "kdtree_ref.cpp")]
    if force or not os.path.exists(LIB) or any(
        os.path.getmtime(s) > os.path.getmtime(LIB) for s in srcs
    ):
        objs = []
        cmds = []
        for s in srcs:
            o = os.path.join(BUILD, os.path.basename(s) + ".o")
            objs.append(o)
            cmds.append(["g++", "-O2", "-std=c++17", "-fPIC", "-fopenmp", "-ffp-contract=off",
                         "-c", s, "-o", o])
        with ThreadPoolExecutor(len(cmds)) as ex:
            list(ex.map(_run, cmds))
        _run(["g++", "-shared", "-fopenmp", "-o", LIB] + objs)
    return LIB


def build_ref_launcher(force: bool = False) -> str | None:
    """Driver-API launcher for the reference kernel cubins (run on a GPU)."""
    src = os.path.join(HERE, "ref_launch.cpp")
    if not os.path.exists(src):
        return None
    os.makedirs(BUILD, exist_ok=True)
    if force or not os.path.exists(REF_LAUNCH_LIB) or os.path.getmtime(src) > os.path.getmtime(
        REF_LAUNCH_LIB
    ):
        _run(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-I/usr/local/cuda/include", src,
              "-o", REF_LAUNCH_LIB, "-L/usr/local/cuda/lib64", "-L/usr/local/cuda/lib64/stubs",
              "-lcuda"])
    return REF_LAUNCH_LIB


def build_reference() -> bool:
    """Compile the reference's own pieces when the reference tree exists."""
    if not os.path.isdir(REFERENCE_TREE):
        return False
    _run(["make", "-s", "-C", os.path.join(HERE, "ref"), "-j8", f"OUT={REF_OUT}",
          f"REF={REFERENCE_TREE}"])
    return True


N_COUNTERS = 7  # fields of Counters


class Counters(ctypes.Structure):
    """Per-query work counters (orc_counters): entries_valid, expanded,
    dist_evals, iterations, merges, merges_idle, merges_few."""
    _fields_ = [("entries_valid", ctypes.c_int64), ("expanded", ctypes.c_int64),
                ("dist_evals", ctypes.c_int64), ("iterations", ctypes.c_int64),
                ("merges", ctypes.c_int64), ("merges_idle", ctypes.c_int64),
                ("merges_few", ctypes.c_int64)]


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB)
        P = ctypes.c_void_p
        i64, i32, f32 = ctypes.c_int64, ctypes.c_int, ctypes.c_float
        L.orc_search.argtypes = [P, i64, i32, P, i64, P, i32, P, i32, P, i32, i32, i32, i32, i32,
                                 i32, i32, P, P, P, i32]
        L.orc_search.restype = i32
        L.orc_search_rerank.argtypes = [P, P, i64, i32, P, i64, P, i32, P, i32, P, P, i32, i32,
                                        i32, i32, i32, i32, i32, P, P, P, i32]
        L.orc_search_rerank.restype = i32
        L.orc_search_multi.argtypes = [P, i64, i32, P, i64, P, i32, P, i32, P, i32, i32, i32, i32,
                                       i32, i32, i32, P, P, P, i32]
        L.orc_search_multi.restype = i32
        L.orc_locate_multi.argtypes = [P, i64, P, i64, i32, i32, P, i32]
        L.orc_locate_multi.restype = None
        L.orc_rerank_full.argtypes = [P, i64, i32, P, i64, P, i32, i32, P, P, i32]
        L.orc_rerank_full.restype = i32
        L.orc_l2_ref.argtypes = [P, P, i32]
        L.orc_l2_ref.restype = f32
        L.orc_kdtree_build.argtypes = [P, i64, i32, i64, P, P, ctypes.POINTER(i64)]
        L.orc_kdtree_build.restype = i32
        L.orc_expand_boxes.argtypes = [P, i64, f32]
        L.orc_expand_boxes.restype = None
        L.orc_locate.argtypes = [P, i64, P, i64, i32, P, i32]
        L.orc_locate.restype = None
        L.orc_knn_fp64.argtypes = [P, i64, i32, P, i64, i32, P, P, i32]
        L.orc_knn_fp64.restype = None
        _lib = L
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


def _c(a, dt):
    return np.ascontiguousarray(a, dtype=dt)


def locate_multi(boxes, qp, H, n_threads=0):
    """The H smallest-index expanded leaf boxes containing each point
    ([nq, H], -1 padded)."""
    boxes = _c(boxes, np.float32)
    qp = _c(qp, np.float32)
    out = np.empty((qp.shape[0], H), np.int32)
    lib().orc_locate_multi(_p(boxes), boxes.shape[0], _p(qp), qp.shape[0], qp.shape[1], H, _p(out),
                           n_threads)
    return out


def search_multi(base, queries, graph, *, L, k, hits_multi, leaf_pids, search_width=1,
                 max_iter=100, bloom_words=512, bloom_hashes=3, n_threads=0, with_counters=False):
    """Kd-tree entries from several leaves per query (hits_multi [nq, H])."""
    base = _c(base, np.float32)
    queries = _c(queries, np.float32)
    graph = _c(graph, np.int32)
    hm = _c(hits_multi, np.int32)
    lp = _c(leaf_pids, np.int32)
    np_, d = base.shape
    nq = queries.shape[0]
    ids = np.empty((nq, k), np.int32)
    dists = np.empty((nq, k), np.float32)
    cnt = (Counters * max(nq, 1))() if with_counters else None
    rc = lib().orc_search_multi(_p(base), np_, d, _p(queries), nq, _p(graph), graph.shape[1], _p(lp),
                                lp.shape[1], _p(hm), hm.shape[1], L, k, search_width, max_iter,
                                bloom_words, bloom_hashes, _p(ids), _p(dists),
                                None if cnt is None else ctypes.cast(cnt, ctypes.c_void_p), n_threads)
    if rc != 0:
        raise ValueError("orc_search_multi rejected its arguments")
    if with_counters:
        return ids, dists, np.frombuffer(cnt, dtype=np.int64).reshape(-1, N_COUNTERS)[:nq].copy()
    return ids, dists


def rerank_full(base, queries, pool, k, n_threads=0):
    """Exact FP32 rerank of pools [nq, L] against the original rows -> the
    first k (ids, dists) of the ascending bitonic sort."""
    base = _c(base, np.float32)
    queries = _c(queries, np.float32)
    pool = _c(pool, np.int32)
    np_, dim = base.shape
    nq, L = pool.shape
    ids = np.empty((nq, k), np.int32)
    dists = np.empty((nq, k), np.float32)
    rc = lib().orc_rerank_full(_p(base), np_, dim, _p(queries), nq, _p(pool), L, k, _p(ids),
                               _p(dists), n_threads)
    if rc != 0:
        raise ValueError("orc_rerank_full rejected its arguments")
    return ids, dists


def search(base, queries, graph, *, L, k, search_width=1, max_iter=100, bloom_words=512,
           bloom_hashes=3, entry_mode=1, leaf_pids=None, hits=None, n_threads=0,
           with_counters=False, rerank_base=None, hits2=None):
    """Restated GraphSearchKernel over (base, queries, graph) -> (ids, dists[, counters]).

    With rerank_base, `base` is the reduced-precision copy (as FP32) the
    search runs on and the final pool is reranked exactly on rerank_base."""
    base = _c(base, np.float32)
    rb = None if rerank_base is None else _c(rerank_base, np.float32)
    queries = _c(queries, np.float32)
    graph = _c(graph, np.int32)
    np_, d = base.shape
    nq = queries.shape[0]
    degree = graph.shape[1]
    ids = np.empty((nq, k), np.int32)
    dists = np.empty((nq, k), np.float32)
    cnt = (Counters * max(nq, 1))() if with_counters else None
    lp = None if leaf_pids is None else _c(leaf_pids, np.int32)
    h = None if hits is None else _c(hits, np.int32)
    h2 = None if hits2 is None else _c(hits2, np.int32)
    cap = 0 if lp is None else lp.shape[1]
    rc = lib().orc_search_rerank(_p(base), _p(rb), np_, d, _p(queries), nq, _p(graph), degree, _p(lp), cap, _p(h), _p(h2),
                          L, k, search_width, max_iter, bloom_words, bloom_hashes, entry_mode,
                          _p(ids), _p(dists), None if cnt is None else ctypes.cast(cnt, ctypes.c_void_p),
                          n_threads)
    if rc != 0:
        raise ValueError("orc_search rejected its arguments")
    if with_counters:
        c = np.frombuffer(cnt, dtype=np.int64).reshape(-1, N_COUNTERS)[:nq].copy()
        return ids, dists, c
    return ids, dists


def l2_ref(p, q):
    p = _c(p, np.float32)
    q = _c(q, np.float32)
    return float(lib().orc_l2_ref(_p(p), _p(q), p.shape[0]))


def kdtree_build(pts3, leaf_cap):
    """-> (boxes [n_leaves,6] tight, pids [n_leaves, leaf_cap])."""
    pts3 = _c(pts3, np.float32)
    n = pts3.shape[0]
    max_leaves = 4 * (n // max(1, leaf_cap // 2) + 2)
    boxes = np.empty((max_leaves, 6), np.float32)
    pids = np.empty((max_leaves, leaf_cap), np.int32)
    nl = ctypes.c_int64(0)
    rc = lib().orc_kdtree_build(_p(pts3), n, leaf_cap, max_leaves, _p(boxes), _p(pids),
                                ctypes.byref(nl))
    if rc == -2:
        raise RuntimeError("kd-tree split failed (degenerate points)")
    if rc != 0:
        raise ValueError(f"orc_kdtree_build failed rc={rc}")
    return boxes[: nl.value].copy(), pids[: nl.value].copy()


def expand_boxes(boxes, ratio):
    b = _c(boxes, np.float32).copy()
    lib().orc_expand_boxes(_p(b), b.shape[0], ratio)
    return b


def locate(expanded_boxes, qp, n_threads=0):
    b = _c(expanded_boxes, np.float32)
    qp = _c(qp, np.float32)
    out = np.empty(qp.shape[0], np.int32)
    lib().orc_locate(_p(b), b.shape[0], _p(qp), qp.shape[0], qp.shape[1], _p(out), n_threads)
    return out


def knn_fp64(base, queries, k, n_threads=0):
    base = _c(base, np.float32)
    queries = _c(queries, np.float32)
    ids = np.empty((queries.shape[0], k), np.int32)
    d2 = np.empty((queries.shape[0], k), np.float64)
    lib().orc_knn_fp64(_p(base), base.shape[0], base.shape[1], _p(queries), queries.shape[0], k,
                       _p(ids), _p(d2), n_threads)
    return ids, d2


# ---- the reference's own programs, built from its sources (this machine) ----

def ref_kdtree(pts3, leaf_cap, workdir):
    """Run the reference's kdtree.cpp (oracle/_ref/kdtree_ref_main)."""
    exe = os.path.join(REF_OUT, "kdtree_ref_main")
    pts3 = _c(pts3, np.float32)
    inp = os.path.join(workdir, "kd_in.bin")
    out = os.path.join(workdir, "kd_out.bin")
    with open(inp, "wb") as f:
        f.write(np.int64(pts3.shape[0]).tobytes())
        f.write(pts3.tobytes())
    if os.path.exists(out):
        os.remove(out)
    subprocess.run([exe, inp, str(leaf_cap), out], check=True, stdout=subprocess.DEVNULL)
    if not os.path.exists(out):
        raise RuntimeError("reference kd-tree exited without output (split failed)")
    raw = open(out, "rb").read()
    nl = int(np.frombuffer(raw[:8], np.int64)[0])
    boxes = np.frombuffer(raw[8:8 + 24 * nl], np.float32).reshape(nl, 6).copy()
    pids = np.frombuffer(raw[8 + 24 * nl:], np.int32).reshape(nl, leaf_cap).copy()
    return boxes, pids


def ref_pca(x, workdir):
    """Run the reference's pca.cpp + Eigen -> (mean, eigvals, vec, projected)."""
    exe = os.path.join(REF_OUT, "pca_ref_main")
    x = _c(x, np.float32)
    n, d = x.shape
    inp = os.path.join(workdir, "pca_in.bin")
    out = os.path.join(workdir, "pca_out.bin")
    with open(inp, "wb") as f:
        f.write(np.int64(n).tobytes())
        f.write(np.int64(d).tobytes())
        f.write(x.tobytes())
    subprocess.run([exe, inp, out], check=True, stdout=subprocess.DEVNULL)
    raw = open(out, "rb").read()
    o = 0
    mean = np.frombuffer(raw, np.float64, d, o); o += 8 * d
    val = np.frombuffer(raw, np.float64, d, o); o += 8 * d
    vec = np.frombuffer(raw, np.float64, d * d, o).reshape(d, d); o += 8 * d * d
    proj = np.frombuffer(raw, np.float32, n * d, o).reshape(n, d)
    return mean.copy(), val.copy(), vec.copy(), proj.copy()


# ---- the reference's own search kernel on a GPU (oracle/ref_launch.cpp) ----

def entries_table(leaf_pids, L, np_):
    """aabb_entries [n_leaves x L] (entry.cu:60-69): entry j of a leaf is its
    j-th point for j < leaf size, else np."""
    leaf_pids = np.asarray(leaf_pids)
    nl, cap = leaf_pids.shape
    t = np.full((nl, L), np_, np.int32)
    m = min(cap, L)
    t[:, :m] = leaf_pids[:, :m]
    return t


def ref_kernel_available(dim):
    """True when the reference kernel was compiled for this dimension."""
    return os.path.exists(os.path.join(REF_OUT, f"graph_search_d{dim}.cubin"))


class RefKernel:
    """The reference's GraphSearchKernel, compiled from its own source for
    sm_103a (oracle/_ref/graph_search_d<dim>.cubin), launched as
    graph.cu:318-324 launches it.  Uploads base [np x dim] and graph once."""

    def __init__(self, base, graph):
        base = _c(base, np.float32)
        graph = _c(graph, np.int32)
        self.np, self.dim = base.shape
        cubin = os.path.join(REF_OUT, f"graph_search_d{self.dim}.cubin")
        if not os.path.exists(cubin):
            raise FileNotFoundError(f"{cubin} is not built (oracle/ref/Makefile needs the reference tree)")
        L = ctypes.CDLL(build_ref_launcher())
        P, I = ctypes.c_void_p, ctypes.c_int
        L.ref_last_error.restype = ctypes.c_char_p
        L.ref_open.argtypes = [ctypes.c_char_p, P, I, I, P, I, ctypes.POINTER(P)]
        L.ref_open.restype = I
        L.ref_search.argtypes = [P, P, I, P, I, I, P, I, I, I, I, I, I, P, P]
        L.ref_search.restype = I
        L.ref_close.argtypes = [P]
        L.ref_close.restype = None
        self._lib = L
        self._h = P()
        rc = L.ref_open(cubin.encode(), _p(base), self.np, self.dim, _p(graph), graph.shape[1],
                        ctypes.byref(self._h))
        if rc != 0:
            raise RuntimeError(f"ref_open: {L.ref_last_error().decode()}")

    def search(self, queries, entries, hits, L, topk, max_iter=100, algo=1, scrub=False, reps=0):
        """-> (ids [nq, topk], per-launch device ms [reps])."""
        q = _c(queries, np.float32)
        e = _c(entries, np.int32)
        h = _c(hits, np.int32)
        nq = q.shape[0]
        out = np.empty((nq, topk), np.int32)
        ms = np.zeros(max(reps, 1), np.float32)
        rc = self._lib.ref_search(self._h, _p(q), nq, _p(e), e.shape[0], L, _p(h), topk, 1, max_iter,
                                  algo, int(scrub), reps, _p(ms), _p(out))
        if rc != 0:
            raise RuntimeError(f"ref_search: {self._lib.ref_last_error().decode()}")
        return out, ms[:reps].tolist()

    def close(self):
        if getattr(self, "_h", None):
            self._lib.ref_close(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
