"""rt_entry_gb300 -- GB300 (sm_103a) query path of rt_entry, Python binding.

Thin ctypes layer over the C ABI in ``include/rtentry.h`` (librtentry.so,
built in-tree by ``rt_entry_gb300.build.build()``).  The compute runs in
hand-written CUDA kernels; there is no CPU fallback: importing the binding
without the built library raises.

Arrays may be numpy arrays (host) or torch tensors (host or CUDA).  Results
come back in the same kind of memory as the queries.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_build", "librtentry.so")

RTE_OK, RTE_EINVAL, RTE_ENOMEM, RTE_EIO, RTE_ECUDA, RTE_ETIMEOUT, RTE_ESTATE = range(7)
PREC_FP32, PREC_BF16, PREC_FP8 = 0, 1, 2
COPY_BF16, COPY_FP8, COPY_RAW = 1, 2, 4
ENTRY_RANDOM, ENTRY_KDTREE, ENTRY_LEARNED = 0, 1, 2
MAX_DIST = np.float32(536870912.0)

# every entry point include/rtentry.h declares
EXPORTS = (
    "rte_default_params", "rte_index_from_host", "rte_index_load", "rte_build_pca", "rte_set_pca",
    "rte_build_kdtree", "rte_project", "rte_locate", "rte_search", "rte_search_projected",
    "rte_search_counters", "rte_index_get_info", "rte_get_pca", "rte_get_search_base",
    "rte_get_kdtree", "rte_index_save", "rte_index_load_dir", "rte_index_free", "rte_last_error",
    "rte_kdtree_build_host", "rte_sym_eig_host", "rte_get_search_base_lowp", "rte_gemm_bf16",
    "rte_default_train_params", "rte_learned_train", "rte_learned_predict", "rte_mlp_grad_check",
    "rte_search_projected_noalloc", "rte_gemm_bf16_bias_argmax", "rte_mlp_head_argmax", "rte_knn_graph", "rte_locate_multi", "rte_batcher_create", "rte_batcher_search", "rte_batcher_k",
    "rte_batcher_free", "rte_autotune", "rte_set_wait_limit", "rte_index_load_reference",
    "rte_read_vectors", "rte_index_prepare", "rte_index_release", "rte_scratch_pool_usage",
)


class SearchParams(ctypes.Structure):
    _fields_ = [("k", ctypes.c_int), ("beam", ctypes.c_int), ("search_width", ctypes.c_int),
                ("max_iter", ctypes.c_int), ("bloom_words", ctypes.c_int),
                ("bloom_hashes", ctypes.c_int), ("precision", ctypes.c_int),
                ("rerank", ctypes.c_int), ("entry_mode", ctypes.c_int),
                ("warps_per_block", ctypes.c_int), ("max_hits", ctypes.c_int),
                ("team_warps", ctypes.c_int)]


class IndexInfo(ctypes.Structure):
    _fields_ = [("np", ctypes.c_int64), ("dim", ctypes.c_int), ("search_dim", ctypes.c_int),
                ("degree", ctypes.c_int), ("has_pca", ctypes.c_int), ("has_kdtree", ctypes.c_int),
                ("n_leaves", ctypes.c_int64), ("leaf_size", ctypes.c_int),
                ("expand_ratio", ctypes.c_float), ("has_bf16", ctypes.c_int),
                ("has_fp8", ctypes.c_int), ("device", ctypes.c_int),
                ("device_bytes", ctypes.c_int64)]


class TrainParams(ctypes.Structure):
    _fields_ = [("hidden", ctypes.c_int), ("epochs", ctypes.c_int), ("batch", ctypes.c_int),
                ("lr", ctypes.c_float), ("label_beam", ctypes.c_int), ("seed", ctypes.c_int),
                ("max_classes", ctypes.c_int)]


class TrainReport(ctypes.Structure):
    _fields_ = [("first_loss", ctypes.c_float), ("last_loss", ctypes.c_float),
                ("train_acc", ctypes.c_float), ("n_train", ctypes.c_int64),
                ("classes", ctypes.c_int), ("steps", ctypes.c_int64), ("train_ms", ctypes.c_float)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class AutotuneReport(ctypes.Structure):
    _fields_ = [("met_target", ctypes.c_int), ("recall", ctypes.c_float), ("ms", ctypes.c_float),
                ("qps", ctypes.c_float), ("evaluated", ctypes.c_int)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class RteError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"rte status {status}: {msg}")
        self.status = status


_lib = None


def load_library(path: str = LIB_PATH):
    """Load librtentry.so; raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise ImportError(f"{path} is missing: run `python -m rt_entry_gb300.build` "
                          "(or __graft_entry__.build()) first; there is no CPU fallback")
    L = ctypes.CDLL(path)
    P, i64, i32 = ctypes.c_void_p, ctypes.c_int64, ctypes.c_int
    PP = ctypes.POINTER(ctypes.c_void_p)
    SP = ctypes.POINTER(SearchParams)
    sig = {
        "rte_default_params": ([SP], None),
        "rte_index_from_host": ([P, i64, i32, P, i32, i32, PP], i32),
        "rte_index_load": ([ctypes.c_char_p, ctypes.c_char_p, i32, PP], i32),
        "rte_build_pca": ([P, i32], i32),
        "rte_set_pca": ([P, P, P, i32], i32),
        "rte_build_kdtree": ([P, i32, ctypes.c_float], i32),
        "rte_project": ([P, P, i64, P, P], i32),
        "rte_locate": ([P, P, i64, P, P], i32),
        "rte_search": ([P, P, i64, SP, P, P, P], i32),
        "rte_search_projected": ([P, P, P, i64, SP, P, P, P], i32),
        "rte_search_counters": ([P, P, P, i64, SP, P, P], i32),
        "rte_index_get_info": ([P, ctypes.POINTER(IndexInfo)], i32),
        "rte_get_pca": ([P, P, P, P], i32),
        "rte_get_search_base": ([P, P], i32),
        "rte_get_kdtree": ([P, P, P, P], i32),
        "rte_index_save": ([P, ctypes.c_char_p], i32),
        "rte_index_load_dir": ([ctypes.c_char_p, i32, PP], i32),
        "rte_index_free": ([P], None),
        "rte_last_error": ([], ctypes.c_char_p),
        "rte_kdtree_build_host": ([P, i64, i32, ctypes.c_float, i64, P, P, P,
                                   ctypes.POINTER(i64)], i32),
        "rte_sym_eig_host": ([P, i32, P, P], i32),
        "rte_get_search_base_lowp": ([P, i32, P], i32),
        "rte_gemm_bf16": ([P, P, i32, i32, i32, P, P], i32),
        "rte_gemm_bf16_bias_argmax": ([P, P, P, i32, i32, i32, P, P], i32),
        "rte_mlp_head_argmax": ([P, i32, i32, P, P, P, P, P, P, i32, i32, i32, P, P], i32),
        "rte_knn_graph": ([P, i64, i32, i32, i32, P, P], i32),
        "rte_locate_multi": ([P, P, i64, i32, P, P], i32),
        "rte_default_train_params": ([ctypes.POINTER(TrainParams)], None),
        "rte_learned_train": ([P, P, i64, ctypes.POINTER(TrainParams), ctypes.POINTER(TrainReport)], i32),
        "rte_learned_predict": ([P, P, i64, P, P], i32),
        "rte_mlp_grad_check": ([P, P, i32, i32, i32, i32] + [P] * 13, i32),
        "rte_search_projected_noalloc": ([P, P, P, i64, SP, P, P, P], i32),
        "rte_batcher_create": ([P, i64, SP, PP], i32),
        "rte_batcher_search": ([P, P, i64, P, P, P], i32),
        "rte_batcher_k": ([P], i32),
        "rte_batcher_free": ([P], None),
        "rte_autotune": ([P, P, i64, P, i32, i32, ctypes.c_float, SP,
                          ctypes.POINTER(AutotuneReport)], i32),
        "rte_set_wait_limit": ([ctypes.c_longlong], None),
        "rte_index_load_reference": ([ctypes.c_char_p, ctypes.c_char_p, ctypes.c_char_p, i32, i32,
                                      ctypes.c_float, i32, PP], i32),
        "rte_read_vectors": ([ctypes.c_char_p, P, i64, ctypes.POINTER(i64), ctypes.POINTER(i32)], i32),
        "rte_index_prepare": ([P, ctypes.c_uint], i32),
        "rte_index_release": ([P, ctypes.c_uint], i32),
    }
    for name, (args, res) in sig.items():
        f = getattr(L, name)
        f.argtypes = args
        f.restype = res
    _lib = L
    return L


def _check(rc: int):
    if rc != RTE_OK:
        raise RteError(rc, load_library().rte_last_error().decode())


def default_params(**kw) -> SearchParams:
    p = SearchParams()
    load_library().rte_default_params(ctypes.byref(p))
    for k, v in kw.items():
        if not hasattr(p, k):
            raise TypeError(f"unknown search parameter {k}")
        setattr(p, k, int(v))
    return p


def _is_torch(x):
    return type(x).__module__.startswith("torch")


def _ptr(x):
    """(pointer, keepalive) of a C-contiguous numpy array or torch tensor."""
    if x is None:
        return None, None
    if _is_torch(x):
        if not x.is_contiguous():
            x = x.contiguous()
        return ctypes.c_void_p(x.data_ptr()), x
    a = np.ascontiguousarray(x)
    return a.ctypes.data_as(ctypes.c_void_p), a


def _as(x, np_dtype, torch_dtype_name):
    if _is_torch(x):
        import torch
        dt = getattr(torch, torch_dtype_name)
        if x.dtype != dt:  # skips the dispatcher when nothing is to be done
            x = x.to(dt)
        return x if x.is_contiguous() else x.contiguous()
    return np.ascontiguousarray(x, dtype=np_dtype)


def _empty_like_kind(ref, shape, np_dtype, torch_dtype_name):
    if _is_torch(ref):
        import torch
        return torch.empty(shape, dtype=getattr(torch, torch_dtype_name), device=ref.device)
    return np.empty(shape, dtype=np_dtype)


def _stream_ptr(stream):
    if stream is None:
        return None
    if hasattr(stream, "cuda_stream"):
        return ctypes.c_void_p(stream.cuda_stream)
    return ctypes.c_void_p(int(stream))


def kdtree_build_host(xyz, leaf_size: int, expand_ratio: float = 0.2):
    """Host kd-tree build alone -> (tight [n,6], expanded [n,6], pids [n, leaf_size])."""
    xyz = np.ascontiguousarray(xyz, np.float32)
    n = xyz.shape[0]
    cap = 4 * (n // max(1, leaf_size // 2) + 2)
    t = np.empty((cap, 6), np.float32)
    e = np.empty((cap, 6), np.float32)
    p = np.empty((cap, leaf_size), np.int32)
    nl = ctypes.c_int64(0)
    _check(load_library().rte_kdtree_build_host(
        xyz.ctypes.data_as(ctypes.c_void_p), n, leaf_size, expand_ratio, cap,
        t.ctypes.data_as(ctypes.c_void_p), e.ctypes.data_as(ctypes.c_void_p),
        p.ctypes.data_as(ctypes.c_void_p), ctypes.byref(nl)))
    k = nl.value
    return t[:k].copy(), e[:k].copy(), p[:k].copy()


def sym_eig_host(a):
    """FP64 eigendecomposition of the build path -> (w descending, V columns)."""
    a = np.ascontiguousarray(a, np.float64)
    n = a.shape[0]
    w = np.empty(n, np.float64)
    v = np.empty((n, n), np.float64)
    _check(load_library().rte_sym_eig_host(a.ctypes.data_as(ctypes.c_void_p), n,
                                           w.ctypes.data_as(ctypes.c_void_p),
                                           v.ctypes.data_as(ctypes.c_void_p)))
    return w, v


def read_vectors(path: str) -> np.ndarray:
    """A vector file as the reference reads it (.fvecs, .bvecs, .fbin,
    .hvecs, .hh, .txt) -> float32 [n, d], on the host."""
    L = load_library()
    n, d = ctypes.c_int64(), ctypes.c_int()
    _check(L.rte_read_vectors(path.encode(), None, 0, ctypes.byref(n), ctypes.byref(d)))
    out = np.empty((n.value, d.value), np.float32)
    _check(L.rte_read_vectors(path.encode(), out.ctypes.data_as(ctypes.c_void_p), out.size,
                              ctypes.byref(n), ctypes.byref(d)))
    return out


def bf16_bits(x):
    """FP32 -> BF16 bit patterns (round to nearest even), as uint16."""
    b = np.ascontiguousarray(x, np.float32).view(np.uint32).astype(np.uint64)
    return ((b + 0x7FFF + ((b >> 16) & 1)) >> 16).astype(np.uint16)


def knn_graph(base, degree: int, device: int = 0):
    """Exact degree-R kNN graph of base [n, d] on the GPU: [n, R] int32, rows
    in (FP64 distance, id) order, self excluded.  numpy or torch (device) in;
    numpy out for numpy in, torch for torch."""
    b = _as(base, np.float32, "float32")
    n, d = b.shape
    out = _empty_like_kind(b, (n, degree), np.int32, "int32")
    pb, kb = _ptr(b)
    po, ko = _ptr(out)
    _check(load_library().rte_knn_graph(pb, n, d, degree, device, po, None))
    return out


def gemm_bf16_bias_argmax(a_bits, b_bits, bias):
    """Row argmax of A @ B.T + bias on the tensor cores (the learned head's
    last layer); A [M,K], B [N,K] BF16 bit patterns, bias [N] FP32."""
    a = np.ascontiguousarray(a_bits, np.uint16)
    b = np.ascontiguousarray(b_bits, np.uint16)
    bias = np.ascontiguousarray(bias, np.float32)
    M, K = a.shape
    N = b.shape[0]
    out = np.empty(M, np.int32)
    _check(load_library().rte_gemm_bf16_bias_argmax(
        a.ctypes.data_as(ctypes.c_void_p), b.ctypes.data_as(ctypes.c_void_p),
        bias.ctypes.data_as(ctypes.c_void_p), M, N, K, out.ctypes.data_as(ctypes.c_void_p), None))
    return out


def mlp_head_argmax(x, w1, b1, w2, b2, w3, b3, path: int = 0, stream=None):
    """Row argmax of the learned head's forward pass on device tensors:
    x [M, dp], w1 [H, dp], w2 [H, H], w3 [N, H] BF16 (torch.bfloat16 or
    int16/uint16 bit patterns), biases FP32.  path 0 is the fused kernel,
    path 1 the three layer-by-layer GEMMs.  Returns cols [M] int32 on the
    device."""
    import torch
    ts = [x, w1, b1, w2, b2, w3, b3]
    for t in ts:
        if not (isinstance(t, torch.Tensor) and t.is_cuda and t.is_contiguous()):
            raise ValueError("mlp_head_argmax takes contiguous CUDA tensors")
    M, dp = x.shape
    H, N = w1.shape[0], w3.shape[0]
    cols = torch.empty(M, dtype=torch.int32, device=x.device)
    _check(load_library().rte_mlp_head_argmax(
        x.data_ptr(), M, dp, w1.data_ptr(), b1.data_ptr(), w2.data_ptr(), b2.data_ptr(),
        w3.data_ptr(), b3.data_ptr(), H, N, path, cols.data_ptr(), _stream_ptr(stream)))
    return cols


def gemm_bf16(a_bits, b_bits):
    """C = A @ B.T on the tensor cores; A [M,K], B [N,K] BF16 bit patterns."""
    a = np.ascontiguousarray(a_bits, np.uint16)
    b = np.ascontiguousarray(b_bits, np.uint16)
    M, K = a.shape
    N = b.shape[0]
    c = np.empty((M, N), np.float32)
    _check(load_library().rte_gemm_bf16(a.ctypes.data_as(ctypes.c_void_p),
                                        b.ctypes.data_as(ctypes.c_void_p), M, N, K,
                                        c.ctypes.data_as(ctypes.c_void_p), None))
    return c


def mlp_grad_check(X, labels, W1, b1, W2, b2, W3, b3):
    """GPU forward+backward of the learned-entry MLP -> (grads dict, loss[M])."""
    X = np.ascontiguousarray(X, np.float32)
    labels = np.ascontiguousarray(labels, np.int32)
    ws = [np.ascontiguousarray(w, np.float32) for w in (W1, b1, W2, b2, W3, b3)]
    M, d = X.shape
    H, C = ws[0].shape[0], ws[4].shape[0]
    gs = [np.empty_like(w) for w in ws]
    loss = np.empty(M, np.float32)
    p = lambda a: a.ctypes.data_as(ctypes.c_void_p)
    _check(load_library().rte_mlp_grad_check(p(X), p(labels), M, d, H, C, *[p(w) for w in ws],
                                             p(gs[0]), p(gs[1]), p(gs[2]), p(gs[3]), p(gs[4]),
                                             p(gs[5]), p(loss)))
    return dict(zip(("W1", "b1", "W2", "b2", "W3", "b3"), gs)), loss


class Index:
    """One index on one GPU (the reference's Graph, graph.h:10-82)."""

    def __init__(self, handle):
        self._h = handle

    # ---- construction -------------------------------------------------
    @classmethod
    def from_arrays(cls, base, graph, device: int = 0) -> "Index":
        base = _as(base, np.float32, "float32")
        graph = _as(graph, np.int32, "int32")
        pb, kb = _ptr(base)
        pg, kg = _ptr(graph)
        h = ctypes.c_void_p()
        _check(load_library().rte_index_from_host(pb, base.shape[0], base.shape[1], pg,
                                                  graph.shape[1], device, ctypes.byref(h)))
        return cls(h)

    @classmethod
    def load(cls, base_path: str, graph_path: str, device: int = 0) -> "Index":
        h = ctypes.c_void_p()
        _check(load_library().rte_index_load(base_path.encode(), graph_path.encode(), device,
                                             ctypes.byref(h)))
        return cls(h)

    @classmethod
    def load_reference(cls, data_dir: str, base_path: str, graph_path: str, keep_dims: int = 0,
                       leaf_size: int = 0, expand_ratio: float = 0.2, device: int = 0) -> "Index":
        """An index from the reference's data directory (O.fbin, mean.fbin,
        pca_base.fbin, <leaf_size>_0.aabbs) plus its base and graph files."""
        h = ctypes.c_void_p()
        _check(load_library().rte_index_load_reference(data_dir.encode(), base_path.encode(),
                                                       graph_path.encode(), keep_dims, leaf_size,
                                                       expand_ratio, device, ctypes.byref(h)))
        return cls(h)

    @classmethod
    def load_dir(cls, path: str, device: int = 0) -> "Index":
        h = ctypes.c_void_p()
        _check(load_library().rte_index_load_dir(path.encode(), device, ctypes.byref(h)))
        return cls(h)

    def close(self):
        if getattr(self, "_h", None):
            load_library().rte_index_free(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def prepare(self, copies: int):
        """Make the BF16 (COPY_BF16) / FP8 (COPY_FP8) copies now."""
        _check(load_library().rte_index_prepare(self._h, copies))
        return self

    def release(self, copies: int):
        """Free the BF16 / FP8 copies (made again on next use) or the raw base."""
        _check(load_library().rte_index_release(self._h, copies))
        return self

    # ---- build steps ----------------------------------------------------
    def build_pca(self, keep_dims: int = 0):
        _check(load_library().rte_build_pca(self._h, keep_dims))
        return self

    def set_pca(self, mean, rotation, keep_dims: int = 0):
        m, km = _ptr(np.ascontiguousarray(mean, np.float32))
        r, kr = _ptr(np.ascontiguousarray(rotation, np.float32))
        _check(load_library().rte_set_pca(self._h, m, r, keep_dims))
        return self

    def build_kdtree(self, leaf_size: int, expand_ratio: float = 0.2):
        _check(load_library().rte_build_kdtree(self._h, leaf_size, expand_ratio))
        return self

    # ---- queries ----------------------------------------------------------
    @property
    def info(self) -> IndexInfo:
        i = IndexInfo()
        _check(load_library().rte_index_get_info(self._h, ctypes.byref(i)))
        return i

    def project(self, queries, stream=None):
        queries = _as(queries, np.float32, "float32")
        out = _empty_like_kind(queries, (queries.shape[0], self.info.search_dim), np.float32, "float32")
        pq, kq = _ptr(queries)
        po, ko = _ptr(out)
        _check(load_library().rte_project(self._h, pq, queries.shape[0], po, _stream_ptr(stream)))
        return out

    def locate(self, projected, stream=None, max_hits: int = 1):
        """Leaf per projected query ([nq]); with max_hits > 1 the first
        max_hits containing leaves ([nq, max_hits], -1 padded)."""
        projected = _as(projected, np.float32, "float32")
        shape = (projected.shape[0],) if max_hits == 1 else (projected.shape[0], max_hits)
        out = _empty_like_kind(projected, shape, np.int32, "int32")
        pp, kp = _ptr(projected)
        po, ko = _ptr(out)
        if max_hits == 1:
            _check(load_library().rte_locate(self._h, pp, projected.shape[0], po, _stream_ptr(stream)))
        else:
            _check(load_library().rte_locate_multi(self._h, pp, projected.shape[0], max_hits, po,
                                                   _stream_ptr(stream)))
        return out

    def _params(self, params, kw):
        if params is None:
            params = default_params(**kw)
        elif kw:
            raise TypeError("pass either params or keyword parameters")
        return params

    def _k(self, params):
        L = 1
        while L < params.beam:
            L <<= 1
        return params.k if params.k else L

    def search(self, queries, params: SearchParams | None = None, stream=None, out_ids=None,
               out_dists=None, **kw):
        """Whole query path: projection, entry selection, beam search."""
        params = self._params(params, kw)
        queries = _as(queries, np.float32, "float32")
        nq = queries.shape[0]
        k = self._k(params)
        if out_ids is None:
            out_ids = _empty_like_kind(queries, (nq, k), np.int32, "int32")
        if out_dists is None:
            out_dists = _empty_like_kind(queries, (nq, k), np.float32, "float32")
        pq, kq = _ptr(queries)
        pi, ki = _ptr(out_ids)
        pd, kd = _ptr(out_dists)
        _check(load_library().rte_search(self._h, pq, nq, ctypes.byref(params), pi, pd,
                                         _stream_ptr(stream)))
        return out_ids, out_dists

    def search_projected(self, projected, hits=None, params: SearchParams | None = None,
                         stream=None, **kw):
        params = self._params(params, kw)
        projected = _as(projected, np.float32, "float32")
        nq = projected.shape[0]
        k = self._k(params)
        ids = _empty_like_kind(projected, (nq, k), np.int32, "int32")
        dists = _empty_like_kind(projected, (nq, k), np.float32, "float32")
        if hits is not None:
            hits = _as(hits, np.int32, "int32")
        pp, kp = _ptr(projected)
        ph, kh = _ptr(hits)
        pi, ki = _ptr(ids)
        pd, kd = _ptr(dists)
        _check(load_library().rte_search_projected(self._h, pp, ph, nq, ctypes.byref(params), pi,
                                                   pd, _stream_ptr(stream)))
        return ids, dists

    def counters(self, projected, hits=None, params: SearchParams | None = None, **kw):
        """Per-query [entries_valid, expanded, dist_evals, iterations]."""
        params = self._params(params, kw)
        projected = _as(projected, np.float32, "float32")
        nq = projected.shape[0]
        out = np.empty((nq, 4), np.int64)
        if hits is not None:
            hits = _as(hits, np.int32, "int32")
        pp, kp = _ptr(projected)
        ph, kh = _ptr(hits)
        po, ko = _ptr(out)
        _check(load_library().rte_search_counters(self._h, pp, ph, nq, ctypes.byref(params), po,
                                                  None))
        return out

    # ---- artifacts --------------------------------------------------------
    def pca(self):
        inf = self.info
        d = inf.dim
        mean = np.empty(d, np.float32)
        rot = np.empty((d, d), np.float32)
        ev = np.empty(d, np.float64)
        _check(load_library().rte_get_pca(self._h, mean.ctypes.data_as(ctypes.c_void_p),
                                          rot.ctypes.data_as(ctypes.c_void_p),
                                          ev.ctypes.data_as(ctypes.c_void_p)))
        return mean, rot, ev

    def search_base(self):
        inf = self.info
        out = np.empty((inf.np, inf.search_dim), np.float32)
        _check(load_library().rte_get_search_base(self._h, out.ctypes.data_as(ctypes.c_void_p)))
        return out

    def search_base_lowp(self, precision: int):
        """Search-space base as the BF16 (1) / FP8 (2) path computes with it."""
        inf = self.info
        out = np.empty((inf.np, inf.search_dim), np.float32)
        _check(load_library().rte_get_search_base_lowp(self._h, precision,
                                                       out.ctypes.data_as(ctypes.c_void_p)))
        return out

    def kdtree(self):
        inf = self.info
        t = np.empty((inf.n_leaves, 6), np.float32)
        e = np.empty((inf.n_leaves, 6), np.float32)
        p = np.empty((inf.n_leaves, inf.leaf_size), np.int32)
        _check(load_library().rte_get_kdtree(self._h, t.ctypes.data_as(ctypes.c_void_p),
                                             e.ctypes.data_as(ctypes.c_void_p),
                                             p.ctypes.data_as(ctypes.c_void_p)))
        return t, e, p

    def train_learned(self, train_queries, **kw) -> dict:
        """Train the learned-entry MLP on raw training queries; returns the report."""
        p = TrainParams()
        load_library().rte_default_train_params(ctypes.byref(p))
        for k, v in kw.items():
            if not hasattr(p, k):
                raise TypeError(f"unknown training parameter {k}")
            setattr(p, k, v)
        tq = _as(train_queries, np.float32, "float32")
        pq, kq = _ptr(tq)
        rep = TrainReport()
        _check(load_library().rte_learned_train(self._h, pq, tq.shape[0], ctypes.byref(p),
                                                ctypes.byref(rep)))
        return rep.as_dict()

    def learned_leaves(self, projected, stream=None):
        projected = _as(projected, np.float32, "float32")
        out = _empty_like_kind(projected, (projected.shape[0],), np.int32, "int32")
        pp, kp = _ptr(projected)
        po, ko = _ptr(out)
        _check(load_library().rte_learned_predict(self._h, pp, projected.shape[0], po,
                                                  _stream_ptr(stream)))
        return out

    def autotune(self, queries, gt, k: int, target_recall: float = 0.95, **base):
        """Fastest (beam, width, bloom, warps/block) reaching the recall target."""
        p = default_params(**base)
        q = _as(queries, np.float32, "float32")
        g = np.ascontiguousarray(gt, np.int32)
        pq, kq = _ptr(q)
        rep = AutotuneReport()
        _check(load_library().rte_autotune(self._h, pq, q.shape[0], g.ctypes.data_as(ctypes.c_void_p),
                                           g.shape[1], k, target_recall, ctypes.byref(p),
                                           ctypes.byref(rep)))
        return p, rep.as_dict()

    def batcher(self, max_nq: int, params: SearchParams | None = None, **kw) -> "Batcher":
        return Batcher(self, max_nq, self._params(params, kw))

    def save(self, path: str):
        _check(load_library().rte_index_save(self._h, path.encode()))


class Batcher:
    """CUDA-graph replay of the whole query path for batches of <= max_nq."""

    def __init__(self, index: Index, max_nq: int, params: SearchParams):
        self.index = index
        self._h = ctypes.c_void_p()
        _check(load_library().rte_batcher_create(index._h, max_nq, ctypes.byref(params),
                                                 ctypes.byref(self._h)))
        self.k = load_library().rte_batcher_k(self._h)

    def search(self, queries, out_ids=None, out_dists=None, stream=None):
        q = _as(queries, np.float32, "float32")
        nq = q.shape[0]
        if out_ids is None:
            out_ids = _empty_like_kind(q, (nq, self.k), np.int32, "int32")
        if out_dists is None:
            out_dists = _empty_like_kind(q, (nq, self.k), np.float32, "float32")
        pq, kq = _ptr(q)
        pi, ki = _ptr(out_ids)
        pd, kd = _ptr(out_dists)
        _check(load_library().rte_batcher_search(self._h, pq, nq, pi, pd, _stream_ptr(stream)))
        return out_ids, out_dists

    def close(self):
        if getattr(self, "_h", None):
            load_library().rte_batcher_free(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
