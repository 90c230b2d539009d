"""The allocation-free search entry point, through the C ABI.

rte_search_projected_noalloc serves callers that cannot let the library
allocate device memory while they run (all buffers reserved up front, or an
allocator that owns the device).  Its output must equal the allocating entry
point's -- ids and distances bit for bit, the bar of every search test here --
on two calls in a row, since the second call reuses the scratch array the
first one left behind.  The second call must also allocate nothing: the
library's scratch pool (which its other entry points draw their per-call
buffers from) and the device's default pool record no use, and the free
device memory does not move.  The file sorts last so that a run stopping at the first failure has
already run every other test.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

_CU_MEMPOOL_ATTR_USED_MEM_CURRENT = 7  # CUmemPool_attribute, cuda.h
_CU_MEMPOOL_ATTR_USED_MEM_HIGH = 8


class _ScratchPool:
    """The library's own stream-ordered pool on one device, through
    rte_scratch_pool_usage."""

    def __init__(self, lib, ordinal=0):
        self.lib, self.dev = lib, ordinal
        lib.rte_scratch_pool_usage.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_uint64),
                                               ctypes.POINTER(ctypes.c_uint64), ctypes.c_int]
        lib.rte_scratch_pool_usage.restype = ctypes.c_int

    def _get(self, reset=0):
        now, high = ctypes.c_uint64(), ctypes.c_uint64()
        assert self.lib.rte_scratch_pool_usage(self.dev, ctypes.byref(now), ctypes.byref(high), reset) == 0
        return now.value, high.value

    def reset_used_high(self):
        self._get(reset=1)

    def used_now(self):
        return self._get()[0]

    def used_high(self):
        return self._get()[1]


class _DefaultPool:
    """The device's default memory pool through the driver API: the pool
    cudaMallocAsync draws from."""

    def __init__(self, ordinal=0):
        self.cu = ctypes.CDLL("libcuda.so.1")
        assert self.cu.cuInit(0) == 0
        dev = ctypes.c_int()
        assert self.cu.cuDeviceGet(ctypes.byref(dev), ordinal) == 0
        self.pool = ctypes.c_void_p()
        assert self.cu.cuDeviceGetDefaultMemPool(ctypes.byref(self.pool), dev) == 0

    def reset_used_high(self):
        zero = ctypes.c_uint64(0)
        assert self.cu.cuMemPoolSetAttribute(self.pool, _CU_MEMPOOL_ATTR_USED_MEM_HIGH,
                                             ctypes.byref(zero)) == 0

    def _get(self, attr):
        v = ctypes.c_uint64()
        assert self.cu.cuMemPoolGetAttribute(self.pool, attr, ctypes.byref(v)) == 0
        return v.value

    def used_now(self):
        return self._get(_CU_MEMPOOL_ATTR_USED_MEM_CURRENT)

    def used_high(self):
        return self._get(_CU_MEMPOOL_ATTR_USED_MEM_HIGH)


def _data(n=6000, nq=700, d=128, seed=21):
    rng = np.random.Generator(np.random.Philox(seed))
    cent = rng.uniform(40, 215, (16, d))
    x = cent[rng.integers(0, 16, n + nq)] + 45.0 * rng.standard_normal((n + nq, d))
    x = np.rint(np.clip(x, 0, 255)).astype(np.float32)
    return x[:n], x[n:]


def _noalloc(lib, idx, qp, hits, params, nq, ids, dd):
    import torch
    rc = lib.rte_search_projected_noalloc(idx._h, ctypes.c_void_p(qp.data_ptr()),
                                          None if hits is None else ctypes.c_void_p(hits.data_ptr()),
                                          nq, ctypes.byref(params), ctypes.c_void_p(ids.data_ptr()),
                                          ctypes.c_void_p(dd.data_ptr()), None)
    torch.cuda.synchronize()
    return rc, ids, dd


def test_noalloc_search_equals_allocating_search(lib, cuda):
    import torch

    import rt_entry_gb300 as r
    from rt_entry_gb300 import datasets as ds

    base, q = _data()
    graph = ds.knn_graph(base, 64)
    idx = r.Index.from_arrays(base, graph).build_pca().build_kdtree(32, 0.2)
    qp = idx.project(torch.from_numpy(q).cuda())
    nq = qp.shape[0]
    leaves = idx.locate(qp)  # caller-supplied entry leaves (device memory)
    pool = _DefaultPool(torch.cuda.current_device())
    scratch = _ScratchPool(lib, torch.cuda.current_device())
    for kw, hits in ((dict(beam=64, k=10), None),
                     (dict(beam=128, k=128, precision=r.PREC_BF16, rerank=1), None),
                     (dict(beam=32, k=16, entry_mode=r.ENTRY_RANDOM), None),
                     (dict(beam=32, k=10), leaves),
                     # one warp per query: the single-warp kernel and its tail helping
                     (dict(beam=32, k=10, precision=r.PREC_BF16, rerank=1, team_warps=1), None)):
        params = r.default_params(**kw)
        want_ids, want_d = idx.search_projected(qp, hits=hits, params=params)
        torch.cuda.synchronize()
        k = want_ids.shape[1]
        for call in range(2):  # the second call starts from the first call's scratch
            ids = torch.full((nq, k), -7, dtype=torch.int32, device="cuda")
            dd = torch.full((nq, k), float("nan"), dtype=torch.float32, device="cuda")
            torch.cuda.synchronize()
            if call == 1:
                free0 = torch.cuda.mem_get_info()[0]
                used0 = pool.used_now()
                pool.reset_used_high()
                sused0 = scratch.used_now()
                scratch.reset_used_high()
            rc, ids, dd = _noalloc(lib, idx, qp, hits, params, nq, ids, dd)
            assert rc == r.RTE_OK, lib.rte_last_error()
            assert torch.equal(ids, want_ids), (kw, call)
            assert torch.equal(dd, want_d), (kw, call)
            if call == 1:
                assert pool.used_high() <= used0, "the call drew memory from the default pool"
                assert scratch.used_high() <= sused0, "the call drew memory from the scratch pool"
                assert torch.cuda.mem_get_info()[0] == free0, "the call changed the free device memory"


def test_noalloc_large_batch_in_leaf_order(lib, cuda):
    """20,000 queries outnumber the resident warps, so both entry points take
    them in entry-leaf order (the order lives in the fixed scratch here):
    the same ids and distances as the allocating search, whose large batches
    are checked against the oracle, with the library's own leaves and with
    leaves the caller supplies."""
    import torch

    import rt_entry_gb300 as r
    from rt_entry_gb300 import datasets as ds

    base, q = _data(n=6000, nq=20000, seed=23)
    graph = ds.knn_graph(base, 64)
    idx = r.Index.from_arrays(base, graph).build_pca().build_kdtree(32, 0.2)
    qp = idx.project(torch.from_numpy(q).cuda())
    nq = qp.shape[0]
    leaves = idx.locate(qp)
    for kw, hits in ((dict(beam=32, k=10), None),
                     (dict(beam=16, k=10, precision=r.PREC_BF16, rerank=1), leaves)):
        params = r.default_params(**kw)
        want_ids, want_d = idx.search_projected(qp, hits=hits, params=params)
        ids = torch.full((nq, 10), -7, dtype=torch.int32, device="cuda")
        dd = torch.full((nq, 10), float("nan"), dtype=torch.float32, device="cuda")
        rc, ids, dd = _noalloc(lib, idx, qp, hits, params, nq, ids, dd)
        assert rc == r.RTE_OK, lib.rte_last_error()
        assert torch.equal(ids, want_ids), kw
        assert torch.equal(dd, want_d), kw


def test_noalloc_rejects_what_it_cannot_serve(lib, cuda):
    import torch

    import rt_entry_gb300 as r
    from rt_entry_gb300 import datasets as ds

    base, q = _data(n=3000, nq=10)
    idx = r.Index.from_arrays(base, ds.knn_graph(base, 64)).build_kdtree(32, 0.2)
    params = r.default_params(beam=64, k=10)
    out = torch.empty((10, 10), dtype=torch.int32, device="cuda")
    qd = torch.from_numpy(q).cuda()
    too_many = 65537
    rc = lib.rte_search_projected_noalloc(idx._h, ctypes.c_void_p(qd.data_ptr()), None, too_many,
                                          ctypes.byref(params), ctypes.c_void_p(out.data_ptr()), None,
                                          None)
    assert rc == r.RTE_EINVAL and b"at most 65536" in lib.rte_last_error()
    host_q = np.ascontiguousarray(q)
    rc = lib.rte_search_projected_noalloc(idx._h, host_q.ctypes.data_as(ctypes.c_void_p), None, 10,
                                          ctypes.byref(params), ctypes.c_void_p(out.data_ptr()), None,
                                          None)
    assert rc == r.RTE_EINVAL and b"device pointers" in lib.rte_last_error()
    # an empty batch still has its parameters checked, as rte_search_projected does
    bad = r.default_params(beam=64, k=10, bloom_words=100)
    for fn in (lib.rte_search_projected_noalloc, lib.rte_search_projected):
        rc = fn(idx._h, None, None, 0, ctypes.byref(bad), None, None, None)
        assert rc == r.RTE_EINVAL and b"bloom_words" in lib.rte_last_error()
