"""The allocation-free search entry point, through the C ABI.

rte_search_projected_noalloc serves callers that cannot let the library
allocate device memory while they run (all buffers reserved up front, or an
allocator that owns the device).  Its output must equal the allocating entry
point's -- ids and distances bit for bit, the bar of every search test here --
on two calls in a row, since the second call reuses the scratch array the
first one left behind.  The file sorts last so that a run stopping at the
first failure has already run every other test.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _data(n=6000, nq=700, d=128, seed=21):
    rng = np.random.Generator(np.random.Philox(seed))
    cent = rng.uniform(40, 215, (16, d))
    x = cent[rng.integers(0, 16, n + nq)] + 45.0 * rng.standard_normal((n + nq, d))
    x = np.rint(np.clip(x, 0, 255)).astype(np.float32)
    return x[:n], x[n:]


def test_noalloc_search_equals_allocating_search(lib, cuda):
    import torch

    import rt_entry_gb300 as r
    from rt_entry_gb300 import datasets as ds

    base, q = _data()
    graph = ds.knn_graph(base, 64)
    idx = r.Index.from_arrays(base, graph).build_pca().build_kdtree(32, 0.2)
    qp = idx.project(torch.from_numpy(q).cuda())
    nq = qp.shape[0]
    for kw in (dict(beam=64, k=10), dict(beam=128, k=128, precision=r.PREC_BF16, rerank=1),
               dict(beam=32, k=16, entry_mode=r.ENTRY_RANDOM)):
        params = r.default_params(**kw)
        want_ids, want_d = idx.search_projected(qp, params=params)
        torch.cuda.synchronize()
        k = want_ids.shape[1]
        for _ in range(2):  # the second call starts from the first call's scratch
            ids = torch.full((nq, k), -7, dtype=torch.int32, device="cuda")
            dd = torch.full((nq, k), float("nan"), dtype=torch.float32, device="cuda")
            rc = lib.rte_search_projected_noalloc(idx._h, ctypes.c_void_p(qp.data_ptr()), None, nq,
                                                  ctypes.byref(params), ctypes.c_void_p(ids.data_ptr()),
                                                  ctypes.c_void_p(dd.data_ptr()), None)
            torch.cuda.synchronize()
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
