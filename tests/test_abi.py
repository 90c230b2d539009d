"""The C ABI: library loads, exports every declared symbol, rejects bad
arguments with a status (never exits), and its host-only build steps."""
import ctypes
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    txt = open(os.path.join(ROOT, "include", "rtentry.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(rte_[a-z0-9_]+)\s*\(", txt)))


def test_library_exports_every_declared_symbol(lib):
    syms = declared_symbols()
    assert len(syms) >= 20
    for s in syms:
        assert hasattr(lib, s), s
    import rt_entry_gb300 as r
    assert sorted(r.EXPORTS) == syms


def test_default_params(lib):
    import rt_entry_gb300 as r
    p = r.default_params()
    assert (p.k, p.beam, p.search_width, p.max_iter, p.bloom_words, p.bloom_hashes) == (10, 64, 1, 100, 512, 3)
    assert p.entry_mode == r.ENTRY_KDTREE and p.precision == r.PREC_FP32


def test_search_params_layout_matches_the_header(lib):
    """The ctypes struct has the header's fields in the header's order, and
    rte_default_params writes exactly that many bytes."""
    import ctypes
    import re

    import rt_entry_gb300 as r
    text = open(os.path.join(ROOT, "include", "rtentry.h")).read()
    body = re.search(r"typedef struct \{(.*?)\} rte_search_params;", text, re.S).group(1)
    body = re.sub(r"/\*.*?\*/", "", body, flags=re.S)
    fields = re.findall(r"\bint\s+(\w+)\s*;", body)
    assert fields == [f for f, _ in r.SearchParams._fields_]
    n = ctypes.sizeof(r.SearchParams)
    buf = (ctypes.c_ubyte * (n + 64))(*([0xA5] * (n + 64)))
    lib.rte_default_params(ctypes.cast(buf, ctypes.POINTER(r.SearchParams)))
    assert bytes(buf[n:]) == bytes([0xA5] * 64), "rte_default_params wrote past the struct"
    p = r.SearchParams.from_buffer_copy(bytes(buf[:n]))
    assert p.team_warps == 0 and p.max_hits == 1


def test_null_and_bad_arguments_return_status(lib):
    import rt_entry_gb300 as r
    h = ctypes.c_void_p()
    assert lib.rte_index_from_host(None, 10, 4, None, 32, 0, ctypes.byref(h)) == r.RTE_EINVAL
    base = np.zeros((100, 8), np.float32)
    g = np.zeros((100, 24), np.int32)  # degree not a power of two
    rc = lib.rte_index_from_host(base.ctypes.data_as(ctypes.c_void_p), 100, 8,
                                 g.ctypes.data_as(ctypes.c_void_p), 24, 0, ctypes.byref(h))
    assert rc == r.RTE_EINVAL
    assert b"power of two" in lib.rte_last_error()
    g = np.full((100, 32), 101, np.int32)  # id > np
    rc = lib.rte_index_from_host(base.ctypes.data_as(ctypes.c_void_p), 100, 8,
                                 g.ctypes.data_as(ctypes.c_void_p), 32, 0, ctypes.byref(h))
    assert rc == r.RTE_EINVAL
    assert lib.rte_index_load(b"/nonexistent/base.fvecs", b"/nonexistent/g", 0, ctypes.byref(h)) == r.RTE_EIO
    assert lib.rte_search(None, None, 0, None, None, None, None) == r.RTE_EINVAL
    # the learned head's entry point: NULL arguments, an unknown path and host
    # pointers (it takes device arrays) are rejected before any GPU work
    x = np.zeros((4, 8), np.uint16)
    b = np.zeros(64, np.float32)
    cols = np.zeros(4, np.int32)
    P = lambda a: a.ctypes.data_as(ctypes.c_void_p)
    assert lib.rte_mlp_head_argmax(None, 4, 8, None, None, None, None, None, None, 64, 8, 0, None,
                                   None) == r.RTE_EINVAL
    assert lib.rte_mlp_head_argmax(P(x), 4, 8, P(x), P(b), P(x), P(b), P(x), P(b), 64, 8, 2, P(cols),
                                   None) == r.RTE_EINVAL
    assert lib.rte_mlp_head_argmax(P(x), 4, 8, P(x), P(b), P(x), P(b), P(x), P(b), 64, 8, 0, P(cols),
                                   None) == r.RTE_EINVAL
    assert b"device pointers" in lib.rte_last_error()


def test_truncated_files_are_rejected(lib, tmp_path):
    import rt_entry_gb300 as r
    p = tmp_path / "b.fvecs"
    rec = np.concatenate([np.array([4], np.int32).view(np.uint8), np.arange(4, dtype=np.float32).view(np.uint8)])
    p.write_bytes(rec.tobytes() * 3 + rec.tobytes()[:7])
    g = tmp_path / "g.ibin"
    g.write_bytes(np.zeros((3, 32), np.int32).tobytes())
    h = ctypes.c_void_p()
    assert lib.rte_index_load(str(p).encode(), str(g).encode(), 0, ctypes.byref(h)) == r.RTE_EIO
    assert b"truncated" in lib.rte_last_error()
    p2 = tmp_path / "b.fbin"
    p2.write_bytes(np.array([5, 4], np.int32).tobytes() + np.zeros(19, np.float32).tobytes())
    assert lib.rte_index_load(str(p2).encode(), str(g).encode(), 0, ctypes.byref(h)) == r.RTE_EIO


def test_host_kdtree_matches_reference_golden(lib):
    """rte_kdtree_build_host == the reference's kdtree.cpp (fixture)."""
    import rt_entry_gb300 as r
    import oracle
    z = np.load(os.path.join(ROOT, "tests", "golden", "kdtree_ref.npz"))
    names = sorted(set(k.split("__")[0] for k in z.files))
    assert len(names) >= 5
    for n in names:
        pts, cap = z[n + "__pts"], int(z[n + "__cap"])
        t, e, p = r.kdtree_build_host(pts, cap, 0.2)
        assert np.array_equal(t, z[n + "__boxes"]), n
        assert np.array_equal(p, z[n + "__pids"]), n
        assert np.array_equal(e, oracle.expand_boxes(z[n + "__boxes"], 0.2)), n


def test_host_kdtree_rejects_degenerate_split(lib):
    import rt_entry_gb300 as r
    pts = np.zeros((100, 3), np.float32)  # every point equal: no split exists
    with pytest.raises(r.RteError) as ei:
        r.kdtree_build_host(pts, 32, 0.2)
    assert ei.value.status == r.RTE_EINVAL


def test_sym_eig_host_against_numpy_and_eigen_golden(lib):
    import rt_entry_gb300 as r
    rng = np.random.default_rng(3)
    for n in (3, 17, 128):
        a = rng.standard_normal((n, n))
        a = a @ a.T
        w, v = r.sym_eig_host(a)
        w2 = np.linalg.eigvalsh(a)[::-1]
        assert np.allclose(w, w2, rtol=1e-11, atol=1e-11 * w2[0])
        assert np.abs(a @ v - v * w).max() <= 1e-10 * w2[0]
        assert np.abs(v.T @ v - np.eye(n)).max() < 1e-12
        big = np.abs(v).argmax(axis=0)
        assert (v[big, np.arange(n)] > 0).all()
    z = np.load(os.path.join(ROOT, "tests", "golden", "pca_ref.npz"))
    x = z["x"].astype(np.float64)
    xc = x - x.mean(0)
    cov = xc.T @ xc / (x.shape[0] - 1)
    w, v = r.sym_eig_host(cov)
    assert np.allclose(w, z["eigvals"], rtol=1e-9, atol=1e-9 * w[0])
    ref = z["eigvecs"]
    # columns equal up to sign where the eigenvalue is well separated
    gaps = np.minimum(np.abs(np.diff(w, prepend=np.inf)), np.abs(np.diff(w, append=-np.inf)))
    for j in np.where(gaps > 1e-6 * w[0])[0]:
        s = np.sign(ref[:, j] @ v[:, j])
        assert np.abs(ref[:, j] * s - v[:, j]).max() < 1e-7, j
