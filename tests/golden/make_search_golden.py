"""Golden vectors for the beam search, pinned to the reference's own kernel.

Three steps:
  python tests/golden/make_search_golden.py inputs
      (any machine) writes tests/golden/search_<case>.npz with the inputs:
      base / queries (exactly representable integers or sixteenths stored
      as int16), the exact kNN graph, the kd-tree leaf table and the hits.
  python tests/golden/make_search_golden.py reference <outdir>
      (a machine with a GB300 and the cubins oracle/_ref/graph_search_d*.cubin
      compiled from the reference's graph_search.cuh by oracle/ref/Makefile)
      runs the reference GraphSearchKernel through oracle/ref_launch.cpp and
      writes <outdir>/search_<case>_ref.npy (the returned ids, topk = beam so
      the whole final pool is pinned), and for the kd-tree cases
      <outdir>/search_<case>_ref_scrub.npy from one launch per query on
      zeroed shared memory (the reference never clears its bloom filter).
  python tests/golden/make_search_golden.py merge <outdir>
      stores those ids as `ref_ids` inside each fixture.
"""
from __future__ import annotations

import ctypes
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

# name, dim, values, n, nq, degree, beam, max_iter, algo (1 kd-tree, 0 random)
CASES = [
    ("int_d32_r32_l64", 32, "int", 2000, 200, 32, 64, 100, 1),
    ("frac_d64_r64_l32", 64, "frac", 2000, 200, 64, 32, 100, 1),
    ("int_d128_r64_l128", 128, "int", 2000, 150, 64, 128, 100, 1),
    ("frac_d96_r32_l64_random", 96, "frac", 2000, 150, 32, 64, 60, 0),
    ("frac_d128_r32_l256", 128, "frac", 2000, 100, 32, 256, 100, 1),
]
LEAF = 32
EXPAND = 0.2


def path_of(name):
    return os.path.join(HERE, f"search_{name}.npz")


def load_case(name):
    z = np.load(path_of(name))
    scale = float(z["scale"])
    out = {k: z[k] for k in z.files}
    out["base"] = z["base_q"].astype(np.float32) * np.float32(scale)
    out["queries"] = z["queries_q"].astype(np.float32) * np.float32(scale)
    return out


def make_inputs():
    import oracle
    from rt_entry_gb300 import datasets as ds
    for i, (name, d, kind, n, nq, R, L, max_iter, algo) in enumerate(CASES):
        rng = np.random.Generator(np.random.Philox(5000 + i))
        k = 16
        cent = rng.uniform(40, 215, (k, d))
        lab = rng.integers(0, k, n + nq)
        x = cent[lab] + 45.0 * rng.standard_normal((n + nq, d))
        if kind == "int":
            xq = np.rint(np.clip(x, 0, 255)).astype(np.int16)
            scale = 1.0
        else:
            xq = np.rint(np.clip(x, 0, 255) * 16).astype(np.int16)
            scale = 1.0 / 16
        xs = xq.astype(np.float32) * np.float32(scale)
        base, queries = xs[:n], xs[n:]
        graph = ds.knn_graph(base, R, device="cpu")
        boxes, pids = oracle.kdtree_build(base[:, :3], LEAF)
        hits = oracle.locate(oracle.expand_boxes(boxes, EXPAND), queries[:, :3])
        np.savez_compressed(path_of(name), base_q=xq[:n], queries_q=xq[n:], scale=np.float64(scale),
                            graph=graph.astype(np.int32), leaf_pids=pids, hits=hits,
                            degree=R, beam=L, max_iter=max_iter, algo=algo, leaf=LEAF,
                            expand_ratio=np.float32(EXPAND))
        print("wrote", path_of(name))


def entries_table(leaf_pids, L, np_):
    """aabb_entries [n_leaves x L] (entry.cu:60-69)."""
    nl, cap = leaf_pids.shape
    t = np.full((nl, L), np_, np.int32)
    m = min(cap, L)
    t[:, :m] = leaf_pids[:, :m]
    return t


def run_reference(outdir, scrub=False):
    """scrub: per-query launches on scrubbed shared memory (kd-tree cases),
    so the reference's uninitialised bloom filter starts empty."""
    import oracle
    lib_path = oracle.build_ref_launcher()
    lib = ctypes.CDLL(lib_path)
    lib.ref_last_error.restype = ctypes.c_char_p
    P = ctypes.c_void_p
    I = ctypes.c_int
    lib.ref_graph_search.argtypes = [ctypes.c_char_p, P, I, I, P, I, P, I, P, I, I, P, I, I, I, I, I,
                                     P]
    lib.ref_graph_search.restype = I
    os.makedirs(outdir, exist_ok=True)
    for name, d, *_ in CASES:
        c = load_case(name)
        base, q, graph = c["base"], c["queries"], c["graph"]
        L = int(c["beam"])
        ent = entries_table(c["leaf_pids"], L, base.shape[0])
        hits = c["hits"].astype(np.int32)
        if scrub and int(c["algo"]) != 1:
            continue
        out = np.empty((q.shape[0], L), np.int32)
        cubin = os.path.join(oracle.REF_OUT, f"graph_search_d{d}.cubin")
        rc = lib.ref_graph_search(cubin.encode(), base.ctypes.data, base.shape[0], d, q.ctypes.data,
                                  q.shape[0], graph.ctypes.data, graph.shape[1], ent.ctypes.data,
                                  ent.shape[0], L, hits.ctypes.data, L, 1, int(c["max_iter"]),
                                  int(c["algo"]), int(scrub), out.ctypes.data)
        if rc != 0:
            raise RuntimeError(f"{name}: {lib.ref_last_error().decode()}")
        np.save(os.path.join(outdir, f"search_{name}_ref{'_scrub' if scrub else ''}.npy"), out)
        print("reference ran", name)


def merge(outdir):
    for name, *_ in CASES:
        ref = np.load(os.path.join(outdir, f"search_{name}_ref.npy"))
        z = dict(np.load(path_of(name)))
        z["ref_ids"] = ref.astype(np.int32)
        sp = os.path.join(outdir, f"search_{name}_ref_scrub.npy")
        if os.path.exists(sp):
            z["ref_ids_scrub"] = np.load(sp).astype(np.int32)
        np.savez_compressed(path_of(name), **z)
        print("merged", name)


if __name__ == "__main__":
    cmd = sys.argv[1]
    if cmd == "inputs":
        make_inputs()
    elif cmd == "reference":
        run_reference(sys.argv[2])
        run_reference(sys.argv[2], scrub=True)
    elif cmd == "merge":
        merge(sys.argv[2])
    else:
        raise SystemExit(__doc__)
