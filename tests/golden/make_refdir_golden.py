"""A data directory as the reference's Graph leaves it, written by the
reference's own code, plus the same base in every vector format its readers
take.

    python tests/golden/make_refdir_golden.py

Runs oracle/_ref/refdir_main (built by oracle/ref/Makefile from the
reference's pca.cpp and kdtree.cpp, so it needs the reference tree: this
machine only) on a seeded 2000 x 32 integer-valued base.  It writes
mean.fbin and O.fbin through PCA::save_mean_rotation, pca_base.fbin through
PCA::save_result, and 32_0.aabbs in RT_Entry::write_aabbs' layout from the
reference's Kdtree.  This script adds the exact degree-32 graph (raw int32,
as file_read::read_graph reads it) and the base as .fvecs, .bvecs, .fbin,
.hvecs, .hh and .txt in the layouts file_read.cu reads.  Every file's bytes
are stored unchanged in tests/golden/refdir.npz (file i under `file<i>`,
names in `names`), with 200 queries of the same mixture.
"""
from __future__ import annotations

import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

N, D, R, LEAF, NQ = 2000, 32, 32, 32, 200


def data():
    rng = np.random.Generator(np.random.Philox(7101))
    cent = rng.uniform(30, 220, (10, D))
    x = cent[rng.integers(0, 10, N + NQ)] + 25 * rng.standard_normal((N + NQ, D))
    x = np.rint(np.clip(x, 0, 255)).astype(np.float32)
    return x[:N], x[N:]


def write_formats(base, t):
    n, d = base.shape
    hdr = np.full((n, 1), d, np.int32)
    with open(os.path.join(t, "base.fvecs"), "wb") as f:
        f.write(np.concatenate([hdr.view(np.float32), base], 1).tobytes())
    with open(os.path.join(t, "base.bvecs"), "wb") as f:
        for row in base.astype(np.uint8):
            f.write(np.int32(d).tobytes() + row.tobytes())
    with open(os.path.join(t, "base.fbin"), "wb") as f:
        f.write(np.array([n, d], np.int32).tobytes() + base.tobytes())
    for ext in ("hvecs", "hh"):
        with open(os.path.join(t, f"base.{ext}"), "wb") as f:
            f.write(np.int32(d).tobytes() + base.tobytes())
    with open(os.path.join(t, "base.txt"), "w") as f:
        f.write(f"{n} {d}\n")
        for row in base:
            f.write(",".join(f"{v:.9g}" for v in row) + "\n")


def main():
    import oracle
    from rt_entry_gb300 import datasets as ds
    if not oracle.build_reference():
        raise SystemExit("the reference tree is needed to make this fixture")
    base, queries = data()
    graph = ds.knn_graph(base, R, device="cpu").astype(np.int32)
    with tempfile.TemporaryDirectory() as t:
        inp = os.path.join(t, "in.bin")
        with open(inp, "wb") as f:
            f.write(np.int64(N).tobytes() + np.int64(D).tobytes() + base.tobytes())
        out = os.path.join(t, "dir")
        os.mkdir(out)
        subprocess.run([os.path.join(oracle.REF_OUT, "refdir_main"), inp, str(LEAF), out], check=True,
                       stdout=subprocess.DEVNULL)
        with open(os.path.join(out, "graph.int32"), "wb") as f:
            f.write(graph.tobytes())
        write_formats(base, out)
        names = sorted(os.listdir(out))
        blobs = {f"file{i}": np.frombuffer(open(os.path.join(out, nm), "rb").read(), np.uint8)
                 for i, nm in enumerate(names)}
    np.savez_compressed(os.path.join(HERE, "refdir.npz"), names=np.array(names), queries=queries,
                        leaf=np.int32(LEAF), **blobs)
    print("wrote", os.path.join(HERE, "refdir.npz"), names)


def materialise(dst):
    """Writes the stored files, byte for byte, into dst; returns the queries."""
    z = np.load(os.path.join(HERE, "refdir.npz"))
    for i, nm in enumerate(z["names"]):
        with open(os.path.join(dst, str(nm)), "wb") as f:
            f.write(z[f"file{i}"].tobytes())
    return z["queries"], int(z["leaf"])


if __name__ == "__main__":
    main()
