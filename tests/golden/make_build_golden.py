"""Golden vectors for the build side, produced by the reference's own code.

Runs the reference's kdtree.cpp (leaves, tight boxes, leaf point ids) and
pca.cpp with its vendored Eigen (mean, eigenvalues, eigenvectors, projected
base), both compiled from the reference sources by oracle/ref/Makefile, on
seeded inputs, and stores inputs and outputs in tests/golden/kdtree_ref.npz
and tests/golden/pca_ref.npz.  Needs the reference tree (this machine only);
the fixtures it writes are what the tests read everywhere else.

    python tests/golden/make_build_golden.py
"""
from __future__ import annotations

import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))


def kd_inputs():
    """Named 3-d point sets covering the split rule's branches."""
    sets = {}
    r = np.random.Generator(np.random.Philox(7001))
    sets["gauss_5000_leaf32"] = (r.standard_normal((5000, 3)).astype(np.float32) * 40, 32)
    sets["uniform_3000_leaf16"] = (r.uniform(-1, 1, (3000, 3)).astype(np.float32), 16)
    # flat along z and integer-valued: ties at the split value, zero-width axis
    g = r.integers(0, 60, (4000, 3)).astype(np.float32)
    g[:, 2] = 7.0
    g += r.uniform(0, 1e-3, g.shape).astype(np.float32) * np.array([1, 1, 0], np.float32)
    sets["grid_flat_4000_leaf32"] = (g, 32)
    c = np.concatenate([r.standard_normal((700, 3)) * s + m for s, m in
                        ((0.5, 0), (3.0, 20), (0.01, -15), (8.0, 5))]).astype(np.float32)
    sets["clusters_2800_leaf20"] = (c, 20)
    sets["small_37_leaf32"] = (r.standard_normal((37, 3)).astype(np.float32), 32)
    sets["leaf_larger_than_beam_2000_leaf100"] = (r.standard_normal((2000, 3)).astype(np.float32), 100)
    return sets


def main():
    import oracle
    if not oracle.build_reference():
        raise SystemExit("the reference tree is needed to make these fixtures")
    out = {}
    with tempfile.TemporaryDirectory() as t:
        for name, (pts, cap) in kd_inputs().items():
            boxes, pids = oracle.ref_kdtree(pts, cap, t)
            out[f"{name}__pts"] = pts
            out[f"{name}__cap"] = np.int32(cap)
            out[f"{name}__boxes"] = boxes
            out[f"{name}__pids"] = pids
            print(name, boxes.shape)
        np.savez_compressed(os.path.join(HERE, "kdtree_ref.npz"), **out)
        # PCA on a small mixture (integers 0..255 like SIFT bvecs, 64-d)
        r = np.random.Generator(np.random.Philox(7002))
        cent = r.uniform(30, 220, (12, 64))
        x = np.rint(np.clip(cent[r.integers(0, 12, 3000)] + 30 * r.standard_normal((3000, 64)), 0, 255))
        x = x.astype(np.float32)
        mean, val, vec, proj = oracle.ref_pca(x, t)
        np.savez_compressed(os.path.join(HERE, "pca_ref.npz"), x=x.astype(np.uint8), mean=mean,
                            eigvals=val, eigvecs=vec, projected=proj)
        print("pca", vec.shape)


if __name__ == "__main__":
    main()
