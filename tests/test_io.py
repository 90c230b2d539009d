"""The reference's file formats on the host (no device): every vector
format file_read.cu reads gives the same base, and the data directory
written by the reference's own PCA code is self-consistent."""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))
import make_refdir_golden as refdir  # noqa: E402


def test_every_vector_format_reads_the_same_base(lib, tmp_path):
    import rt_entry_gb300 as r
    refdir.materialise(str(tmp_path))
    want = r.read_vectors(str(tmp_path / "base.fvecs"))
    assert want.shape == (refdir.N, refdir.D)
    for ext in ("bvecs", "fbin", "hvecs", "hh", "txt"):
        got = r.read_vectors(str(tmp_path / f"base.{ext}"))
        assert np.array_equal(got, want), ext
    base, _ = refdir.data()
    assert np.array_equal(want, base)


def test_reader_rejects_truncated_and_unknown_files(lib, tmp_path):
    import rt_entry_gb300 as r
    refdir.materialise(str(tmp_path))
    raw = (tmp_path / "base.fvecs").read_bytes()
    (tmp_path / "cut.fvecs").write_bytes(raw[:-3])
    (tmp_path / "cut.hvecs").write_bytes((tmp_path / "base.hvecs").read_bytes()[:-2])
    (tmp_path / "base.xyz").write_bytes(raw)
    for name in ("cut.fvecs", "cut.hvecs", "base.xyz", "missing.fbin"):
        try:
            r.read_vectors(str(tmp_path / name))
        except r.RteError as e:
            assert e.status in (r.RTE_EIO, r.RTE_EINVAL), name
        else:
            raise AssertionError(f"{name} was accepted")


def test_reference_pca_files_are_consistent(lib, tmp_path):
    """mean.fbin, O.fbin and pca_base.fbin as PCA::save_mean_rotation and
    PCA::save_result wrote them: pca_base = (base - mean) O to FP32
    rounding, O orthonormal."""
    import rt_entry_gb300 as r
    refdir.materialise(str(tmp_path))
    base = r.read_vectors(str(tmp_path / "base.fvecs")).astype(np.float64)
    mean = r.read_vectors(str(tmp_path / "mean.fbin"))
    O = r.read_vectors(str(tmp_path / "O.fbin")).astype(np.float64)
    pb = r.read_vectors(str(tmp_path / "pca_base.fbin"))
    assert mean.shape == (1, refdir.D) and O.shape == (refdir.D, refdir.D) and pb.shape == base.shape
    assert np.abs(O.T @ O - np.eye(refdir.D)).max() < 1e-5
    exact = (base - base.mean(0)) @ O
    assert np.abs(pb - exact).max() <= 1e-4 * np.abs(exact).max()
