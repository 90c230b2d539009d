"""The GPU exact kNN-graph builder (rte_knn_graph) against an FP64 brute
force on the host: identical rows, (distance, id) order, self excluded."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _mixture(n, d, integer, seed, k=16, spread=30.0):
    rng = np.random.Generator(np.random.Philox(seed))
    cent = rng.uniform(40, 215, (k, d))
    x = cent[rng.integers(0, k, n)] + spread * rng.standard_normal((n, d))
    x = np.clip(x, 0, 255)
    return (np.rint(x) if integer else x).astype(np.float32)


@pytest.mark.parametrize("integer,n,d,R", [(True, 6000, 128, 32), (False, 5000, 96, 64),
                                           (False, 2500, 960, 16), (True, 3000, 32, 64)])
def test_knn_graph_matches_fp64_brute_force(lib, cuda, integer, n, d, R):
    import rt_entry_gb300 as r
    from rt_entry_gb300 import datasets as ds
    base = _mixture(n, d, integer, seed=n + d + R)
    g = r.knn_graph(base, R)
    want = ds.knn_graph(base, R, device="cpu")
    assert g.shape == (n, R)
    assert np.array_equal(g, want), f"{(g != want).any(1).sum()} rows differ"


def test_knn_graph_device_io_and_duplicates(lib, cuda):
    """Device in, device out; duplicated rows (distance 0) order by id."""
    import torch
    import rt_entry_gb300 as r
    from rt_entry_gb300 import datasets as ds
    base = _mixture(2000, 64, True, seed=3)
    base[1000:1100] = base[:100]
    g = r.knn_graph(torch.from_numpy(base).cuda(), 24)
    assert isinstance(g, torch.Tensor) and g.is_cuda
    assert np.array_equal(g.cpu().numpy(), ds.knn_graph(base, 24, device="cpu"))
    with pytest.raises(r.RteError):
        r.knn_graph(base[:10], 10)  # degree must be below n


def test_knn_graph_on_offset_high_dim_data(lib, cuda):
    """Values in [0, 1] around 0.5 in 960 dimensions (the high-dimension
    configuration's data): certified from the centred rows."""
    import rt_entry_gb300 as r
    from rt_entry_gb300 import datasets as ds
    base = ds.make_config(3, n=3000, nq=10, with_graph=False, with_gt=False).base
    assert base.min() >= 0.0 and base.max() <= 1.0 and abs(float(base.mean()) - 0.5) < 0.1
    g = r.knn_graph(base, 64)
    assert np.array_equal(g, ds.knn_graph(base, 64, device="cpu"))


def test_knn_graph_retries_rows_with_many_equal_distances(lib, cuda, capfd, monkeypatch):
    """300 copies of one row: each has 299 neighbours at distance 0, more
    than the first pass's 2R + 32 candidates, so its R-th distance equals the
    left-out bound and it is redone with 1024 candidates from the same block
    of dot products."""
    import rt_entry_gb300 as r
    from rt_entry_gb300 import datasets as ds
    base = _mixture(4000, 64, True, seed=11)
    base[1000:1300] = base[1000]
    monkeypatch.setenv("RTE_KNN_VERBOSE", "1")
    g = r.knn_graph(base, 32)
    import re
    err = capfd.readouterr().err
    m = re.search(r"(\d+) rows retried", err)
    assert m and int(m.group(1)) >= 300, err
    assert np.array_equal(g, ds.knn_graph(base, 32, device="cpu"))
