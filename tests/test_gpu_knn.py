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
