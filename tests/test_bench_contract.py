"""bench.py's host-side pieces, without a GPU: the DRAM-traffic figures it
reads from the ncu summaries under profiles/, and the algorithmic-byte
count behind every roofline fraction."""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
import bench  # noqa: E402

# The arms whose roofline the default run reports, at the beams and widths
# the held-out selection picks on the seeded workloads.
KEYS = (
    "search_kernel/config2/bf16_rerank/learned/beam16/width1",
    "search_kernel/config2/fp32/kdtree/beam32/width1",
    "search_kernel/config1/plain_fp32/beam128/width2",
    "search_kernel/config1/learned_bf16/beam128/width2",
    "search_kernel/config3/plain_fp32/beam256/width4",
    "search_kernel/config3/bf16_rerank/beam256/width4",
    "search_kernel/config3/fp8_rerank/beam256/width4",
    "search_kernel/config4/plain_fp32/beam256/width4",
    "search_kernel/config4/learned_bf16/beam256/width4",
)


def test_profiled_traffic_covers_every_reported_arm():
    tr = bench.profiled_traffic()
    for k in KEYS:
        assert k in tr, k
        nbytes, source = tr[k]
        assert nbytes > 0 and source.startswith("ncu, "), (k, tr[k])
        # each source is a committed summary that gives its own command
        text = open(os.path.join(ROOT, "profiles", source[len("ncu, "):])).read()
        assert "ncu " in text and "--clock-control none" in text


def test_algorithmic_bytes_per_query():
    # B(q) = 4d + 4L + s*d*E + 4R*X + s*d*D + 8k (+ 4dL rerank), summed
    cnt = np.array([[3, 2, 10, 0], [1, 0, 4, 0]], np.int64)  # entries, expansions, distances
    d, L, R, k = 128, 16, 64, 10
    want = sum(4 * d + 4 * L + 2 * d * (e + dist) + 4 * R * x + 8 * k + 4 * d * L
               for e, x, dist, _ in cnt)
    got = bench.algorithmic_bytes(cnt, d, L, R, k, elem_bytes=2, rerank=True)
    assert got == want
    # FP8 rows carry a 4-byte scale each
    got8 = bench.algorithmic_bytes(cnt, d, L, R, k, elem_bytes=1, rerank=False, scale_bytes=4)
    want8 = sum(4 * d + 4 * L + (d + 4) * (e + dist) + 4 * R * x + 8 * k for e, x, dist, _ in cnt)
    assert got8 == want8
