"""Route parity at d <= 30.

The reference fits inputs of at least 256 rows and at most 30 features through its KD-tree
search by default (crates/hdbscan/src/estimator.rs:133-141) and requires that route to give the
brute-force route's neighbours, MST endpoints, labels and linkage
(crates/hdbscan/tests/test_estimator.rs:550-750, ``compare_search_routes``). This library has
one exact route, the brute-force semantics restated by the oracle, so matching the oracle
bit for bit on the reference's route-parity inputs is matching both reference routes.

The inputs are the reference's own closed-form route-parity sets (test_estimator.rs:714-749):
a 47 x 7 tie-free set and a 24 x 2 set of eight points repeated three times (ties), plus a
d = 10 blob set at the KD route's size (>= 256 rows).
"""
from __future__ import annotations

import numpy as np
import pytest

from oracle import oracle as O


def tie_free_rows():
    rows = np.empty((47, 7), np.float32)
    for r in range(47):
        for f in range(7):
            value = np.float32((r * 101 + f * 37 + r * f * 13) % 997)
            rows[r, f] = value / np.float32(31.0) + np.float32(f) * np.float32(0.017)
    return rows


def duplicate_rows():
    pts = [r % 8 for r in range(24)]
    return np.array([[p % 4, p // 4] for p in pts], np.float32)


def kd_sized_blobs():
    from cuscan_gb300 import synthetic
    return synthetic.gaussian_mixture(600, 10, blobs=4, std_range=(0.3, 1.0), seed=73)


CASES = [("tie_free_47x7", tie_free_rows, 4, 5, False),
         ("duplicates_24x2", duplicate_rows, 3, 4, True),
         ("blobs_600x10", kd_sized_blobs, 10, 5, False)]


def assert_tree_invariants(linkage, n):
    """test_estimator.rs:680-698: n-1 merges, children before parents, sizes add up, distances
    non-decreasing, the last merge holds every row."""
    assert linkage.shape[0] == max(n - 1, 0)
    sizes = np.ones(2 * n - 1, np.int64)
    for row, (left, right, dist, size) in enumerate(linkage):
        parent = n + row
        left, right = int(left), int(right)
        assert left < parent and right < parent and left != right
        assert int(size) == sizes[left] + sizes[right]
        sizes[parent] = int(size)
        if row > 0:
            assert linkage[row - 1, 2] <= dist
    if n > 0:
        assert sizes[n + linkage.shape[0] - 1] == n


@pytest.mark.parametrize("name,make,mcs,ms,tied", CASES, ids=[c[0] for c in CASES])
def test_oracle_seeded_weights_equal_independent_oracle(name, make, mcs, ms, tied):
    """The seeded production semantics and the singleton-start oracle agree on the MST weight
    multiset (the tie-robust check of test_estimator.rs:613-619)."""
    x = make()
    fc = O.fit_core(x, ms)
    _, _, w = O.brute_force_mst(x, ms)
    assert np.sort(fc.wsq).tobytes() == np.sort(w).tobytes()


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp32", "bf16_refined", "fp16_refined"])
@pytest.mark.parametrize("name,make,mcs,ms,tied", CASES, ids=[c[0] for c in CASES])
def test_route_parity_sets_match_oracle(name, make, mcs, ms, tied, precision):
    from cuscan_gb300 import HDBSCAN
    x = make()
    n = x.shape[0]
    model = HDBSCAN(min_cluster_size=mcs, min_samples=ms, precision=precision).fit(x)
    fc = O.fit_core(x, ms)
    k = min(ms, n - 1)
    neighbors = model.neighbors_
    assert neighbors.shape == (n, ms)
    assert (neighbors[:, :k] == fc.knn_ids).all(), "route neighbour ids"
    core = model.core_distances_
    assert core.tobytes() == np.sqrt(fc.core_sq).astype(np.float32).tobytes()
    mst = model.minimum_spanning_tree_
    exp = O.finalize_mst(fc.src, fc.dst, fc.wsq)
    assert mst.shape == exp.shape
    assert (mst[:, :2] == exp[:, :2]).all(), "MST endpoints"
    assert mst[:, 2].tobytes() == exp[:, 2].tobytes(), "MST weights"
    if tied:
        _, _, w = O.brute_force_mst(x, ms)
        oracle_w = np.sort(np.sqrt(w.astype(np.float64)))
        assert np.sort(mst[:, 2]).tobytes() == oracle_w.tobytes()
    assert_tree_invariants(model.single_linkage_tree_, n)
    again = HDBSCAN(min_cluster_size=mcs, min_samples=ms, precision="fp32").fit(x)
    assert (model.labels_ == again.labels_).all()
    assert model.single_linkage_tree_.tobytes() == again.single_linkage_tree_.tobytes()
    assert model.probabilities_.tobytes() == again.probabilities_.tobytes()
