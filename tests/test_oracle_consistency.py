"""The oracle's production-semantics fit core (kNN seed, then Borůvka rounds) against its own
independent all-pairs Borůvka (crates/hdbscan-core/src/oracle.rs:70-168) on the edge cases
the GPU parity tests use: exact duplicates, integer lattices, identical rows, underflowing and
overflowing distances. Ties may give the two different trees, but every minimum spanning tree
of a graph has the same sorted multiset of edge weights, +inf edges included."""
from __future__ import annotations

import numpy as np
import pytest

from oracle import oracle as O
from tests.test_gpu_fit import refined_edge_sets


@pytest.mark.parametrize("name,x,ms", list(refined_edge_sets()),
                         ids=lambda v: v if isinstance(v, str) else "")
def test_seeded_mst_has_the_all_pairs_weight_multiset(name, x, ms):
    fc = O.fit_core(x, ms)
    _, _, w_all = O.brute_force_mst(x, ms)
    n = x.shape[0]
    assert fc.wsq.shape[0] == n - 1 == w_all.shape[0]
    np.testing.assert_array_equal(np.sort(fc.wsq).view(np.uint32) & 0x7fffffff,
                                  np.sort(w_all).view(np.uint32) & 0x7fffffff)
    # the f64 totals of the finalised trees (sqrt per edge) agree to the last bits of a sum
    t_seed = np.sqrt(fc.wsq.astype(np.float64)).sum()
    t_all = np.sqrt(w_all.astype(np.float64)).sum()
    assert (np.isinf(t_seed) and np.isinf(t_all)) or abs(t_seed - t_all) <= 1e-12 * max(t_all, 1)


def _tie_heavy_sets():
    rng = np.random.default_rng(5)
    yield "lattice", rng.integers(-3, 4, size=(333, 7)).astype(np.float32), 5
    yield "blobs", rng.normal(size=(517, 33)).astype(np.float32), 4
    dup = rng.normal(size=(40, 12)).astype(np.float32)
    yield "duplicates", np.repeat(dup, 9, axis=0), 6
    wide = rng.normal(size=(129, 130)).astype(np.float32) * np.float32(1e18)
    yield "overflowing", wide, 3


@pytest.mark.parametrize("name,x,ms", list(_tie_heavy_sets()),
                         ids=lambda v: v if isinstance(v, str) else "")
def test_blocked_loops_equal_row_at_a_time_loops(name, x, ms):
    """The blocked all-pairs loops give the row-at-a-time loops' outputs bit for bit: kNN rows,
    Borůvka candidates of a random component split, and the whole fit core."""
    n = x.shape[0]
    k = min(ms, n - 1)
    ids_a, d_a = O.exact_neighbors(x, x, k)
    ids_b, d_b = O.exact_neighbors(x, x, k, blocked=True)
    np.testing.assert_array_equal(ids_a, ids_b)
    np.testing.assert_array_equal(d_a.view(np.uint32), d_b.view(np.uint32))
    rng = np.random.default_rng(n)
    comps = rng.integers(0, 6, size=n).astype(np.int32)
    core = O.core_from_knn(d_a, ms)
    w_a, j_a = O.boruvka_candidates(x, core, comps)
    w_b, j_b = O.boruvka_candidates(x, core, comps, blocked=True)
    np.testing.assert_array_equal(j_a, j_b)
    np.testing.assert_array_equal(w_a.view(np.uint32), w_b.view(np.uint32))
    O.set_blocked(False)
    try:
        fa = O.fit_core(x, ms)
    finally:
        O.set_blocked(True)
    fb = O.fit_core(x, ms)
    for key in ("knn_ids", "src", "dst"):
        np.testing.assert_array_equal(getattr(fa, key), getattr(fb, key))
    for key in ("knn_sq", "core_sq", "wsq"):
        np.testing.assert_array_equal(getattr(fa, key).view(np.uint32),
                                      getattr(fb, key).view(np.uint32))
