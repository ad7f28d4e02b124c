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
