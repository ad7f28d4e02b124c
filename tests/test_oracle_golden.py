"""Pin the CPU oracle to the reference's golden fixtures and known-answer tests.

The fixtures (tests/golden, copied from crates/hdbscan/tests/fixtures by make_golden.py) were
produced by fast_hdbscan 0.3.2; the reference checks its estimator against them with exact
MST endpoints and 1e-5 relative weights (crates/hdbscan/tests/test_estimator.rs:125-310).
"""
from __future__ import annotations

import numpy as np
import pytest

from oracle import oracle as O
from tests.conftest import load_case

ESTIMATOR_CASES = ["blobs_d2", "blobs_d10", "blobs_d50", "moons_leaf", "varying_density",
                   "single_cluster", "duplicates_ties", "mixed_nonfinite", "overflow_finite"]
EXTRA_CASES = ["persistence_equal", "selection_interactions", "two_finite", "padding",
               "n_below_min_samples"]


def finite_rows(case):
    x = case["input"]
    keep = np.isfinite(x).all(axis=1)
    return np.ascontiguousarray(x[keep]), keep


def close(a, b, rel=1e-5):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return np.all((a == b) | (np.abs(a - b) <= rel * np.maximum(np.abs(b), 1.0)))


@pytest.mark.parametrize("cid", ESTIMATOR_CASES + EXTRA_CASES)
def test_oracle_mst_matches_fixture(cid, manifest):
    meta = {c["id"]: c for c in manifest["cases"]}[cid]
    case = load_case(cid)
    x, keep = finite_rows(case)
    ms = meta["params"]["min_samples"]
    fc = O.fit_core(x, ms)
    mst = O.finalize_mst(fc.src, fc.dst, fc.wsq)
    expected = case["mst"]
    assert mst.shape == expected.shape
    assert close(mst[:, 2], expected[:, 2]), "MST weights"
    if cid == "duplicates_ties":
        # tie case: the reference pins its MST to the all-pairs oracle instead
        # (test_estimator.rs:159-187)
        bf = O.finalize_mst(*O.brute_force_mst(x, ms))
        np.testing.assert_array_equal(mst[:, :2], bf[:, :2])
        assert close(mst[:, 2], bf[:, 2])
    else:
        np.testing.assert_array_equal(mst[:, :2], expected[:, :2])
    core = np.sqrt(fc.core_sq)
    np.testing.assert_allclose(core, case["core_distances"], rtol=1e-6, atol=0)
    np.testing.assert_array_equal(np.flatnonzero(keep), case["finite_index"])


def test_fused_and_unfused_sums_agree_on_fixtures():
    # The reference's own host oracle sums unfused; on the fixture data both orders give the
    # same MST, which is what its tests pin.
    for cid in ESTIMATOR_CASES:
        x, _ = finite_rows(load_case(cid))
        if x.shape[0] < 2:
            continue
        a = O.pair_distances(x[:-1], x[1:], fused=True)
        b = O.pair_distances(x[:-1], x[1:], fused=False)
        assert np.max(np.abs(a.astype(np.float64) - b) / np.maximum(b, 1e-30)) < 1e-5


def test_knn_seed_known_answer():
    # crates/hdbscan-core/tests/mst_oracle.rs:10-32
    core = np.array([2.0, 2.0, 3.0], np.float32)
    nb = np.array([[-1, 1], [0, -1], [0, -1]], np.int32)
    ds = np.array([[np.inf, 1.0], [1.0, np.inf], [4.0, np.inf]], np.float32)
    src, dst, w, _ = O.init_from_knn(core, nb, ds)
    assert list(zip(src.tolist(), dst.tolist(), w.tolist())) == [(0, 1, 2.0), (2, 0, 4.0)]


def test_core_boundaries_and_infinite_mst():
    # mst_oracle.rs:96-124
    x = np.array([[0.0], [1.0], [3.0]], np.float32)
    for ms, expected in [(1, [0.0, 0.0, 0.0]), (2, [9.0, 4.0, 9.0])]:
        fc = O.fit_core(x, ms)
        np.testing.assert_array_equal(fc.core_sq, np.array(expected, np.float32))
    for ms in (3, 5):
        fc = O.fit_core(x, ms)
        assert np.all(np.isinf(fc.core_sq))
        mst = O.finalize_mst(fc.src, fc.dst, fc.wsq)
        assert mst.shape[0] == 2 and np.all(np.isinf(mst[:, 2]))


def test_duplicate_points_tie_by_index():
    # mst_oracle.rs:126-133
    x = np.array([[0.0], [0.0], [1.0], [2.0]], np.float32)
    ids, _ = O.exact_neighbors(x, x, 2)
    assert ids[0].tolist() == [1, 2]
    assert O.brute_force_mst(x, 2)[0].shape[0] == 3


def test_component_plan_golden():
    # mst_oracle.rs:135-146
    plan = O.component_plan(np.array([2, 1, 2, 0, 1, 1], np.int32), 2)
    assert plan.members.tolist() == [0, 2, 1, 4, 5, 3]
    assert plan.offsets.tolist() == [0, 2, 5, 6]
    assert plan.tile_starts.tolist() == [0, 2, 4, 5]
    assert plan.tile_ends.tolist() == [2, 4, 5, 6]
    assert plan.partial_offsets.tolist() == [0, 1, 3, 4]
    for labels in ([-1], [1], [0, 2]):
        with pytest.raises(O.OracleError):
            O.component_plan(np.array(labels, np.int32), 1)


def test_padding_and_offset_self_known_answer():
    # crates/cuscan-common/src/neighbors.rs:440-465
    q = np.array([[10.0], [20.0]], np.float32)
    r = np.array([[0.0], [10.0], [20.0]], np.float32)
    ids, d = O.exact_neighbors(q, r, 3, exclude_self=True, query_offset=1)
    assert ids.ravel().tolist() == [0, 2, 3, 1, 0, 3]
    np.testing.assert_array_equal(d.ravel(), np.array([100, 100, np.inf, 100, 400, np.inf],
                                                      np.float32))
    ids, d = O.exact_neighbors(np.zeros((1, 1), np.float32), np.zeros((1, 1), np.float32), 2)
    assert ids.ravel().tolist() == [1, 1] and np.all(np.isinf(d))


def test_overflow_tail_known_answer():
    # neighbors.rs:407-438: an f32::MAX query row overflows every distance to +inf; those
    # +inf rows still enter the list by id ahead of the (inf, nr) padding.
    query = (np.arange(701) % 17).astype(np.float32)
    query[700] = np.finfo(np.float32).max
    ref = ((np.arange(763) * 7) % 23).astype(np.float32)
    ref[12:713] = query
    ids, d = O.exact_neighbors(query[:, None], ref[:, None], 1300, exclude_self=True,
                               query_offset=12)
    assert ids[0, :2].tolist() == [0, 29] and d[0, :2].tolist() == [0.0, 0.0]
    assert 4.0 in d[0]
    row = ids[700]
    assert row[:2].tolist() == [0, 1] and 712 not in row
    assert np.all(row[:762] < 763) and np.all(row[762:] == 763) and np.all(np.isinf(d[700]))


def test_candidates_match_closed_form_cases():
    # crates/hdbscan/tests/test_candidates.rs:8-53 data, compared with a numpy restatement
    for n, comps in [(1, 1), (2, 2), (257, 2), (513, 7)]:
        i = np.arange(n)
        x = np.stack([((i * 17 + i // 7) % 97) * 0.125, ((i * 11) % 53) * 0.25,
                      (i % 13).astype(np.float64)], 1).astype(np.float32)
        core = ((i % 9) * 0.125).astype(np.float32)
        comp = ((i * 7 + i // 19) % comps).astype(np.int32)
        w, dst = O.boruvka_candidates(x, core, comp)
        d2 = ((x[:, None, :].astype(np.float64) - x[None, :, :]) ** 2).sum(-1)  # exact here
        wt = np.maximum(np.maximum(d2, core[:, None]), core[None, :])
        wt[comp[:, None] == comp[None, :]] = np.inf
        exp_dst = np.where(np.isinf(wt).all(1), n, np.argmin(wt, 1))
        exp_w = np.where(np.isinf(wt).all(1), np.inf, wt.min(1)).astype(np.float32)
        np.testing.assert_array_equal(w, exp_w)
        np.testing.assert_array_equal(dst, exp_dst)


def test_component_reduce_semantics():
    # -0 canonicalisation, +inf real edges, earliest bad row (component_reduce.rs:61-76,
    # 317-353; mst_oracle.rs:163-242)
    labels = np.array([3, 1, 3, 1], np.int32)
    plan = O.component_plan(labels, 2)
    w = np.array([-0.0, 5.0, 0.0, np.inf], np.float32)
    dst = np.array([1, 0, 1, 2], np.int32)
    ww, wm = O.component_reduce(w, dst, plan)
    assert wm[0].tolist() == [0, 1, 4, 0, -1] and np.signbit(ww[0])
    assert wm[1].tolist() == [1, 0, 4, 0, -1] and ww[1] == 5.0
    w2 = np.array([np.nan, 1.0, 2.0, 1.0], np.float32)
    dst2 = np.array([1, 9, 1, 0], np.int32)
    ww, wm = O.component_reduce(w2, dst2, plan)
    assert wm[0].tolist() == [2, 1, 0, 1, -1]
    assert wm[1].tolist() == [3, 0, 1, 2, 9]
