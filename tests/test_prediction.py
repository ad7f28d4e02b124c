"""approximate_predict: the oracle and the library's hierarchy math against the reference's own
prediction fixture (crates/hdbscan/tests/fixtures/hdbscan_prediction.json, copied to
tests/golden/), then, on the GPU, the full prediction (device candidate search + hierarchy)
against the fixture's fitted models and against the oracle on fitted blobs.

Labels and connecting points are compared exactly; strengths to rel 1e-5 against the fixture
(the tolerance of crates/hdbscan-core/tests/prediction.rs:581-587, whose expected values come
from the original f64 ``hdbscan`` package) and bit for bit against the oracle.
"""
from __future__ import annotations

import json
import math
import warnings
from pathlib import Path

import numpy as np
import pytest

from cuscan_gb300 import synthetic
from cuscan_gb300.prediction import NO_CLUSTER_WARNING, Predictor
from oracle import oracle as O

FIXTURE = json.loads((Path(__file__).parent / "golden" / "hdbscan_prediction.json").read_text())


def fl(v):
    if isinstance(v, str):
        return {"inf": math.inf, "-inf": -math.inf, "nan": math.nan}[v]
    return float(v)


def floats(seq):
    return np.array([fl(v) for v in seq], np.float64)


def tree_of(raw):
    t = np.empty(len(raw["parent"]), dtype=[("parent", np.int64), ("child", np.int64),
                                              ("lambda_val", np.float64),
                                              ("child_size", np.float64)])
    t["parent"] = raw["parent"]
    t["child"] = raw["child"]
    t["lambda_val"] = np.array(floats(raw["lambda_val"]), np.float32)
    t["child_size"] = np.array(floats(raw["child_size"]), np.float32)
    return t


def assert_rel(actual, expected):
    tol = 1e-6 + 1e-5 * np.abs(expected)
    assert np.all(np.abs(np.asarray(actual) - expected) <= tol), (actual, expected)


def controlled_cases():
    trees = FIXTURE["controlled"]["trees"]
    for q in FIXTURE["controlled"]["queries"]:
        spec = trees[q["tree"]]
        yield q["name"], spec, q


def fitted_cases():
    for case in FIXTURE["fitted"]:
        yield case["id"], case


@pytest.mark.parametrize("name,spec,query", list(controlled_cases()),
                         ids=[c[0] for c in controlled_cases()])
def test_controlled_queries(name, spec, query):
    labels = np.array(spec["labels"], np.int32)
    fi = np.arange(labels.shape[0], dtype=np.uint32)
    tree = tree_of(spec["raw_tree"])
    ids = np.array([query["indices"]], np.int32)
    dist = floats(query["distances"])[None, :]
    cores = floats(query["core_distances"])
    s = int(query["min_samples"])
    exp = query["expected"]
    ol, os_, oc, _ = O.predict_candidates(tree, labels, fi, s, cores, ids, dist)
    p = Predictor(condensed_tree=tree, labels=labels, finite_index=fi, min_samples=s,
                  n_features=1, prediction_core=cores)
    pl, ps, pc = p.predict_candidates(ids, dist)
    for lab, st, conn in ((ol, os_, oc), (pl, ps, pc)):
        assert int(lab[0]) == exp["label"], name
        assert int(conn[0]) == exp["neighbor"], name
        assert_rel(st, np.array([fl(exp["strength"])]))
    assert ps.view(np.uint64)[0] == os_.view(np.uint64)[0]


@pytest.mark.parametrize("cid,case", list(fitted_cases()), ids=[c[0] for c in fitted_cases()])
def test_fitted_models_from_fixture_candidates(cid, case):
    labels = np.array(case["labels_compact"], np.int32)
    compact = np.arange(labels.shape[0], dtype=np.uint32)
    tree = tree_of(case["raw_tree"])
    s = int(case["resolved_min_samples"])
    exp = case["expected"]
    cores = floats(case["prediction_core_distances"])
    p = Predictor(condensed_tree=tree, labels=labels, finite_index=compact, min_samples=s,
                  n_features=len(case["train_float32"][0]), prediction_core=cores)
    assert p.no_cluster_tree == case["no_cluster_tree"]
    if case["no_cluster_tree"]:
        assert all(v == -1 for v in exp["labels"])
        return
    ids = np.array(case["candidate_indices_compact"], np.int32)
    dist = np.array([floats(r) for r in case["candidate_distances"]])
    ol, os_, oc, _ = O.predict_candidates(tree, labels, compact, s, cores, ids, dist)
    pl, ps, pc = p.predict_candidates(ids, dist)
    np.testing.assert_array_equal(ol, exp["labels"])
    np.testing.assert_array_equal(oc, exp["connecting_points_compact"])
    assert_rel(os_, floats(exp["strengths"]))
    np.testing.assert_array_equal(pl, ol)
    np.testing.assert_array_equal(pc, oc)
    np.testing.assert_array_equal(ps.view(np.uint64), os_.view(np.uint64))


def test_oracle_cores_match_the_fixture():
    core = FIXTURE["core_rank"]
    train = np.array([floats(r) for r in core["train"]], np.float32)
    s = int(core["min_samples"])
    assert_rel(O.prediction_cores(train, s), floats(core["prediction_core_inclusive_self"]))
    q = floats(core["query_candidate_distances"])
    assert q[s] == fl(core["query_core"])
    for cid, case in fitted_cases():
        if case["no_cluster_tree"]:
            continue
        fi = np.array(case["finite_index"], np.int64)
        raw = np.array([floats(r) for r in case["train_float32"]], np.float32)
        train = raw if raw.shape[0] == fi.shape[0] else raw[fi]
        assert_rel(O.prediction_cores(train, int(case["resolved_min_samples"])),
                   floats(case["prediction_core_distances"]))


def test_hierarchy_validation_errors():
    labels = np.array([0, 0, 0, 1, 1, 1], np.int32)
    fi = np.arange(6, dtype=np.uint32)
    rows = [(6, 7, 1.0, 3.0), (6, 8, 1.0, 3.0)] + [(7, i, 2.0, 1.0) for i in range(3)] + \
           [(8, i, 2.0, 1.0) for i in range(3, 6)]
    t = np.array(rows, dtype=[("parent", np.int64), ("child", np.int64),
                              ("lambda_val", np.float64), ("child_size", np.float64)])
    cores = np.zeros(6)
    p = Predictor(condensed_tree=t, labels=labels, finite_index=fi, min_samples=3,
                  n_features=1, prediction_core=cores)
    assert not p.no_cluster_tree
    with pytest.raises(ValueError, match="2\\*min_samples"):
        Predictor(condensed_tree=t, labels=labels, finite_index=fi, min_samples=4,
                  n_features=1, prediction_core=cores)
    bad = t.copy()
    bad["child"][2] = 1                     # point 1 attached twice
    with pytest.raises(ValueError, match="more than one condensed tree row"):
        Predictor(condensed_tree=bad, labels=labels, finite_index=fi, min_samples=1,
                  n_features=1, prediction_core=cores)
    bad = t.copy()
    bad["parent"][0] = 2                    # a point id as a parent
    with pytest.raises(ValueError, match="as a parent"):
        Predictor(condensed_tree=bad, labels=labels, finite_index=fi, min_samples=1,
                  n_features=1, prediction_core=cores)
    with pytest.raises(RuntimeError, match="invalid prediction core"):
        Predictor(condensed_tree=t, labels=labels, finite_index=fi, min_samples=1,
                  n_features=1, prediction_core=np.array([0, 0, -1.0, 0, 0, 0]))
    with pytest.raises(ValueError, match="invalid fitted label"):
        Predictor(condensed_tree=t, labels=np.array([0, 0, 0, 1, 1, -2], np.int32),
                  finite_index=fi, min_samples=1, n_features=1, prediction_core=cores)


# ---------------------------------------------------------------- GPU ----------------------

@pytest.mark.gpu
@pytest.mark.parametrize("cid,case", list(fitted_cases()), ids=[c[0] for c in fitted_cases()])
def test_device_prediction_matches_fixture(cid, case):
    """Device search + cores on the fixture's training rows and queries."""
    import cuscan_gb300 as cg
    labels = np.array(case["labels_compact"], np.int32)
    compact = np.arange(labels.shape[0], dtype=np.uint32)
    fi = np.array(case["finite_index"], np.int64)
    raw = np.array([floats(r) for r in case["train_float32"]], np.float32)
    train = raw if raw.shape[0] == fi.shape[0] else raw[fi]
    queries = np.array([floats(r) for r in case["queries_float32"]], np.float32)
    s = int(case["resolved_min_samples"])
    tree = tree_of(case["raw_tree"])
    p = Predictor(condensed_tree=tree, labels=labels, finite_index=compact, min_samples=s,
                  n_features=train.shape[1], train=train, context=cg.context(0))
    exp = case["expected"]
    if case["no_cluster_tree"]:
        assert p.no_cluster_tree
        return
    assert_rel(p.cores(), floats(case["prediction_core_distances"]))
    lab, st, conn = p.predict(queries)
    np.testing.assert_array_equal(lab, exp["labels"])
    # the fixture's candidate order among exact ties comes from the original package's search;
    # the reference exempts the connector identity of those queries (and only that):
    # python/tests/test_hdbscan_prediction.py:263-270
    sensitive = {t["query"] for t in case["tie_annotations"] if t["connector_order_sensitive"]}
    stable = [i for i in range(len(queries)) if i not in sensitive]
    np.testing.assert_array_equal(conn[stable],
                                  np.asarray(exp["connecting_points_compact"])[stable])
    assert_rel(st, floats(exp["strengths"]))
    ol, os_, oc, _ = O.approximate_predict(tree, labels, compact, s, train, queries)
    np.testing.assert_array_equal(lab, ol)
    np.testing.assert_array_equal(conn, oc)
    np.testing.assert_array_equal(st.view(np.uint64), os_.view(np.uint64))


@pytest.mark.gpu
@pytest.mark.parametrize("n,d,blobs,ms,prec", [(3000, 8, 6, 5, "fp32"), (12000, 32, 20, 10,
                                                                           "bf16_refined"),
                                               (20000, 64, 40, 10, "fp16_refined")])
def test_estimator_approximate_predict_matches_oracle(n, d, blobs, ms, prec):
    import cuscan_gb300 as cg
    x = synthetic.gaussian_mixture(n, d, blobs, seed=n + d)
    x[7, 0] = np.nan                                   # a non-finite training row
    model = cg.HDBSCAN(min_cluster_size=max(5, n // 200), min_samples=ms, precision=prec).fit(x)
    q = synthetic.gaussian_mixture(777, d, blobs, seed=n + d)[:777] + np.float32(0.01)
    lab, st, conn = model.approximate_predict(q, return_connecting_points=True)
    fi = model.finite_index_
    tree = model.condensed_tree_
    cores = O.prediction_cores(x[fi], ms)
    pred = model.to_predictor()._predictor
    np.testing.assert_array_equal(pred.cores().view(np.uint64), cores.view(np.uint64))
    ol, os_, oc, _ = O.approximate_predict(tree, model.labels_, fi, ms, x[fi], q, cores=cores)
    np.testing.assert_array_equal(lab, ol)
    np.testing.assert_array_equal(conn, oc)
    np.testing.assert_array_equal(st.view(np.uint64), os_.view(np.uint64))
    assert lab.dtype == np.intp and st.dtype == np.float64
    assert len(set(lab.tolist()) - {-1}) >= 2
    # cores computed on the device equal those derived from the fit's kNN rows
    dev = Predictor(condensed_tree=tree, labels=model.labels_, finite_index=fi, min_samples=ms,
                    n_features=d, train=x[fi], context=cg.context(0))
    np.testing.assert_array_equal(dev.cores().view(np.uint64), cores.view(np.uint64))


@pytest.mark.gpu
def test_no_cluster_tree_predicts_noise_with_one_warning():
    import cuscan_gb300 as cg
    x = np.random.default_rng(0).uniform(size=(60, 3)).astype(np.float32)
    model = cg.HDBSCAN(min_cluster_size=60).fit(x)
    assert np.all(model.labels_ == -1)
    with warnings.catch_warnings(record=True) as w:
        warnings.simplefilter("always")
        lab, st, conn = model.approximate_predict(x[:5], return_connecting_points=True)
    assert [str(r.message) for r in w] == [NO_CLUSTER_WARNING]
    assert lab.tolist() == [-1] * 5 and st.tolist() == [0.0] * 5 and conn.tolist() == [-1] * 5


@pytest.mark.gpu
def test_approximate_predict_input_validation():
    import cuscan_gb300 as cg
    x = synthetic.gaussian_mixture(400, 4, 3, seed=1)
    model = cg.HDBSCAN(min_cluster_size=10).fit(x)
    with pytest.raises(ValueError, match="boolean"):
        model.approximate_predict(x[:3], return_connecting_points=1)
    with pytest.raises(ValueError, match="only finite"):
        model.approximate_predict(np.array([[np.nan, 0, 0, 0]], np.float32))
    with pytest.raises(ValueError, match="features"):
        model.approximate_predict(np.zeros((2, 3), np.float32))
    with pytest.raises(ValueError, match="at least one row"):
        model.approximate_predict(np.zeros((0, 4), np.float32))
    lab, st = model.approximate_predict(x[:10])
    assert lab.shape == (10,) and st.shape == (10,)
