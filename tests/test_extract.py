"""Host extraction of the library (labels, strengths, linkage, condensed tree) against the
reference fixtures, fed with the fixture MST and with the oracle's MST.

Tolerances are the reference's own (crates/hdbscan/tests/test_estimator.rs:140-265): labels and
linkage structure exact, probabilities within 1e-5, lambdas within 1e-5 relative.
"""
from __future__ import annotations

import numpy as np
import pytest

import cuscan_gb300 as cg
from cuscan_gb300.hdbscan import _remap_condensed, _remap_linkage
from oracle import oracle as O
from tests.conftest import load_case

CASES = ["blobs_d2", "blobs_d10", "blobs_d50", "moons_leaf", "varying_density",
         "single_cluster", "duplicates_ties", "mixed_nonfinite", "overflow_finite",
         "persistence_equal", "selection_interactions", "all_noise", "two_finite", "padding",
         "n_below_min_samples"]


def params(manifest, cid):
    return {c["id"]: c for c in manifest["cases"]}[cid]["params"]


def extract(mst, p):
    return cg.clusters_from_spanning_tree(
        mst[:, 0].astype(np.uint32), mst[:, 1].astype(np.uint32), mst[:, 2],
        min_cluster_size=p["min_cluster_size"], cluster_selection_method=p["selection"],
        allow_single_cluster=p["allow_single_cluster"], max_cluster_size=p["max_cluster_size"],
        cluster_selection_epsilon=float(p["epsilon"]),
        cluster_selection_persistence=float(p["persistence"]))


def leaves(node, parent, child, size, n_points):
    if node < n_points:
        return [node]
    out = []
    for i in np.flatnonzero(parent == node):
        c = int(child[i])
        out.extend(leaves(c, parent, child, size, n_points) if size[i] > 1.0 or c >= n_points
                   else [c])
    return sorted(out)


def canonical_condensed(parent, child, lam, size, n_points):
    """Rows as (leaves(parent), leaves(child) or [child], lambda, size), sorted — the
    reference's normalisation (test_estimator.rs:67-123)."""
    rows = []
    for i in range(parent.shape[0]):
        pl = leaves(int(parent[i]), parent, child, size, n_points)
        cl = leaves(int(child[i]), parent, child, size, n_points) if size[i] > 1.0 else [int(child[i])]
        rows.append((pl, cl, float(lam[i]), float(size[i])))
    rows.sort(key=lambda r: (r[0], r[1], r[2], r[3]))
    return rows


def close(a, b, rel=1e-5):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    with np.errstate(invalid="ignore"):
        return np.all((a == b) | (np.abs(a - b) <= rel * np.maximum(np.abs(b), 1.0)))


@pytest.mark.parametrize("source", ["fixture_mst", "oracle_mst"])
@pytest.mark.parametrize("cid", CASES)
def test_extraction_matches_fixture(cid, source, manifest):
    p = params(manifest, cid)
    case = load_case(cid)
    x = case["input"]
    keep = np.isfinite(x).all(axis=1)
    finite_index = np.flatnonzero(keep)
    outliers = np.flatnonzero(~keep)
    if source == "fixture_mst":
        mst = case["mst"]
    else:
        fc = O.fit_core(np.ascontiguousarray(x[keep]), p["min_samples"])
        mst = O.finalize_mst(fc.src, fc.dst, fc.wsq)
    tied = cid in ("duplicates_ties", "all_noise")
    r = extract(mst, p)
    labels = np.full(x.shape[0], -1, np.int64)
    labels[finite_index] = r["labels"]
    np.testing.assert_array_equal(labels, case["labels"], err_msg=f"{cid}: labels")
    prob = np.zeros(x.shape[0], np.float64)
    prob[finite_index] = r["probabilities"]
    assert np.all(np.abs(prob - case["probabilities"]) <= 1e-5), f"{cid}: probabilities"
    linkage = r["linkage"]
    cp, cc, cl, cs = (r["condensed_parent"], r["condensed_child"], r["condensed_lambda"],
                      r["condensed_child_size"])
    if outliers.size:
        linkage = _remap_linkage(linkage, finite_index, outliers)
        cp, cc, cl, cs = _remap_condensed(cp, cc, cl, cs, finite_index, outliers)
    exp_link = case.get("remapped_linkage", case["linkage"])
    assert linkage.shape == exp_link.shape
    if not tied:
        np.testing.assert_array_equal(linkage[:, [0, 1, 3]], exp_link[:, [0, 1, 3]])
    else:
        np.testing.assert_array_equal(linkage[:, 3], exp_link[:, 3])
    assert close(linkage[:, 2], exp_link[:, 2])
    exp_ct = case.get("remapped_condensed_tree", case["condensed_tree"])
    n_points = x.shape[0]
    got = canonical_condensed(cp, cc, cl, cs, n_points)
    exp = canonical_condensed(exp_ct["parent"], exp_ct["child"],
                              exp_ct["lambda_val"].astype(np.float32), exp_ct["child_size"],
                              n_points)
    assert len(got) == len(exp), f"{cid}: condensed rows"
    for g, e in zip(got, exp):
        if not tied:
            assert (g[0], g[1]) == (e[0], e[1]), f"{cid}: condensed leaves"
        assert close([g[2]], [e[2]]), f"{cid}: condensed lambda"
        assert abs(g[3] - e[3]) <= 1e-5


@pytest.mark.parametrize("cid", ["blobs_d2", "blobs_d10", "varying_density",
                                 "selection_interactions", "moons_leaf"])
def test_dbscan_cut_matches_fixture(cid, manifest):
    p = params(manifest, cid)
    case = load_case(cid)
    got = cg.dbscan_cut(case["linkage"], float(p["epsilon"]), p["min_samples"])
    np.testing.assert_array_equal(got, case["dbscan_labels"])


def test_dbscan_cut_rejects_nan():
    with pytest.raises(ValueError):
        cg.dbscan_cut(np.zeros((1, 4)), float("nan"), 2)


def test_extraction_rejects_cycles_and_nan():
    with pytest.raises(ValueError):
        cg.clusters_from_spanning_tree(np.array([0, 1], np.uint32), np.array([1, 0], np.uint32),
                                       np.array([1.0, 1.0]), min_cluster_size=2)
    with pytest.raises(ValueError):
        cg.clusters_from_spanning_tree(np.array([0], np.uint32), np.array([1], np.uint32),
                                       np.array([np.nan]), min_cluster_size=2)


def test_one_finite_contract():
    r = cg.clusters_from_spanning_tree(np.empty(0, np.uint32), np.empty(0, np.uint32),
                                       np.empty(0), min_cluster_size=2)
    assert r["labels"].tolist() == [-1] and r["probabilities"].tolist() == [0.0]
