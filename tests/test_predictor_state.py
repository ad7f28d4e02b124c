"""Portable predictor state: the arrays and metadata of the reference's predictor schema v1
(python/cuscan/_hdbscan_predictor_serialization_v1.py) and the import rules of
PredictionHierarchy::from_state / import_predictor_state (crates/hdbscan-core/src/prediction.rs:
279-433, crates/hdbscan/src/prediction.rs:1335-1424).

The CPU cases run on host-only predictors built from the reference's controlled prediction
fixture (no geometry); they mirror crates/hdbscan/tests/test_predictor_state.rs: exact round
trips, the malformed-state table and the rank-one canonical-zero rule. The GPU cases fit a
model, export it, import it on the device and require bit-identical predictions.
"""
from __future__ import annotations

import copy
import warnings

import numpy as np
import pytest

from cuscan_gb300.prediction import STATE_ARRAYS, STATE_DTYPES, Predictor
from tests.test_prediction import FIXTURE, floats, tree_of


def host_predictor(tree_index: int = 0, min_samples: int | None = None):
    name = sorted(FIXTURE["controlled"]["trees"])[tree_index]
    spec = FIXTURE["controlled"]["trees"][name]
    labels = np.array(spec["labels"], np.int32)
    query = next(q for q in FIXTURE["controlled"]["queries"] if q["tree"] == name)
    s = int(query["min_samples"]) if min_samples is None else min_samples
    cores = floats(query["core_distances"])
    if s == 1:
        cores = np.zeros_like(cores)
    p = Predictor(condensed_tree=tree_of(spec["raw_tree"]), labels=labels,
                  finite_index=np.arange(labels.shape[0], dtype=np.uint32), min_samples=s,
                  n_features=1, prediction_core=cores)
    return p, query


def assert_states_equal(a, b):
    (arr_a, meta_a), (arr_b, meta_b) = a, b
    assert meta_a == meta_b
    assert set(arr_a) == set(arr_b) == set(STATE_ARRAYS)
    for name in STATE_ARRAYS:
        if arr_a[name] is None or arr_b[name] is None:
            assert arr_a[name] is None and arr_b[name] is None, name
            continue
        assert arr_a[name].dtype == np.dtype(STATE_DTYPES[name]), name
        assert arr_a[name].dtype == arr_b[name].dtype, name
        assert arr_a[name].tobytes() == arr_b[name].tobytes(), name


def no_tree_state():
    arrays = dict.fromkeys(STATE_ARRAYS)
    metadata = {"n_features": 2, "n_finite": 0, "min_samples": 2, "cluster_nodes": 0,
                "cores_status": "not_required_no_cluster_tree", "cores_rank": 0}
    return arrays, metadata


@pytest.mark.parametrize("tree_index", range(len(FIXTURE["controlled"]["trees"])))
def test_host_state_roundtrip_is_exact(tree_index):
    p, query = host_predictor(tree_index)
    arrays, meta = p.export_state()
    assert meta["cores_status"] == "ready" and meta["cores_rank"] == meta["min_samples"]
    assert arrays["geometry"] is None
    nn, nf = meta["cluster_nodes"], meta["n_finite"]
    for name in STATE_ARRAYS[1:]:
        assert arrays[name].shape == ((nn,) if name.startswith("node_") else (nf,))
    assert arrays["node_parent_indices"][0] == np.iinfo(np.uint64).max
    assert arrays["node_birth_lambdas"][0].tobytes() == np.float64(0.0).tobytes()
    q = Predictor.from_state(arrays, meta, None)
    assert_states_equal((arrays, meta), q.export_state())
    ids = np.array([query["indices"]], np.int32)
    dist = floats(query["distances"])[None, :]
    for a, b in zip(p.predict_candidates(ids, dist), q.predict_candidates(ids, dist)):
        assert a.tobytes() == b.tobytes()


def test_no_tree_state_roundtrips_without_payload():
    arrays, meta = no_tree_state()
    q = Predictor.from_state(arrays, meta, None)
    assert q.no_cluster_tree
    assert_states_equal((arrays, meta), q.export_state())


def _set(name, index, value):
    def mutate(arrays, meta):
        arrays[name] = arrays[name].copy()
        arrays[name][index] = value
    return mutate


def _meta(name, value):
    def mutate(arrays, meta):
        meta[name] = value
    return mutate


def _pop(name):
    def mutate(arrays, meta):
        arrays[name] = arrays[name][:-1].copy()
    return mutate


def _nonascending(arrays, meta):
    arrays["finite_index"] = arrays["finite_index"].copy()
    arrays["finite_index"][1] = arrays["finite_index"][0]


def _status_no_tree(arrays, meta):
    meta["cores_status"] = "not_required_no_cluster_tree"


MALFORMED = [
    ("zero feature count", _meta("n_features", 0)),
    ("zero min_samples", _meta("min_samples", 0)),
    ("core rank mismatch", lambda a, m: m.__setitem__("cores_rank", m["cores_rank"] + 1)),
    ("NaN prediction core", _set("prediction_cores", 0, np.nan)),
    ("negative prediction core", _set("prediction_cores", 0, -1.0)),
    ("infinite prediction core", _set("prediction_cores", 0, np.inf)),
    ("prediction core count mismatch", _pop("prediction_cores")),
    ("invalid root parent", _set("node_parent_indices", 0, 0)),
    ("nonascending finite map", _nonascending),
    ("out-of-range point node", _set("point_node_indices", 0, np.iinfo(np.uint64).max)),
    ("NaN node birth", _set("node_birth_lambdas", 0, np.nan)),
    ("candidate width", _meta("min_samples", 10 ** 9)),
    ("clustered state marked no-tree", _status_no_tree),
    ("negative node birth", _set("node_birth_lambdas", 1, -0.5)),
    ("node label below -1", _set("node_labels", 0, -2)),
    ("NaN departure", _set("point_departure_lambdas", 0, np.nan)),
    ("duplicate node id", lambda a, m: _set("node_ids", 1, a["node_ids"][0])(a, m)),
    ("wrong dtype", lambda a, m: a.__setitem__("node_labels", a["node_labels"].astype("<i8"))),
    ("extra metadata", _meta("format", 1)),
    ("boolean count", _meta("n_finite", True)),
]


@pytest.mark.parametrize("case,mutate", MALFORMED, ids=[c[0] for c in MALFORMED])
def test_rejects_malformed_state(case, mutate):
    p, _ = host_predictor(0)
    arrays, meta = p.export_state()
    arrays, meta = dict(arrays), copy.deepcopy(meta)
    if case == "candidate width":
        meta["cores_rank"] = meta["min_samples"] = 10 ** 9
    mutate(arrays, meta)
    with pytest.raises(ValueError):
        Predictor.from_state(arrays, meta, None)


def test_rejects_inherited_maximum_and_parent_order():
    p, _ = host_predictor(0)
    arrays, meta = p.export_state()
    if meta["cluster_nodes"] < 2:
        pytest.skip("tree has a single node")
    bad = dict(arrays)
    bad["node_parent_indices"] = arrays["node_parent_indices"].copy()
    bad["node_parent_indices"][1] = 1  # a node that is its own parent
    with pytest.raises(ValueError, match="parent graph"):
        Predictor.from_state(bad, meta, None)
    bad = dict(arrays)
    bad["node_ids"] = arrays["node_ids"].copy()
    bad["node_ids"][0] = bad["node_ids"].max() + 1  # the root is not the smallest id
    with pytest.raises(ValueError, match="root"):
        Predictor.from_state(bad, meta, None)


def test_rank_one_state_requires_canonical_zero_cores():
    p, _ = host_predictor(0, min_samples=1)
    arrays, meta = p.export_state()
    assert all(v.tobytes() == np.float64(0.0).tobytes() for v in arrays["prediction_cores"])
    Predictor.from_state(arrays, meta, None)
    arrays = dict(arrays)
    arrays["prediction_cores"] = arrays["prediction_cores"].copy()
    arrays["prediction_cores"][0] = -0.0
    with pytest.raises(ValueError, match="canonical positive zero"):
        Predictor.from_state(arrays, meta, None)


def test_no_tree_presence_rules():
    arrays, meta = no_tree_state()
    bad = dict(arrays, geometry=np.zeros(2, "<f4"))
    with pytest.raises(ValueError, match="presence"):
        Predictor.from_state(bad, meta, None)
    with pytest.raises(ValueError, match="noncanonical"):
        Predictor.from_state(arrays, dict(meta, cores_rank=2), None)
    with pytest.raises(ValueError, match="noncanonical"):
        Predictor.from_state(arrays, dict(meta, n_finite=3), None)


def test_file_serialization_needs_h5py():
    pytest.importorskip("numpy")
    try:
        import h5py  # noqa: F401
        pytest.skip("h5py is installed")
    except ImportError:
        pass
    from cuscan_gb300.prediction import HDBSCANPredictor
    obj = HDBSCANPredictor.__new__(HDBSCANPredictor)
    with pytest.raises(ImportError, match="cuscan\\[serialization\\]"):
        obj.save("predictor.h5")
    with pytest.raises(ImportError, match="cuscan\\[serialization\\]"):
        HDBSCANPredictor.load("predictor.h5")


# ---- GPU: fitted predictors through export -> import ----

@pytest.mark.gpu
@pytest.mark.parametrize("prec", ["fp32", "bf16_refined"])
def test_fitted_state_imports_on_device_and_predicts_identically(prec):
    from cuscan_gb300 import HDBSCAN, HDBSCANPredictor, synthetic
    x = synthetic.gaussian_mixture(3000, 8, blobs=5, std_range=(0.05, 0.3), seed=21)
    q = synthetic.gaussian_mixture(700, 8, blobs=5, std_range=(0.05, 0.5), seed=22)
    model = HDBSCAN(min_cluster_size=20, min_samples=6, precision=prec).fit(x)
    pred = model.to_predictor()
    arrays, meta = pred.export_state()
    assert meta == {"n_features": 8, "n_finite": 3000, "min_samples": 6,
                    "cluster_nodes": meta["cluster_nodes"], "cores_status": "ready",
                    "cores_rank": 6}
    assert arrays["geometry"].tobytes() == np.ascontiguousarray(x, np.float32).tobytes()
    restored = HDBSCANPredictor.from_state(arrays, meta)
    assert_states_equal((arrays, meta), restored.export_state())
    want = pred.approximate_predict(q, return_connecting_points=True)
    got = restored.approximate_predict(q, return_connecting_points=True)
    for a, b in zip(want, got):
        assert a.dtype == b.dtype and a.tobytes() == b.tobytes()


@pytest.mark.gpu
def test_device_import_rejects_bad_geometry():
    from cuscan_gb300 import HDBSCAN, HDBSCANPredictor, synthetic
    x = synthetic.gaussian_mixture(600, 4, blobs=3, std_range=(0.05, 0.2), seed=5)
    arrays, meta = HDBSCAN(min_cluster_size=15, min_samples=4).fit(x).to_predictor().export_state()
    bad = dict(arrays, geometry=arrays["geometry"].copy())
    bad["geometry"][3] = np.nan
    with pytest.raises(ValueError, match="finite"):
        HDBSCANPredictor.from_state(bad, meta)
    bad = dict(arrays, geometry=arrays["geometry"][:-1].copy())
    with pytest.raises(ValueError, match="geometry"):
        HDBSCANPredictor.from_state(bad, meta)


@pytest.mark.gpu
def test_no_tree_predictor_state_on_device():
    from cuscan_gb300 import HDBSCAN, HDBSCANPredictor
    x = np.random.default_rng(3).normal(size=(30, 3)).astype(np.float32)
    model = HDBSCAN(min_cluster_size=40, min_samples=5).fit(x)
    arrays, meta = model.to_predictor().export_state()
    assert meta["cores_status"] == "not_required_no_cluster_tree"
    assert all(v is None for v in arrays.values())
    restored = HDBSCANPredictor.from_state(arrays, meta)
    with warnings.catch_warnings(record=True) as caught:
        warnings.simplefilter("always")
        labels, strengths = restored.approximate_predict(x[:4])
    assert len(caught) == 1
    assert (labels == -1).all() and (strengths == 0).all()
