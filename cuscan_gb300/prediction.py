"""``approximate_predict`` and the detached predictor (the ``cuscan_predictor_*`` C ABI).

Mirrors ``cuscan.HDBSCAN.approximate_predict`` / ``HDBSCANPredictor`` (python/cuscan/hdbscan.py:
30-133, 533-574 of lega0208/cuscan) and the hierarchy math of
crates/hdbscan-core/src/prediction.rs: labels are existing fitted labels (``-1`` noise),
strengths are f64, connecting points are original training-row indices. A model whose tree has
no clusters predicts all noise / ``0`` / ``-1`` with one ``UserWarning``.

The exact candidate searches (queries against the finite training rows, width
``2 * min_samples``) run on the GPU; the hierarchy walk is host f64 arithmetic in the library.
"""
from __future__ import annotations

import ctypes as C
import warnings

import numpy as np

from . import _lib

NO_CLUSTER_WARNING = ("Clusterer does not have any defined clusters, new data will be "
                      "automatically predicted as noise.")


# Arrays and metadata of the predictor schema v1
# (python/cuscan/_hdbscan_predictor_serialization_v1.py:10-35 of the reference).
STATE_ARRAYS = ("geometry", "finite_index", "node_ids", "node_parent_indices",
                "node_birth_lambdas", "node_labels", "node_max_lambdas", "point_node_indices",
                "point_departure_lambdas", "prediction_cores")
STATE_DTYPES = {"geometry": "<f4", "finite_index": "<u4", "node_ids": "<u8",
                "node_parent_indices": "<u8", "node_birth_lambdas": "<f8", "node_labels": "<i4",
                "node_max_lambdas": "<f8", "point_node_indices": "<u8",
                "point_departure_lambdas": "<f8", "prediction_cores": "<f8"}
STATE_META = {"n_features", "n_finite", "min_samples", "cluster_nodes", "cores_status",
              "cores_rank"}


def _uint(value, name):
    if isinstance(value, bool) or not isinstance(value, (int, np.integer)) or value < 0:
        raise ValueError(f"invalid predictor metadata: {name}")
    return int(value)


def validate_state(arrays: dict, metadata: dict, geometry: bool = True) -> tuple[dict, bool]:
    """The schema's metadata, presence, dtype and length rules (serialization_v1.py:49-116 of
    the reference); the hierarchy itself is validated by the library. ``geometry=False`` checks
    a host-only state, whose ``geometry`` entry is None."""
    if set(metadata) != STATE_META:
        raise ValueError("invalid predictor metadata fields")
    if set(arrays) != set(STATE_ARRAYS):
        raise ValueError("invalid predictor array fields")
    vals = {name: _uint(metadata[name], name)
            for name in ("n_features", "n_finite", "min_samples", "cluster_nodes", "cores_rank")}
    status = metadata["cores_status"]
    if status not in ("ready", "not_required_no_cluster_tree"):
        raise ValueError("invalid predictor core status")
    vals["cores_status"] = status
    if vals["n_features"] == 0 or vals["min_samples"] == 0:
        raise ValueError("predictor feature count and min_samples must be positive")
    no_tree = status == "not_required_no_cluster_tree"
    for name in STATE_ARRAYS:
        present = arrays[name] is not None
        if name == "geometry" and not geometry and not no_tree:
            if present:
                raise ValueError("a host-only predictor state has no geometry")
            continue
        if present == no_tree:
            raise ValueError("predictor dataset presence disagrees with core status")
    if no_tree:
        if any(vals[name] != 0 for name in ("n_finite", "cluster_nodes", "cores_rank")):
            raise ValueError("noncanonical no-cluster predictor metadata")
        return vals, True
    if vals["n_finite"] == 0 or vals["cluster_nodes"] == 0:
        raise ValueError("clustered predictor dimensions must be positive")
    if vals["n_finite"] > np.iinfo(np.int32).max or vals["cluster_nodes"] > np.iinfo(np.int32).max:
        raise ValueError("predictor row and cluster counts exceed i32 limits")
    if vals["cores_rank"] != vals["min_samples"]:
        raise ValueError("predictor core rank disagrees with min_samples")
    if vals["min_samples"] > vals["n_finite"] // 2:
        raise ValueError("predictor min_samples exceeds candidate-width limit")
    lengths = {name: (vals["n_finite"] * vals["n_features"] if name == "geometry"
                      else vals["cluster_nodes"] if name.startswith("node_") else vals["n_finite"])
               for name in STATE_ARRAYS}
    for name, length in lengths.items():
        if name == "geometry" and not geometry:
            continue
        value = np.asarray(arrays[name])
        if value.ndim != 1 or value.size != length or value.dtype != np.dtype(STATE_DTYPES[name]):
            raise ValueError(f"invalid predictor array dtype, rank or shape: {name}")
    return vals, False


def prediction_core_from_knn(knn_sq: np.ndarray, min_samples: int) -> np.ndarray:
    """Training prediction cores from the fit's self-excluding kNN rows: the self-inclusive
    distance at rank ``s - 1`` is the self-excluding one at rank ``s - 2`` (self is at distance
    0), as Euclidean f64 (crates/hdbscan-core/src/prediction.rs:94-120)."""
    n = knn_sq.shape[0]
    if min_samples == 1:
        return np.zeros(n, np.float64)
    col = np.asarray(knn_sq[:, min_samples - 2], np.float32)
    if not np.all(np.isfinite(col)) or np.any(col < 0):
        raise RuntimeError("neighbor search returned invalid squared distance")
    return np.sqrt(col.astype(np.float64))


class Predictor:
    """Prediction state of one fitted model: hierarchy, cores and (with a device context) the
    finite training rows on the GPU."""

    def __init__(self, *, condensed_tree, labels, finite_index, min_samples: int,
                 n_features: int, train=None, prediction_core=None, context=None):
        self._lib = _lib.load()
        tree = np.asarray(condensed_tree)
        parent = np.ascontiguousarray(tree["parent"], np.int64)
        child = np.ascontiguousarray(tree["child"], np.int64)
        lam = np.ascontiguousarray(tree["lambda_val"], np.float32)
        size = np.ascontiguousarray(tree["child_size"], np.float32)
        labels = np.ascontiguousarray(labels, np.int32)
        finite_index = np.ascontiguousarray(finite_index, np.uint32)
        self.n_features_in_ = int(n_features)
        self.min_samples = int(min_samples)
        self.n_finite = int(finite_index.shape[0])
        train_ptr = None
        if train is not None:
            train = np.ascontiguousarray(train, np.float32)
            if train.shape != (self.n_finite, self.n_features_in_):
                raise ValueError("training rows do not match the finite index")
            train_ptr = train.ctypes.data
        core_ptr = None
        if prediction_core is not None:
            prediction_core = np.ascontiguousarray(prediction_core, np.float64)
            core_ptr = prediction_core.ctypes.data
        handle = C.c_void_p()
        err = C.create_string_buffer(512)
        code = self._lib.cuscan_predictor_create(
            context.handle if context is not None else None, train_ptr, self.n_finite,
            self.n_features_in_, self.min_samples, parent.ctypes.data, child.ctypes.data,
            lam.ctypes.data, size.ctypes.data, int(parent.shape[0]), labels.ctypes.data,
            int(labels.shape[0]), finite_index.ctypes.data, core_ptr, C.byref(handle), err, 512)
        _lib.raise_for(code, err.value.decode("utf-8", "replace"))
        self.handle = handle
        self.context = context
        self.has_rows = train is not None
        self.no_cluster_tree = bool(self._lib.cuscan_predictor_no_cluster_tree(handle))

    def cores(self) -> np.ndarray:
        out = np.empty(self.n_finite, np.float64)
        _lib.raise_for(self._lib.cuscan_predictor_read_cores(self.handle, out.ctypes.data), "")
        return out

    def predict(self, x: np.ndarray):
        """(labels, strengths, connecting points) of finite query rows."""
        x = np.ascontiguousarray(x, np.float32)
        m = x.shape[0]
        labels = np.empty(m, np.int32)
        strengths = np.empty(m, np.float64)
        conn = np.empty(m, np.int32)
        if self.context is None:
            raise RuntimeError("this predictor has no device context")
        self.context.check(self._lib.cuscan_predictor_predict(
            self.context.handle, self.handle, x.ctypes.data, m, labels.ctypes.data,
            strengths.ctypes.data, conn.ctypes.data))
        return labels, strengths, conn

    def predict_candidates(self, ids: np.ndarray, distances: np.ndarray):
        """The candidate math on given rows of width 2 * min_samples (compact ids, Euclidean
        distances)."""
        ids = np.ascontiguousarray(ids, np.int32)
        distances = np.ascontiguousarray(distances, np.float64)
        m = ids.shape[0]
        labels = np.empty(m, np.int32)
        strengths = np.empty(m, np.float64)
        conn = np.empty(m, np.int32)
        err = C.create_string_buffer(512)
        code = self._lib.cuscan_predictor_predict_candidates(
            self.handle, ids.ctypes.data, distances.ctypes.data, m, labels.ctypes.data,
            strengths.ctypes.data, conn.ctypes.data, err, 512)
        _lib.raise_for(code, err.value.decode("utf-8", "replace"))
        return labels, strengths, conn

    # ---- portable state (the arrays and metadata of the predictor schema v1) ----
    def export_state(self) -> tuple[dict, dict]:
        """(arrays, metadata) in the layout of python/cuscan/_hdbscan_predictor_serialization_v1.py
        of the reference; all arrays are None for the no-cluster-tree state, and ``geometry`` is
        None for a host-only predictor (one without training rows)."""
        nf, nn = C.c_int64(0), C.c_int64(0)
        _lib.raise_for(self._lib.cuscan_predictor_state_shape(self.handle, C.byref(nf),
                                                              C.byref(nn)), "state shape")
        nf, nn = int(nf.value), int(nn.value)
        meta = {"n_features": self.n_features_in_, "n_finite": nf, "min_samples": self.min_samples,
                "cluster_nodes": nn}
        if nn == 0:
            meta.update(cores_status="not_required_no_cluster_tree", cores_rank=0)
            return {name: None for name in STATE_ARRAYS}, meta
        arrays = {name: np.empty(nf * self.n_features_in_ if name == "geometry"
                                 else (nn if name.startswith("node_") else nf),
                                 STATE_DTYPES[name]) for name in STATE_ARRAYS}
        if not self.has_rows:
            arrays["geometry"] = None
            ptrs = [None if arrays[name] is None else arrays[name].ctypes.data
                    for name in STATE_ARRAYS]
            _lib.raise_for(self._lib.cuscan_predictor_export(None, self.handle, *ptrs),
                           "predictor export failed")
        else:
            if self.context is None:
                raise RuntimeError("this predictor has no device context")
            self.context.check(self._lib.cuscan_predictor_export(
                self.context.handle, self.handle,
                *[arrays[name].ctypes.data for name in STATE_ARRAYS]))
        meta.update(cores_status="ready", cores_rank=self.min_samples)
        return arrays, meta

    @classmethod
    def from_state(cls, arrays: dict, metadata: dict, context) -> "Predictor":
        """Validate portable state (the schema v1 rules of the reference) and build a predictor
        on the context's device (host-only when ``geometry`` is None and no context is given)."""
        host_only = arrays.get("geometry") is None and context is None
        meta, no_tree = validate_state(arrays, metadata, geometry=not host_only)
        obj = cls.__new__(cls)
        obj._lib = _lib.load()
        obj.n_features_in_ = meta["n_features"]
        obj.min_samples = meta["min_samples"]
        obj.n_finite = meta["n_finite"]
        obj.context = context
        obj.has_rows = not host_only and not no_tree
        handle = C.c_void_p()
        err = C.create_string_buffer(512)
        if no_tree:
            code = obj._lib.cuscan_predictor_from_state(
                context.handle if context is not None else None, None, 0, obj.n_features_in_,
                obj.min_samples, None, 0, None, None, None, None, None, None, None, None,
                C.byref(handle), err, 512)
        else:
            cols = {name: np.ascontiguousarray(arrays[name], STATE_DTYPES[name])
                    for name in STATE_ARRAYS if not (host_only and name == "geometry")}
            code = obj._lib.cuscan_predictor_from_state(
                None if context is None else context.handle,
                None if host_only else cols["geometry"].ctypes.data, meta["n_finite"],
                obj.n_features_in_, obj.min_samples, cols["finite_index"].ctypes.data,
                meta["cluster_nodes"], cols["node_ids"].ctypes.data,
                cols["node_parent_indices"].ctypes.data, cols["node_birth_lambdas"].ctypes.data,
                cols["node_labels"].ctypes.data, cols["node_max_lambdas"].ctypes.data,
                cols["point_node_indices"].ctypes.data,
                cols["point_departure_lambdas"].ctypes.data,
                cols["prediction_cores"].ctypes.data, C.byref(handle), err, 512)
        _lib.raise_for(code, err.value.decode("utf-8", "replace"))
        obj.handle = handle
        obj.no_cluster_tree = bool(obj._lib.cuscan_predictor_no_cluster_tree(handle))
        return obj

    def close(self):
        if getattr(self, "handle", None):
            self._lib.cuscan_predictor_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def approximate_predict(predictor: Predictor, X, return_connecting_points=False,
                        stacklevel: int = 3):
    """Validation and output conventions of python/cuscan/hdbscan.py:30-63."""
    from .hdbscan import HDBSCAN
    if not isinstance(return_connecting_points, (bool, np.bool_)):
        raise ValueError("return_connecting_points must be a boolean")
    x, finite_rows = HDBSCAN._input_array(X)
    if x.shape[0] == 0 or x.shape[1] == 0:
        raise ValueError("X must contain at least one row and one feature")
    if not finite_rows.all():
        raise ValueError("X must contain only finite values")
    if x.shape[1] != predictor.n_features_in_:
        raise ValueError(f"X has {x.shape[1]} features, but the model was fitted with "
                         f"{predictor.n_features_in_}")
    if x.shape[0] > np.iinfo(np.int32).max:
        raise OverflowError("X row count exceeds i32::MAX")
    if predictor.no_cluster_tree:
        m = x.shape[0]
        labels = np.full(m, -1, np.intp)
        strengths = np.zeros(m, np.float64)
        conn = np.full(m, -1, np.intp)
        warnings.warn(NO_CLUSTER_WARNING, UserWarning, stacklevel=stacklevel)
    else:
        lab, strengths, conn = predictor.predict(x)
        labels = lab.astype(np.intp)
        conn = conn.astype(np.intp)
    if bool(return_connecting_points):
        return labels, strengths, conn
    return labels, strengths


class HDBSCANPredictor:
    """Lightweight detached predictor for an already-fitted HDBSCAN hierarchy
    (python/cuscan/hdbscan.py:67-133)."""

    def __init__(self):
        raise TypeError("use HDBSCAN.to_predictor()")

    @classmethod
    def _from_predictor(cls, predictor: Predictor) -> "HDBSCANPredictor":
        obj = cls.__new__(cls)
        obj._predictor = predictor
        return obj

    @property
    def n_features_in_(self) -> int:
        return self._predictor.n_features_in_

    def approximate_predict(self, X, return_connecting_points=False):
        """Predict into the fixed hierarchy and return new arrays in query order."""
        return approximate_predict(self._predictor, X, return_connecting_points)

    def export_state(self) -> tuple[dict, dict]:
        """(arrays, metadata) of the predictor schema v1."""
        return self._predictor.export_state()

    @classmethod
    def from_state(cls, arrays: dict, metadata: dict, *, device_index: int = 0):
        """A predictor from schema v1 arrays and metadata, on a CUDA device."""
        from .hdbscan import context
        meta, no_tree = validate_state(arrays, metadata)
        ctx = None if no_tree else context(device_index)
        return cls._from_predictor(Predictor.from_state(arrays, metadata, ctx))

    def save(self, path, overwrite: bool = False):
        """HDF5 files need h5py and hdf5plugin, as in the reference."""
        _hdf5_deps()
        raise NotImplementedError("HDF5 predictor files are not written by cuscan_gb300; use "
                                  "export_state() and store the arrays")

    @classmethod
    def load(cls, path, *, backend: str = "auto", device_index: int = 0):
        _hdf5_deps()
        raise NotImplementedError("HDF5 predictor files are not read by cuscan_gb300; use "
                                  "from_state() with the stored arrays")


def _hdf5_deps():
    try:
        import h5py  # noqa: F401
        import hdf5plugin  # noqa: F401
    except ImportError as error:
        raise ImportError("HDBSCAN predictor serialization requires cuscan[serialization] (h5py "
                          "and hdf5plugin)") from error
