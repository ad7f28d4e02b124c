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
