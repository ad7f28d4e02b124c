"""sklearn-style ``HDBSCAN`` with the keyword surface of cuscan's Python estimator.

Provenance: the constructor, its attribute assignments, ``_input_array``, ``_positive_integer``,
``_validate_parameters`` and the unsupported-keyword checks follow python/cuscan/hdbscan.py of
lega0208/cuscan (MIT licence, Copyright 2026 M.L.) nearly line for line, because
they are the drop-in surface: the same keywords, defaults, validation order and messages. The
fit path behind them (the C ABI calls, finite-row handling around them) is this library's own.

Mirrors ``cuscan.HDBSCAN`` (python/cuscan/hdbscan.py:148-574 of lega0208/cuscan): the same
constructor keywords, validation messages, fitted attributes and error types. The fit core
(exact kNN core distances + Borůvka MST) runs in the sm_103a library through its C ABI; the
downstream extraction runs in the same library's host code.

Differences from the reference, by design:
 * The graph is always the exact complete mutual-reachability graph (the reference's
   ``MstGraph::Complete`` with brute-force search). The reference's default ``Auto`` graph
   switches to an approximate kNN graph above 30 features and 4096 rows
   (crates/hdbscan/src/estimator.rs:36,71-97); ``knn_k`` is accepted and ignored, as it is on
   the reference's complete-graph route.
 * ``backend`` may be "auto" or "cuda"; both run on the GPU. "cpu" raises: this library ships
   no CPU implementation and never falls back to one.
 * ``precision`` selects the distance arithmetic: "fp32" (exact f32 direct differences) or
   "bf16_refined" (bf16 tensor-core screening with exact f32 re-evaluation) or "fp16_refined"
   (the same screening with power-of-two-scaled fp16 operands, whose tighter error bound
   leaves fewer pairs to re-evaluate); all give bit-identical results.
 * ``approximate_predict`` runs the exact candidate search on the GPU and the reference's
   hierarchy math on the host (``cuscan_gb300.prediction``).
"""
from __future__ import annotations

import numpy as np

from . import _lib
from .prediction import (HDBSCANPredictor, Predictor, approximate_predict,
                         prediction_core_from_knn)

_ARRAY_NAMES = (
    "labels", "probabilities", "condensed_tree", "single_linkage_tree",
    "minimum_spanning_tree", "neighbors", "core_distances", "finite_index",
)

_CONDENSED_DTYPE = [("parent", np.intp), ("child", np.intp), ("lambda_val", np.float64),
                    ("child_size", np.float32)]

_CONTEXTS: dict[int, _lib.Context] = {}


def context(device_index: int = 0) -> _lib.Context:
    """Process-wide library context for one device (created on first use)."""
    ctx = _CONTEXTS.get(device_index)
    if ctx is None:
        ctx = _lib.Context(device_index)
        _CONTEXTS[device_index] = ctx
    return ctx


def _remap_condensed(parent, child, lam, size, finite_index, outliers):
    """remap_condensed (crates/hdbscan-core/src/finite.rs:193-250)."""
    nf = finite_index.shape[0]
    oc = outliers.shape[0]
    if parent.shape[0] == 0:
        return parent, child, lam, size
    root = parent[0] + oc
    new_child = np.where(child < nf, finite_index[np.minimum(child, nf - 1)], child + oc)
    return (np.concatenate([np.full(oc, root, np.int64), parent + oc]),
            np.concatenate([outliers.astype(np.int64), new_child]),
            np.concatenate([np.zeros(oc, np.float32), lam]),
            np.concatenate([np.ones(oc, np.float32), size]))


def _remap_linkage(linkage, finite_index, outliers):
    """remap_linkage (crates/hdbscan-core/src/finite.rs:258-293)."""
    if linkage.shape[0] == 0:
        return linkage
    nf = finite_index.shape[0]
    oc = outliers.shape[0]
    out = linkage.copy()
    for col in (0, 1):
        ids = linkage[:, col].astype(np.int64)
        out[:, col] = np.where(ids < nf, finite_index[np.minimum(ids, nf - 1)], ids + oc)
    last_id = int(max(out[-1, 0], out[-1, 1]))
    last_size = int(out[-1, 3])
    extra = []
    for o in outliers:
        last_id += 1
        last_size += 1
        extra.append([float(o), float(last_id), np.inf, float(last_size)])
    if extra:
        out = np.vstack([out, np.asarray(extra, np.float64)])
    return out


class HDBSCAN:
    """Hierarchical density-based clustering on the GB300 fit core.

    Keyword-compatible with ``cuscan.HDBSCAN``; see the module docstring for the differences.
    """

    def __init__(self, *, min_cluster_size: int = 5, min_samples: int | None = None,
                 cluster_selection_method: str = "eom", allow_single_cluster: bool = False,
                 max_cluster_size: int | float | None = None,
                 cluster_selection_epsilon: float = 0.0,
                 cluster_selection_persistence: float = 0.0, backend: str = "auto",
                 device_index: int = 0, reproducible: bool = False,
                 semi_supervised: bool = False, ss_algorithm: str = "bc",
                 metric: str = "euclidean", algorithm: str = "boruvka", knn_k: int | None = None,
                 cannot_link: object | None = None, validate_cannot_link: bool = True,
                 cannot_link_groups: object | None = None, metric_kwds: object | None = None,
                 memory_limit_bytes: int | None = None, precision: str = "fp32") -> None:
        self.min_cluster_size = min_cluster_size
        self.min_samples = min_samples
        self.cluster_selection_method = cluster_selection_method
        self.allow_single_cluster = allow_single_cluster
        self.max_cluster_size = max_cluster_size
        self.cluster_selection_epsilon = cluster_selection_epsilon
        self.cluster_selection_persistence = cluster_selection_persistence
        self.backend = backend
        self.device_index = device_index
        self.reproducible = reproducible
        self.semi_supervised = semi_supervised
        self.ss_algorithm = ss_algorithm
        self.metric = metric
        self.algorithm = algorithm
        self.knn_k = knn_k
        self.cannot_link = cannot_link
        self.validate_cannot_link = validate_cannot_link
        self.cannot_link_groups = cannot_link_groups
        self.metric_kwds = metric_kwds
        self.memory_limit_bytes = memory_limit_bytes
        self.precision = precision

    # ---- fitted attributes ----
    def _fitted_array(self, name):
        if not hasattr(self, "_fitted_state"):
            raise ValueError("This HDBSCAN instance is not fitted yet")
        return np.array(self._fitted_state["arrays"][name], copy=True)

    labels_ = property(lambda self: self._fitted_array("labels"))
    probabilities_ = property(lambda self: self._fitted_array("probabilities"))
    condensed_tree_ = property(lambda self: self._fitted_array("condensed_tree"))
    single_linkage_tree_ = property(lambda self: self._fitted_array("single_linkage_tree"))
    minimum_spanning_tree_ = property(lambda self: self._fitted_array("minimum_spanning_tree"))
    neighbors_ = property(lambda self: self._fitted_array("neighbors"))
    core_distances_ = property(lambda self: self._fitted_array("core_distances"))
    finite_index_ = property(lambda self: self._fitted_array("finite_index"))

    @property
    def n_features_in_(self) -> int:
        if not hasattr(self, "_fitted_state"):
            raise ValueError("This HDBSCAN instance is not fitted yet")
        return self._fitted_state["n_features_in"]

    @property
    def fit_stats_(self) -> dict:
        """Stage times and counters of the last fit core (milliseconds, rounds, rows)."""
        if not hasattr(self, "_fitted_state"):
            raise ValueError("This HDBSCAN instance is not fitted yet")
        return dict(self._fitted_state["stats"])

    # ---- validation (python/cuscan/hdbscan.py:275-364) ----
    @staticmethod
    def _input_array(X):
        try:
            values = np.asarray(X)
        except (TypeError, ValueError) as error:
            raise ValueError("X must be a numeric 2-D array") from error
        if values.ndim != 2:
            raise ValueError("X must be a 2-D array")
        if not np.issubdtype(values.dtype, np.number) or np.issubdtype(values.dtype,
                                                                        np.complexfloating):
            raise ValueError("X must be a numeric 2-D array")
        try:
            values64 = np.asarray(values, dtype=np.float64)
        except (TypeError, ValueError, OverflowError) as error:
            raise ValueError("X must be a numeric 2-D array") from error
        finite_rows = np.isfinite(values64).all(axis=1)
        f32_max = np.finfo(np.float32).max
        finite_values = values64[np.isfinite(values64)]
        if np.any(np.abs(finite_values) > f32_max):
            raise ValueError("finite values in X must fit in float32")
        with np.errstate(over="ignore", invalid="ignore"):
            result = np.ascontiguousarray(values64, dtype=np.float32)
        return result, finite_rows

    @staticmethod
    def _positive_integer(name, value, *, allow_none=False):
        if allow_none and value is None:
            return
        suffix = " or None" if allow_none else ""
        if isinstance(value, (bool, np.bool_)) or not isinstance(value, (int, np.integer)):
            raise ValueError(f"{name} must be a positive integer{suffix}")
        if int(value) <= 0:
            raise ValueError(f"{name} must be a positive integer{suffix}")

    def _validate_parameters(self):
        self._positive_integer("min_cluster_size", self.min_cluster_size)
        self._positive_integer("min_samples", self.min_samples, allow_none=True)
        for name, value in (("cluster_selection_epsilon", self.cluster_selection_epsilon),
                            ("cluster_selection_persistence", self.cluster_selection_persistence)):
            if not np.issubdtype(type(value), np.floating):
                raise ValueError(f"{name} must be a floating point number")
            if not np.isfinite(value) or value < 0.0:
                raise ValueError(f"{name} must be finite and non-negative")
        if self.cluster_selection_method not in ("eom", "leaf"):
            raise ValueError("cluster_selection_method must be 'eom' or 'leaf'")
        if not isinstance(self.allow_single_cluster, (bool, np.bool_)):
            raise ValueError("allow_single_cluster must be a boolean")
        if self.max_cluster_size is not None and not (
                isinstance(self.max_cluster_size, (float, np.floating))
                and np.isposinf(self.max_cluster_size)):
            self._positive_integer("max_cluster_size", self.max_cluster_size)
        if self.backend not in ("auto", "cpu", "cuda"):
            raise ValueError("backend must be 'auto', 'cpu' or 'cuda'")
        if not np.issubdtype(type(self.device_index), np.integer) or self.device_index < 0:
            raise ValueError("device_index must be a non-negative integer")
        if not isinstance(self.reproducible, (bool, np.bool_)):
            raise ValueError("reproducible must be a boolean")
        self._positive_integer("knn_k", self.knn_k, allow_none=True)
        if self.memory_limit_bytes is not None and (
                isinstance(self.memory_limit_bytes, (bool, np.bool_))
                or not isinstance(self.memory_limit_bytes, (int, np.integer))
                or not 0 < int(self.memory_limit_bytes) <= 2**64 - 1):
            raise ValueError("memory_limit_bytes must be a positive uint64 integer or None")
        if self.precision not in _lib.PRECISIONS:
            raise ValueError("precision must be 'fp32', 'bf16_refined' or 'fp16_refined'")
        unsupported = (("semi_supervised", self.semi_supervised, False),
                       ("ss_algorithm", self.ss_algorithm, "bc"),
                       ("metric", self.metric, "euclidean"),
                       ("algorithm", self.algorithm, "boruvka"),
                       ("cannot_link", self.cannot_link, None),
                       ("validate_cannot_link", self.validate_cannot_link, True),
                       ("cannot_link_groups", self.cannot_link_groups, None),
                       ("metric_kwds", self.metric_kwds, None))
        for name, value, default in unsupported:
            if default is None:
                is_default = value is None
            elif isinstance(default, bool):
                is_default = value is default
            else:
                is_default = value == default
            if not is_default:
                raise NotImplementedError(f"{name} is not supported")
        if self.backend == "cpu":
            raise NotImplementedError(
                "backend='cpu' is not provided by cuscan_gb300; it runs on CUDA only")

    def fit(self, X, y=None, sample_weight=None, **fit_params):
        if y is not None:
            raise NotImplementedError("y and semi-supervised fitting are not supported")
        if sample_weight is not None:
            raise NotImplementedError("sample_weight is not supported")
        if fit_params:
            raise NotImplementedError(f"fit parameter {next(iter(fit_params))!r} is not supported")
        self._validate_parameters()
        x, finite_rows = self._input_array(X)
        if x.shape[1] == 0:
            raise ValueError("input must contain at least one feature")
        if not np.any(finite_rows):
            raise ValueError("X must contain at least one fully finite row")
        state = fit_hdbscan(x, finite_rows, **self._native_kwargs())
        self._fitted_state = state
        return self

    def fit_predict(self, X, y=None, sample_weight=None, **fit_params):
        return self.fit(X, y, sample_weight, **fit_params).labels_

    def _native_kwargs(self):
        max_cluster_size = self.max_cluster_size
        if max_cluster_size is not None and np.isposinf(max_cluster_size):
            max_cluster_size = None
        return {
            "min_cluster_size": int(self.min_cluster_size),
            "min_samples": None if self.min_samples is None else int(self.min_samples),
            "cluster_selection_method": self.cluster_selection_method,
            "allow_single_cluster": bool(self.allow_single_cluster),
            "max_cluster_size": None if max_cluster_size is None else int(max_cluster_size),
            "cluster_selection_epsilon": float(self.cluster_selection_epsilon),
            "cluster_selection_persistence": float(self.cluster_selection_persistence),
            "device_index": int(self.device_index),
            "precision": self.precision,
        }

    def dbscan_clustering(self, eps: float):
        """DBSCAN labels at a single-linkage cut (estimator.rs:1488-1498)."""
        if not hasattr(self, "_fitted_state"):
            raise ValueError("This HDBSCAN instance is not fitted yet")
        st = self._fitted_state
        raw_n = st["arrays"]["labels"].shape[0]
        nf = st["arrays"]["finite_index"].shape[0]
        if nf <= 1 and nf != raw_n:
            return np.full(raw_n, -1, np.intp)
        linkage = st["arrays"]["single_linkage_tree"]
        if linkage.shape[0] == 0:
            return np.full(raw_n, -1, np.intp)
        return np.asarray(_lib.dbscan_cut(linkage, float(eps), st["min_samples"]), np.intp)

    def _predictor(self) -> Predictor:
        if not hasattr(self, "_fitted_state"):
            raise ValueError("This HDBSCAN instance is not fitted yet")
        st = self._fitted_state
        if st.get("predictor") is None:
            arrays = st["arrays"]
            tree = arrays["condensed_tree"]
            clustered = bool(np.any(np.asarray(tree["child_size"]) > 1))
            ms = st["min_samples"]
            n_finite = arrays["finite_index"].shape[0]
            if clustered and 2 * ms > n_finite:
                raise ValueError(
                    f"approximate_predict needs 2*min_samples = {2 * ms} neighbors but the model "
                    f"has only {n_finite} finite training points")
            st["predictor"] = Predictor(
                condensed_tree=tree, labels=arrays["labels"],
                finite_index=arrays["finite_index"], min_samples=ms,
                n_features=st["n_features_in"],
                train=st["fit_rows"] if clustered else None,
                prediction_core=(st["prediction_core"] if st["prediction_core"] is not None
                                 else np.zeros(n_finite, np.float64)),
                context=context(st["device_index"]) if clustered else None)
        return st["predictor"]

    def approximate_predict(self, X, return_connecting_points=False):
        """Predict fitted cluster labels for new points (original hdbscan
        ``approximate_predict``): ``(labels, strengths)`` or, with
        ``return_connecting_points=True``, ``(labels, strengths, connecting_points)``."""
        if not isinstance(return_connecting_points, (bool, np.bool_)):
            raise ValueError("return_connecting_points must be a boolean")
        return approximate_predict(self._predictor(), X, return_connecting_points)

    def to_predictor(self) -> HDBSCANPredictor:
        """Prepare and return a detached prediction-only view of this fitted model."""
        return HDBSCANPredictor._from_predictor(self._predictor())


def fit_hdbscan(x: np.ndarray, finite_rows: np.ndarray, *, min_cluster_size: int,
                min_samples: int | None, cluster_selection_method: str = "eom",
                allow_single_cluster: bool = False, max_cluster_size: int | None = None,
                cluster_selection_epsilon: float = 0.0,
                cluster_selection_persistence: float = 0.0, device_index: int = 0,
                precision: str = "fp32") -> dict:
    """Fit on float32 rows; the estimator flow of crates/hdbscan/src/estimator.rs:1034-1392."""
    ms = int(min_cluster_size if min_samples is None else min_samples)
    raw_n, d = x.shape
    finite_index = np.flatnonzero(finite_rows).astype(np.intp)
    outliers = np.flatnonzero(~finite_rows).astype(np.intp)
    n = finite_index.shape[0]
    xf = np.ascontiguousarray(x[finite_rows]) if outliers.size else x
    stats = {}
    if n > 1:
        ctx = context(device_index)
        prec = _lib.PRECISIONS[precision]
        core = ctx.fit_core(xf, ms, prec)
        stats = core["stats"]
        prediction_core = (prediction_core_from_knn(core["knn_sq"], ms) if ms <= n else None)
        k = core["knn_ids"].shape[1]
        core_distances = np.sqrt(core["core_sq"]).astype(np.float32)
        if k == ms:
            neighbors = core["knn_ids"].astype(np.intp)
        else:
            neighbors = np.full((n, ms), -1, np.intp)
            neighbors[:, :k] = core["knn_ids"]
        weights = np.sqrt(core["wsq"].astype(np.float64))
        host = _lib.clusters_from_spanning_tree(
            core["src"], core["dst"], weights, min_cluster_size=min_cluster_size,
            cluster_selection_method=cluster_selection_method,
            allow_single_cluster=allow_single_cluster, max_cluster_size=max_cluster_size,
            cluster_selection_epsilon=cluster_selection_epsilon,
            cluster_selection_persistence=cluster_selection_persistence)
        linkage = host["linkage"]
        cp, cc = host["condensed_parent"], host["condensed_child"]
        cl, cs = host["condensed_lambda"], host["condensed_child_size"]
        if outliers.size:
            linkage = _remap_linkage(linkage, finite_index, outliers)
            cp, cc, cl, cs = _remap_condensed(cp, cc, cl, cs, finite_index, outliers)
        labels = np.full(raw_n, -1, np.intp)
        labels[finite_index] = host["labels"]
        prob_f = host["probabilities"]
        mst = host["sorted_mst"]
    else:  # one finite row: all noise, empty trees (hdbscan-core lib.rs:40-50)
        prediction_core = np.zeros(n, np.float64)
        neighbors = np.empty((0, ms), np.intp)
        core_distances = np.full(n, np.inf, np.float32)
        linkage = np.empty((0, 4), np.float64)
        cp = cc = np.empty(0, np.int64)
        cl = cs = np.empty(0, np.float32)
        labels = np.full(raw_n, -1, np.intp)
        prob_f = np.zeros(n, np.float32)
        mst = np.empty((0, 3), np.float64)
    if finite_rows.all():
        probabilities = prob_f.astype(np.float32)
    else:
        probabilities = np.zeros(raw_n, np.float64)
        probabilities[finite_index] = prob_f
    condensed = np.empty(cp.shape[0], dtype=_CONDENSED_DTYPE)
    condensed["parent"] = cp
    condensed["child"] = cc
    condensed["lambda_val"] = cl.astype(np.float64)
    condensed["child_size"] = cs
    return {
        "arrays": {
            "labels": labels,
            "probabilities": probabilities,
            "condensed_tree": condensed,
            "single_linkage_tree": np.asarray(linkage, np.float64),
            "minimum_spanning_tree": np.asarray(mst, np.float64),
            "neighbors": neighbors,
            "core_distances": core_distances,
            "finite_index": finite_index,
        },
        "n_features_in": d,
        "min_samples": ms,
        "stats": stats,
        # prediction state: finite training rows (compact order) and their prediction cores
        "fit_rows": np.ascontiguousarray(xf, np.float32),
        "prediction_core": prediction_core,
        "device_index": device_index,
    }
