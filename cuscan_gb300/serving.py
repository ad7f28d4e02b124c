"""Continuous-batching request server on one GPU (the ``cuscan_server_*`` C ABI).

Requests are HDBSCAN fits of independent point sets and ``approximate_predict`` batches against
resident predictors. They queue in arrival order and are admitted onto execution slots (each
with its own CUDA stream, workspace and host thread) as slots and device memory free up, so
that requests of different sizes overlap on the device. A fit's result is the same as that of
``HDBSCAN(...).fit`` on the same rows (labels, membership strengths, core distances, sorted
MST), a prediction's the same as the predictor's own ``approximate_predict``; the tests check
both bit for bit.

The reference has no serving layer; a request runs the estimator flow of
crates/hdbscan/src/estimator.rs:1034-1392.
"""
from __future__ import annotations

import ctypes as C
import threading

import numpy as np

from . import _lib


MEMORY_RESERVE_BYTES = 64 << 20


def usable_bytes(free_bytes: int, total_bytes: int, live_bytes: int = 0,
                 limit_bytes: int | None = None) -> int:
    """Device memory a plan may commit, by the reference's admission rule
    (crates/cuscan-common/src/memory.rs:17-40): nine tenths of the free bytes (rounded down,
    computed as (free // 10) * 9 + (free % 10) * 9 // 10), plus the bytes the caller already
    holds, capped by an optional limit and by the total, less a 64 MiB reserve; never below 0."""
    for v in (free_bytes, total_bytes, live_bytes):
        if v < 0:
            raise ValueError("memory sizes must be non-negative")
    free = (free_bytes // 10) * 9 + (free_bytes % 10) * 9 // 10
    usable = min(free + live_bytes, total_bytes)
    if limit_bytes is not None:
        usable = min(usable, limit_bytes)
    return max(usable - MEMORY_RESERVE_BYTES, 0)


def default_budget(device: int = 0, limit_bytes: int | None = None) -> int:
    """The server's memory budget on `device` by the reference's rule (usable_bytes) applied
    to the device's free and total memory now."""
    import torch

    free, total = torch.cuda.mem_get_info(device)
    return usable_bytes(int(free), int(total), 0, limit_bytes)


def _precision_code(precision: str) -> int:
    if precision not in _lib.PRECISIONS:
        raise ValueError("precision must be 'fp32', 'bf16_refined' or 'fp16_refined'")
    return _lib.PRECISIONS[precision]


class FitServer:
    """Fit-request server. ``budget_bytes`` bounds the device workspace of all slots together;
    by default it is ``default_budget(device)``, the reference's admission rule on the device's
    free memory (16 GiB for the simulated server).

    ``pack_limit`` is the most small fits (at most ``_lib.PACK_MAX_ROWS`` rows) a slot runs
    together as one pack, each step of every fit in one launch; 8 by default, 1 runs every fit
    on its own (see ``cuscan_server_set_pack_limit``).

    ``simulated_us_per_kpoint`` builds the scheduling test double instead: the same queue and
    admission with slots that run no fit (no GPU needed; results cannot be read)."""

    def __init__(self, device: int = 0, slots: int = 4, budget_bytes: int | None = None, *,
                 pack_limit: int = 8, simulated_us_per_kpoint: float | None = None):
        if budget_bytes is None:
            budget_bytes = (16 << 30 if simulated_us_per_kpoint is not None
                            else default_budget(device))
        self._lib = _lib.load()
        handle = C.c_void_p()
        err = C.create_string_buffer(256)
        if simulated_us_per_kpoint is None:
            code = self._lib.cuscan_server_create(int(device), int(slots), int(budget_bytes),
                                                  C.byref(handle), err, 256)
        else:
            code = self._lib.cuscan_server_create_simulated(int(slots), int(budget_bytes),
                                                            float(simulated_us_per_kpoint),
                                                            C.byref(handle), err, 256)
        _lib.raise_for(code, err.value.decode("utf-8", "replace") or
                       f"could not start a fit server on device {device}")
        code = self._lib.cuscan_server_set_pack_limit(handle, int(pack_limit))
        if code != _lib.OK:
            self._lib.cuscan_server_destroy(handle)
            _lib.raise_for(code, f"pack_limit must be 1 to {_lib.PACK_MAX_FITS}")
        self.handle = handle
        self.simulated = simulated_us_per_kpoint is not None
        self._inputs: dict[int, np.ndarray] = {}
        self._guard = threading.Lock()

    # ---- requests ----
    def submit(self, x, *, min_cluster_size: int = 5, min_samples: int | None = None,
               precision: str = "bf16_refined", cluster_selection_method: str = "eom",
               allow_single_cluster: bool = False, max_cluster_size: int | None = None,
               cluster_selection_epsilon: float = 0.0,
               cluster_selection_persistence: float = 0.0) -> int:
        """Queue one fit; returns its request id. The array is kept alive until the result is
        taken."""
        if cluster_selection_method not in ("eom", "leaf"):
            raise ValueError("cluster_selection_method must be 'eom' or 'leaf'")
        arr = np.ascontiguousarray(x, dtype=np.float32)
        if arr.ndim != 2 or arr.shape[0] == 0 or arr.shape[1] == 0:
            raise ValueError("a fit request needs a non-empty 2-D array")
        ms = int(min_cluster_size if min_samples is None else min_samples)
        cfg = _lib.ExtractConfig(int(min_cluster_size),
                                 1 if cluster_selection_method == "leaf" else 0,
                                 1 if allow_single_cluster else 0,
                                 0 if max_cluster_size is None else int(max_cluster_size),
                                 float(cluster_selection_epsilon),
                                 float(cluster_selection_persistence))
        rid = C.c_int64(0)
        with self._guard:
            code = self._lib.cuscan_server_submit_fit(
                self.handle, arr.ctypes.data, arr.shape[0], arr.shape[1], ms,
                _precision_code(precision), C.byref(cfg), C.byref(rid))
            _lib.raise_for(code, "fit request rejected")
            self._inputs[int(rid.value)] = arr
        return int(rid.value)

    def submit_predict(self, predictor, x) -> int:
        """Queue an approximate_predict of finite query rows against a resident predictor
        (``cuscan_gb300.prediction.Predictor`` or ``HDBSCANPredictor`` on this device)."""
        pred = getattr(predictor, "_predictor", predictor)
        arr = np.ascontiguousarray(x, dtype=np.float32)
        if arr.ndim != 2 or arr.shape[0] == 0 or arr.shape[1] != pred.n_features_in_:
            raise ValueError("query rows must be a non-empty 2-D array with the model's features")
        if not np.all(np.isfinite(arr)):
            raise ValueError("X must contain only finite values")
        rid = C.c_int64(0)
        with self._guard:
            code = self._lib.cuscan_server_submit_predict(self.handle, pred.handle,
                                                          arr.ctypes.data, arr.shape[0],
                                                          C.byref(rid))
            _lib.raise_for(code, "predict request rejected")
            self._inputs[int(rid.value)] = (arr, pred)
        return int(rid.value)

    def wait(self, request_id: int, timeout: float | None = None) -> dict | None:
        """Information on a request once it has finished (None on timeout)."""
        info = _lib.ServerInfo()
        code = self._lib.cuscan_server_wait(self.handle, int(request_id),
                                            -1.0 if timeout is None else 1e3 * timeout,
                                            C.byref(info))
        if code == _lib.PENDING:
            return None
        _lib.raise_for(code, f"unknown request {request_id}")
        return info.as_dict()

    def wait_any(self, timeout: float | None = None) -> int | None:
        """The next finished request in completion order (each returned once), or None."""
        rid = C.c_int64(0)
        code = self._lib.cuscan_server_wait_any(self.handle,
                                                -1.0 if timeout is None else 1e3 * timeout,
                                                C.byref(rid))
        if code == _lib.PENDING:
            return None
        _lib.raise_for(code, "wait_any failed")
        return int(rid.value)

    def result(self, request_id: int, timeout: float | None = None, release: bool = True) -> dict:
        """Wait for a request and return its result with the request information: for a fit,
        labels, probabilities, core_distances and minimum_spanning_tree (sorted, Euclidean);
        for a prediction, labels, strengths and connecting_points. Raises the request's own
        error if it failed."""
        info = self.wait(request_id, timeout)
        if info is None:
            raise TimeoutError(f"request {request_id} has not finished")
        rid = int(request_id)
        try:
            if info["status"] != _lib.OK:
                buf = C.create_string_buffer(512)
                self._lib.cuscan_server_request_error(self.handle, rid, buf, 512)
                _lib.raise_for(info["status"], buf.value.decode("utf-8", "replace"))
            n, nf = int(info["n"]), int(info["finite_rows"])
            if info["kind"] == 1:
                labels = np.empty(n, np.int32)
                strengths = np.empty(n, np.float64)
                conn = np.empty(n, np.int32)
                code = self._lib.cuscan_server_read_predict(self.handle, rid, labels.ctypes.data,
                                                            strengths.ctypes.data,
                                                            conn.ctypes.data)
                _lib.raise_for(code, "the request's result cannot be read")
                return {"labels": labels.astype(np.intp), "strengths": strengths,
                        "connecting_points": conn.astype(np.intp), "info": info}
            labels = np.empty(n, np.int32)
            prob = np.empty(n, np.float32)
            core = np.empty(nf, np.float32)
            mst = np.empty((max(nf - 1, 0), 3), np.float64)
            code = self._lib.cuscan_server_read_fit(self.handle, rid, labels.ctypes.data,
                                                    prob.ctypes.data, core.ctypes.data,
                                                    mst.ctypes.data if mst.size else None)
            _lib.raise_for(code, "the request's result cannot be read")
            return {"labels": labels, "probabilities": prob, "core_distances": core,
                    "minimum_spanning_tree": mst, "info": info}
        finally:
            if release:
                self.release(rid)

    def release(self, request_id: int):
        """Drop a finished request's results and the reference to its input."""
        code = self._lib.cuscan_server_release(self.handle, int(request_id))
        if code == _lib.PENDING:
            raise RuntimeError(f"request {request_id} is still running")
        with self._guard:
            self._inputs.pop(int(request_id), None)

    def stats(self) -> dict:
        out = _lib.ServerStats()
        _lib.raise_for(self._lib.cuscan_server_get_stats(self.handle, C.byref(out)), "stats")
        return out.as_dict()

    def close(self):
        if getattr(self, "handle", None):
            self._lib.cuscan_server_destroy(self.handle)
            self.handle = None
            self._inputs.clear()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
