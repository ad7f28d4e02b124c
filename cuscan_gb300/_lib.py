"""ctypes binding of ``libcuscan_gb300.so`` (the C ABI declared in ``include/cuscan_gb300.h``).

Status codes map to Python exceptions exactly as the reference maps ``HdbscanError``
(crates/cuscan-python/src/hdbscan.rs:956-968): invalid config/input -> ValueError, backend
unavailable/numerical -> RuntimeError, overflow/capacity -> OverflowError, memory -> MemoryError.
There is no fallback: if the library or a CUDA device is missing, calls raise.
"""
from __future__ import annotations

import ctypes as C
import threading
from pathlib import Path

import numpy as np

OK, INVALID_CONFIG, INVALID_INPUT, BACKEND_UNAVAILABLE, NUMERICAL, OVERFLOW, CAPACITY, MEMORY = range(8)
PENDING = 8  # not an error: a server request is still queued or running
PRECISION_PLAIN = 0
PRECISION_BF16_REFINED = 1
PRECISION_FP16_REFINED = 2
PRECISIONS = {"fp32": 0, "bf16_refined": 1, "fp16_refined": 2}

_F32P = C.POINTER(C.c_float)
_F64P = C.POINTER(C.c_double)
_I32P = C.POINTER(C.c_int32)
_U32P = C.POINTER(C.c_uint32)
_I64P = C.POINTER(C.c_int64)
_VP = C.c_void_p

# Every symbol the header declares, with its ctypes signature (restype, argtypes).
SIGNATURES = {
    "cuscan_version": (C.c_char_p, []),
    "cuscan_launch_count": (C.c_int64, []),
    "cuscan_ctx_create": (C.c_int, [C.c_int, C.POINTER(_VP)]),
    "cuscan_ctx_destroy": (None, [_VP]),
    "cuscan_last_error": (C.c_char_p, [_VP]),
    "cuscan_error_kind": (C.c_int, [_VP]),
    "cuscan_ctx_stream": (_VP, [_VP]),
    "cuscan_exact_knn": (C.c_int, [_VP, _VP, C.c_int64, _VP, C.c_int64, C.c_int32, C.c_int32,
                                   C.c_int32, C.c_int64, C.c_int32, _VP, _VP, _VP]),
    "cuscan_boruvka_candidates": (C.c_int, [_VP, _VP, _VP, _VP, C.c_int64, C.c_int32, _VP, _VP,
                                            _VP]),
    "cuscan_component_reduce": (C.c_int, [_VP, _VP, _VP, _VP, _VP, _VP, _VP, C.c_int64,
                                          C.c_int64, C.c_int64, _VP, _VP, _VP]),
    "cuscan_component_reduce_noalloc": (C.c_int, [_VP, _VP, _VP, _VP, _VP, _VP, C.c_int64,
                                                  C.c_int64, C.c_int64, _VP, _VP, _VP,
                                                  C.c_char_p, C.c_size_t]),
    "cuscan_fit_core": (C.c_int, [_VP, _F32P, C.c_int64, C.c_int32, C.c_int32, C.c_int32, _I32P,
                                  _F32P, _F32P, _U32P, _U32P, _F32P, _I64P, _VP]),
    "cuscan_fit_core_device": (C.c_int, [_VP, _VP, C.c_int64, C.c_int32, C.c_int32, C.c_int32,
                                         _VP, _VP, _VP, _VP, _VP, _VP, _I64P, _VP, _VP]),
    "cuscan_fit_core_packed": (C.c_int, [_VP, _VP, C.c_int32]),
    "cuscan_fit_core_packed_launch_stats": (C.c_int, [_VP, _I64P, _I64P]),
    "cuscan_debug_screen_tile": (C.c_int, [_VP, _VP, C.c_int64, C.c_int32, _VP, _VP]),
    "cuscan_debug_screen_tile_operands": (C.c_int, [_VP, _VP, C.c_int64, C.c_int32, C.c_int32,
                                                    _VP, _VP, _VP, C.POINTER(C.c_float), _VP]),
    "cuscan_fit_round_stats": (C.c_int, [_VP, C.c_int32, _VP, _VP, _VP, _VP]),
    "cuscan_shard_seed": (C.c_int, [_VP, C.c_int64, C.c_int32, C.c_int32, _VP, _VP, _VP, _VP,
                                    _VP, _VP, _VP, C.POINTER(C.c_int64),
                                    C.POINTER(C.c_int64), _VP]),
    "cuscan_shard_round_keys": (C.c_int, [_VP, _VP, _VP, _VP, C.c_int64, C.c_int32, C.c_int64,
                                          C.c_int64, _VP, _VP]),
    "cuscan_shard_round_merge": (C.c_int, [_VP, _VP, _VP, _VP, C.c_int64, C.c_int32, _VP, _VP,
                                           _VP, _VP, C.POINTER(C.c_int64),
                                           C.POINTER(C.c_int64), C.POINTER(C.c_double), _VP]),
    "cuscan_clusters_from_spanning_tree": (C.c_int, [_U32P, _U32P, _F64P, C.c_int64, _VP,
                                                     C.POINTER(_VP), C.c_char_p, C.c_size_t]),
    "cuscan_clustering_points": (C.c_int64, [_VP]),
    "cuscan_clustering_condensed_rows": (C.c_int64, [_VP]),
    "cuscan_clustering_read": (None, [_VP, _I32P, _F32P, _F64P, _F64P, _I64P, _I64P, _F32P,
                                      _F32P]),
    "cuscan_clustering_free": (None, [_VP]),
    "cuscan_dbscan_cut": (C.c_int, [_F64P, C.c_int64, C.c_double, C.c_int64, _I32P]),
    "cuscan_predictor_create": (C.c_int, [_VP, _VP, C.c_int64, C.c_int32, C.c_int32, _VP, _VP,
                                          _VP, _VP, C.c_int64, _VP, C.c_int64, _VP, _VP,
                                          C.POINTER(_VP), C.c_char_p, C.c_size_t]),
    "cuscan_predictor_destroy": (None, [_VP]),
    "cuscan_predictor_no_cluster_tree": (C.c_int, [_VP]),
    "cuscan_predictor_read_cores": (C.c_int, [_VP, _VP]),
    "cuscan_predictor_predict": (C.c_int, [_VP, _VP, _VP, C.c_int64, _VP, _VP, _VP]),
    "cuscan_predictor_predict_candidates": (C.c_int, [_VP, _VP, _VP, C.c_int64, _VP, _VP, _VP,
                                                      C.c_char_p, C.c_size_t]),
    "cuscan_fit_workspace_bytes": (C.c_int64, [C.c_int64, C.c_int32, C.c_int32, C.c_int32]),
    "cuscan_ctx_reserved_bytes": (C.c_int64, [_VP]),
    "cuscan_ctx_release_workspace": (C.c_int, [_VP]),
    "cuscan_server_create": (C.c_int, [C.c_int, C.c_int32, C.c_int64, C.POINTER(_VP),
                                       C.c_char_p, C.c_size_t]),
    "cuscan_server_create_simulated": (C.c_int, [C.c_int32, C.c_int64, C.c_double,
                                                 C.POINTER(_VP), C.c_char_p, C.c_size_t]),
    "cuscan_server_destroy": (None, [_VP]),
    "cuscan_server_submit_fit": (C.c_int, [_VP, _VP, C.c_int64, C.c_int32, C.c_int32, C.c_int32,
                                           _VP, _I64P]),
    "cuscan_server_wait": (C.c_int, [_VP, C.c_int64, C.c_double, _VP]),
    "cuscan_server_wait_any": (C.c_int, [_VP, C.c_double, _I64P]),
    "cuscan_server_read_fit": (C.c_int, [_VP, C.c_int64, _VP, _VP, _VP, _VP]),
    "cuscan_server_submit_predict": (C.c_int, [_VP, _VP, _VP, C.c_int64, _I64P]),
    "cuscan_server_read_predict": (C.c_int, [_VP, C.c_int64, _VP, _VP, _VP]),
    "cuscan_predictor_shape": (C.c_int, [_VP, _I64P, C.POINTER(C.c_int32), C.POINTER(C.c_int32)]),
    "cuscan_predict_workspace_bytes": (C.c_int64, [_VP, C.c_int64]),
    "cuscan_predictor_state_shape": (C.c_int, [_VP, _I64P, _I64P]),
    "cuscan_predictor_export": (C.c_int, [_VP, _VP, _VP, _VP, _VP, _VP, _VP, _VP, _VP, _VP, _VP,
                                          _VP]),
    "cuscan_predictor_from_state": (C.c_int, [_VP, _VP, C.c_int64, C.c_int32, C.c_int32, _VP,
                                              C.c_int64, _VP, _VP, _VP, _VP, _VP, _VP, _VP, _VP,
                                              C.POINTER(_VP), C.c_char_p, C.c_size_t]),
    "cuscan_server_request_error": (C.c_int, [_VP, C.c_int64, C.c_char_p, C.c_size_t]),
    "cuscan_server_release": (C.c_int, [_VP, C.c_int64]),
    "cuscan_server_get_stats": (C.c_int, [_VP, _VP]),
    "cuscan_server_set_pack_limit": (C.c_int, [_VP, C.c_int32]),
}


class FitStats(C.Structure):
    _fields_ = [
        ("core_ms", C.c_double),
        ("mst_ms", C.c_double),
        ("knn_kernel_ms", C.c_double),
        ("candidate_kernel_ms", C.c_double),
        ("rounds", C.c_int64),
        ("seed_edges", C.c_int64),
        ("components_after_seed", C.c_int64),
        ("refined_rows", C.c_int64),
        ("fallback_rows", C.c_int64),
        ("boruvka_fallback_rows", C.c_int64),
        ("cross_pairs", C.c_double),
        ("rescreened_rows", C.c_int64),
        ("screen_tile_pairs", C.c_int64),
        ("boruvka_screened_rows", C.c_int64),
        ("mst_weight", C.c_double),
        ("knn_screen_ms", C.c_double),
        ("symmetric_rounds", C.c_int64),
        ("operand_format", C.c_int64),
    ]

    def as_dict(self) -> dict:
        return {name: getattr(self, name) for name, _ in self._fields_}


PACK_MAX_FITS = 16
PACK_MAX_ROWS = 2047
PACK_MAX_FEATURES = 256


class FitItem(C.Structure):
    """One point set of cuscan_fit_core_packed (host pointers)."""
    _fields_ = [
        ("data", _F32P),
        ("n", C.c_int64),
        ("d", C.c_int32),
        ("min_samples", C.c_int32),
        ("precision", C.c_int32),
        ("status", C.c_int32),
        ("knn_ids", _I32P),
        ("knn_sq", _F32P),
        ("core_sq", _F32P),
        ("mst_src", _U32P),
        ("mst_dst", _U32P),
        ("mst_wsq", _F32P),
        ("n_edges", C.c_int64),
        ("stats", FitStats),
    ]


class ExtractConfig(C.Structure):
    _fields_ = [
        ("min_cluster_size", C.c_int64),
        ("selection_leaf", C.c_int32),
        ("allow_single_cluster", C.c_int32),
        ("max_cluster_size", C.c_int64),
        ("cluster_selection_epsilon", C.c_double),
        ("cluster_selection_persistence", C.c_double),
    ]


class ServerInfo(C.Structure):
    _fields_ = [
        ("request_id", C.c_int64),
        ("status", C.c_int32),
        ("slot", C.c_int32),
        ("kind", C.c_int32),
        ("pack_size", C.c_int32),
        ("n", C.c_int64),
        ("finite_rows", C.c_int64),
        ("d", C.c_int32),
        ("n_clusters", C.c_int32),
        ("workspace_bound_bytes", C.c_int64),
        ("submit_ms", C.c_double),
        ("queued_ms", C.c_double),
        ("run_ms", C.c_double),
        ("latency_ms", C.c_double),
        ("done_ms", C.c_double),
        ("prep_ms", C.c_double),
        ("fit_ms", C.c_double),
        ("extract_ms", C.c_double),
        ("stats", FitStats),
    ]

    def as_dict(self) -> dict:
        out = {name: getattr(self, name) for name, _ in self._fields_
               if name not in ("stats", "pad")}
        out["stats"] = self.stats.as_dict()
        return out


class ServerStats(C.Structure):
    _fields_ = [
        ("slots", C.c_int32),
        ("pad", C.c_int32),
        ("budget_bytes", C.c_int64),
        ("submitted", C.c_int64),
        ("completed", C.c_int64),
        ("failed", C.c_int64),
        ("queued", C.c_int64),
        ("running", C.c_int64),
        ("committed_bytes", C.c_int64),
        ("peak_committed_bytes", C.c_int64),
        ("workspace_releases", C.c_int64),
        ("packs", C.c_int64),
        ("packed_requests", C.c_int64),
    ]

    def as_dict(self) -> dict:
        return {name: getattr(self, name) for name, _ in self._fields_ if name != "pad"}


_lock = threading.Lock()
_lib = None


def library_path() -> Path:
    return Path(__file__).resolve().parent / "_build" / "libcuscan_gb300.so"


def load(build_if_missing: bool = True):
    """Load the shared library (building it first when it is absent)."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = library_path()
        if not path.exists() and build_if_missing:
            from . import build as _build
            _build.build()
        if not path.exists():
            raise RuntimeError(f"cuscan_gb300 native library is missing: {path}")
        lib = C.CDLL(str(path))
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
        return lib


def launch_count() -> int:
    """Kernels launched by the library in this process so far."""
    return int(load().cuscan_launch_count())


NOALLOC_MAX_TILES = 65536


def component_reduce_noalloc(weights, indices, members, tile_starts, tile_ends, partial_offsets,
                             n, p, c, win_weights, win_meta, stream=None):
    """cuscan_component_reduce_noalloc on device pointers: the variant that allocates nothing
    (its tile scratch is a fixed static device array of NOALLOC_MAX_TILES entries)."""
    lib = load()
    err = C.create_string_buffer(256)
    code = lib.cuscan_component_reduce_noalloc(weights, indices, members, tile_starts, tile_ends,
                                               partial_offsets, n, p, c, win_weights, win_meta,
                                               stream, err, 256)
    raise_for(code, err.value.decode("utf-8", "replace"))


def fit_workspace_bytes(n: int, d: int, min_samples: int, precision: int) -> int:
    """Upper bound on the device workspace of one fit (cuscan_fit_workspace_bytes)."""
    return int(load().cuscan_fit_workspace_bytes(int(n), int(d), int(min_samples), int(precision)))


def raise_for(code: int, message: str):
    if code == OK:
        return
    if code in (INVALID_CONFIG, INVALID_INPUT):
        raise ValueError(message)
    if code in (BACKEND_UNAVAILABLE, NUMERICAL):
        raise RuntimeError(message)
    if code in (OVERFLOW, CAPACITY):
        raise OverflowError(message)
    if code == MEMORY:
        raise MemoryError(message)
    raise RuntimeError(f"cuscan_gb300 status {code}: {message}")


class Context:
    """One CUDA device context of the library (its own stream and reusable workspace)."""

    def __init__(self, device: int = 0):
        self._lib = load()
        handle = _VP()
        code = self._lib.cuscan_ctx_create(int(device), C.byref(handle))
        if code != OK:
            raise_for(BACKEND_UNAVAILABLE if code == BACKEND_UNAVAILABLE else code,
                      f"CUDA device {device} is unavailable (a Blackwell-class device is required)")
        self.handle = handle
        self.device = int(device)

    def close(self):
        if getattr(self, "handle", None):
            self._lib.cuscan_ctx_destroy(self.handle)
            self.handle = None

    def reserved_bytes(self) -> int:
        """Device bytes this context's workspace holds."""
        return int(self._lib.cuscan_ctx_reserved_bytes(self.handle))

    def release_workspace(self):
        self.check(self._lib.cuscan_ctx_release_workspace(self.handle))

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def stream(self) -> int:
        return int(self._lib.cuscan_ctx_stream(self.handle) or 0)

    def check(self, code: int):
        if code != OK:
            msg = self._lib.cuscan_last_error(self.handle).decode("utf-8", "replace")
            raise_for(code, msg)

    # ---- backend operations on device pointers (integers) ----
    def exact_knn(self, query, nq, reference, nr, d, k, exclude_self, query_offset, squared,
                  ids_out, dist_out, stream=None):
        self.check(self._lib.cuscan_exact_knn(self.handle, query, nq, reference, nr, d, k,
                                              int(exclude_self), query_offset, int(squared),
                                              ids_out, dist_out, stream))

    def boruvka_candidates(self, data, core_sq, components, n, d, weights_out, dst_out,
                           stream=None):
        self.check(self._lib.cuscan_boruvka_candidates(self.handle, data, core_sq, components, n,
                                                       d, weights_out, dst_out, stream))

    def component_reduce(self, weights, indices, members, tile_starts, tile_ends,
                         partial_offsets, n, p, c, win_weights, win_meta, stream=None):
        self.check(self._lib.cuscan_component_reduce(self.handle, weights, indices, members,
                                                     tile_starts, tile_ends, partial_offsets, n,
                                                     p, c, win_weights, win_meta, stream))

    def fit_core_device(self, data, n, d, min_samples, precision, knn_ids, knn_sq, core_sq,
                        src, dst, wsq, stream=None):
        m = C.c_int64(0)
        stats = FitStats()
        self.check(self._lib.cuscan_fit_core_device(self.handle, data, n, d, min_samples,
                                                    precision, knn_ids, knn_sq, core_sq, src,
                                                    dst, wsq, C.byref(m), C.byref(stats), stream))
        return int(m.value), stats

    def debug_screen_tile(self, data, n, d, tile_out, stream=None, operands=None, rows_out=None,
                          chunk_out=None):
        """Raw accumulator of the first 128 x 256 screen tile; with `operands` (0 bf16, 1 fp16,
        2 split bf16) the chosen format, returning the operand scale (the tile holds scale^2 x
        the dots). rows_out (device float[n][4]) receives every row's bound terms
        (ps, pb, cm, m); chunk_out (device float[128][8]) the screen's maxima of the tile's
        32-column chunks."""
        if operands is None and chunk_out is None:
            self.check(self._lib.cuscan_debug_screen_tile(self.handle, data, n, d, tile_out,
                                                          stream))
            return 1.0
        scale = C.c_float(0.0)
        self.check(self._lib.cuscan_debug_screen_tile_operands(
            self.handle, data, n, d, operands or 0, tile_out, rows_out, chunk_out, C.byref(scale),
            stream))
        return float(scale.value)

    def round_stats(self) -> list[dict]:
        """Per Borůvka round of this context's last fit: screened rows, tensor-core tiles,
        candidate-kernel ms and ordered cross-component pairs."""
        cap = 64
        rows = np.zeros(cap, np.int64)
        tiles = np.zeros(cap, np.int64)
        ms = np.zeros(cap, np.float64)
        cross = np.zeros(cap, np.float64)
        count = self._lib.cuscan_fit_round_stats(self.handle, cap, rows.ctypes.data,
                                                 tiles.ctypes.data, ms.ctypes.data,
                                                 cross.ctypes.data)
        return [{"rows": int(rows[r]), "tiles": int(tiles[r]), "ms": float(ms[r]),
                 "cross_pairs": float(cross[r])} for r in range(min(max(count, 0), cap))]

    # ---- row shards (device pointers) ----
    def shard_seed(self, n, d, min_samples, knn_ids, knn_sq, core_sq, labels, src, dst, wsq,
                   stream=None):
        m, comps = C.c_int64(0), C.c_int64(0)
        self.check(self._lib.cuscan_shard_seed(self.handle, n, d, min_samples, knn_ids, knn_sq,
                                               core_sq, labels, src, dst, wsq, C.byref(m),
                                               C.byref(comps), stream))
        return int(m.value), int(comps.value)

    def shard_round_keys(self, data, core_sq, labels, n, d, row_begin, row_end, row_keys,
                         stream=None):
        self.check(self._lib.cuscan_shard_round_keys(self.handle, data, core_sq, labels, n, d,
                                                     row_begin, row_end, row_keys, stream))

    def shard_round_merge(self, data, core_sq, labels, n, d, row_keys, src, dst, wsq,
                          stream=None):
        m, comps, w = C.c_int64(0), C.c_int64(0), C.c_double(float("nan"))
        self.check(self._lib.cuscan_shard_round_merge(self.handle, data, core_sq, labels, n, d,
                                                      row_keys, src, dst, wsq, C.byref(m),
                                                      C.byref(comps), C.byref(w), stream))
        return int(m.value), int(comps.value), float(w.value)

    # ---- host-pointer fit ----
    @staticmethod
    def fit_core_outputs(n: int, min_samples: int, empty=np.empty) -> dict:
        """Output arrays of fit_core for n rows; `empty(shape, dtype)` allocates each (for
        example from pinned host memory, so that the device-to-host copies run at full speed)."""
        k = min(int(min_samples), n - 1)
        m = max(n - 1, 1)
        return {"knn_ids": empty((n, k), np.int32), "knn_sq": empty((n, k), np.float32),
                "core_sq": empty((n,), np.float32), "src": empty((m,), np.uint32),
                "dst": empty((m,), np.uint32), "wsq": empty((m,), np.float32)}

    def fit_core(self, x: np.ndarray, min_samples: int, precision: int = PRECISION_PLAIN,
                 out: dict | None = None):
        """Host-pointer fit core. `out` (from fit_core_outputs) receives the results in place;
        by default new arrays are allocated."""
        x = np.ascontiguousarray(x, dtype=np.float32)
        n, d = x.shape
        o = out if out is not None else self.fit_core_outputs(n, min_samples)
        ids, ksq, core = o["knn_ids"], o["knn_sq"], o["core_sq"]
        src, dst, w = o["src"], o["dst"], o["wsq"]
        k = min(int(min_samples), n - 1)
        need = max(n - 1, 1)
        for a, dt, size in ((ids, np.int32, n * k), (ksq, np.float32, n * k),
                            (core, np.float32, n), (src, np.uint32, need),
                            (dst, np.uint32, need), (w, np.float32, need)):
            if a.dtype != dt or not a.flags.c_contiguous or a.size < size:
                raise ValueError("fit_core outputs must be C-contiguous arrays of the documented "
                                 "dtypes and sizes")
        m = C.c_int64(0)
        stats = FitStats()
        self.check(self._lib.cuscan_fit_core(
            self.handle, x.ctypes.data_as(_F32P), n, d, int(min_samples), int(precision),
            ids.ctypes.data_as(_I32P), ksq.ctypes.data_as(_F32P), core.ctypes.data_as(_F32P),
            src.ctypes.data_as(_U32P), dst.ctypes.data_as(_U32P), w.ctypes.data_as(_F32P),
            C.byref(m), C.byref(stats)))
        e = int(m.value)
        return {"knn_ids": ids, "knn_sq": ksq, "core_sq": core, "src": src[:e], "dst": dst[:e],
                "wsq": w[:e], "stats": stats.as_dict()}


    def fit_core_packed(self, fits):
        """Fit cores of several small point sets, each step of every fit in one launch.

        `fits` is a sequence of (x, min_samples, precision). Returns one dict per fit, shaped
        like fit_core's, plus its "status"; raises if any fit failed (the first failure)."""
        items = (FitItem * len(fits))()
        keep = []
        outs = []
        for item, (x, ms, prec) in zip(items, fits):
            x = np.ascontiguousarray(x, dtype=np.float32)
            n, d = x.shape
            k = min(int(ms), n - 1)
            o = {"knn_ids": np.empty((n, k), np.int32), "knn_sq": np.empty((n, k), np.float32),
                 "core_sq": np.empty(n, np.float32), "src": np.empty(max(n - 1, 1), np.uint32),
                 "dst": np.empty(max(n - 1, 1), np.uint32),
                 "wsq": np.empty(max(n - 1, 1), np.float32)}
            keep.append(x)
            outs.append(o)
            item.data = x.ctypes.data_as(_F32P)
            item.n, item.d, item.min_samples, item.precision = n, d, int(ms), int(prec)
            item.knn_ids = o["knn_ids"].ctypes.data_as(_I32P)
            item.knn_sq = o["knn_sq"].ctypes.data_as(_F32P)
            item.core_sq = o["core_sq"].ctypes.data_as(_F32P)
            item.mst_src = o["src"].ctypes.data_as(_U32P)
            item.mst_dst = o["dst"].ctypes.data_as(_U32P)
            item.mst_wsq = o["wsq"].ctypes.data_as(_F32P)
        self.check(self._lib.cuscan_fit_core_packed(self.handle, items, len(fits)))
        for item, o in zip(items, outs):
            e = int(item.n_edges)
            for key in ("src", "dst", "wsq"):
                o[key] = o[key][:e]
            o["stats"] = item.stats.as_dict()
            o["status"] = int(item.status)
        return outs

    def packed_launch_stats(self) -> dict:
        """The latest pack of this context: kernels launched and host reads of its round
        counter."""
        launches, reads = C.c_int64(0), C.c_int64(0)
        self.check(self._lib.cuscan_fit_core_packed_launch_stats(self.handle, C.byref(launches),
                                                                 C.byref(reads)))
        return {"launches": int(launches.value), "host_reads": int(reads.value)}


def clusters_from_spanning_tree(src, dst, weight, *, min_cluster_size: int,
                                cluster_selection_method: str = "eom",
                                allow_single_cluster: bool = False,
                                max_cluster_size: int | None = None,
                                cluster_selection_epsilon: float = 0.0,
                                cluster_selection_persistence: float = 0.0) -> dict:
    """Host extraction of labels, strengths, linkage and condensed tree from an MST."""
    lib = load()
    src = np.ascontiguousarray(src, np.uint32)
    dst = np.ascontiguousarray(dst, np.uint32)
    weight = np.ascontiguousarray(weight, np.float64)
    m = int(src.shape[0])
    cfg = ExtractConfig(int(min_cluster_size), 1 if cluster_selection_method == "leaf" else 0,
                        1 if allow_single_cluster else 0,
                        0 if max_cluster_size is None else int(max_cluster_size),
                        float(cluster_selection_epsilon), float(cluster_selection_persistence))
    out = _VP()
    err = C.create_string_buffer(512)
    code = lib.cuscan_clusters_from_spanning_tree(
        src.ctypes.data_as(_U32P), dst.ctypes.data_as(_U32P), weight.ctypes.data_as(_F64P), m,
        C.byref(cfg), C.byref(out), err, 512)
    raise_for(code, err.value.decode("utf-8", "replace"))
    try:
        npts = int(lib.cuscan_clustering_points(out))
        rows = int(lib.cuscan_clustering_condensed_rows(out))
        labels = np.empty(npts, np.int32)
        prob = np.empty(npts, np.float32)
        linkage = np.empty((m, 4), np.float64)
        smst = np.empty((m, 3), np.float64)
        cp = np.empty(rows, np.int64)
        cc = np.empty(rows, np.int64)
        cl = np.empty(rows, np.float32)
        cs = np.empty(rows, np.float32)
        lib.cuscan_clustering_read(out, labels.ctypes.data_as(_I32P), prob.ctypes.data_as(_F32P),
                                   linkage.ctypes.data_as(_F64P), smst.ctypes.data_as(_F64P),
                                   cp.ctypes.data_as(_I64P), cc.ctypes.data_as(_I64P),
                                   cl.ctypes.data_as(_F32P), cs.ctypes.data_as(_F32P))
    finally:
        lib.cuscan_clustering_free(out)
    return {"labels": labels, "probabilities": prob, "linkage": linkage, "sorted_mst": smst,
            "condensed_parent": cp, "condensed_child": cc, "condensed_lambda": cl,
            "condensed_child_size": cs}


def dbscan_cut(linkage: np.ndarray, cut: float, min_size: int) -> np.ndarray:
    lib = load()
    linkage = np.ascontiguousarray(linkage, np.float64)
    rows = int(linkage.shape[0])
    out = np.empty(rows + 1, np.int32)
    code = lib.cuscan_dbscan_cut(linkage.ctypes.data_as(_F64P), rows, float(cut), int(min_size),
                                 out.ctypes.data_as(_I32P))
    raise_for(code, "DBSCAN cut must not be NaN" if code == INVALID_CONFIG else "invalid linkage")
    return out
