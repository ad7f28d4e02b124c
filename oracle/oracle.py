"""ctypes view of the C oracle (``hdbscan_oracle.c``).

Test infrastructure only: the pytest suite, ``__graft_entry__.smoke()`` and the CPU baseline of
``bench.py`` use it as the checker. The product path never imports this module.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

from . import build_oracle

_LIB = None

_F32P = C.POINTER(C.c_float)
_I32P = C.POINTER(C.c_int32)
_U32P = C.POINTER(C.c_uint32)
_I64P = C.POINTER(C.c_int64)
_F64P = C.POINTER(C.c_double)


class _FitStats(C.Structure):
    _fields_ = [
        ("rounds", C.c_int64),
        ("seed_edges", C.c_int64),
        ("components_after_seed", C.c_int64),
        ("round_components", _I64P),
        ("round_cross_pairs", _F64P),
        ("max_rounds", C.c_int64),
    ]


class OracleError(RuntimeError):
    def __init__(self, code: int, what: str):
        super().__init__(f"oracle {what} failed with status {code}")
        self.code = code


def lib():
    global _LIB
    if _LIB is None:
        path = build_oracle.build()
        L = C.CDLL(str(path))
        L.orc_exact_neighbors.argtypes = [_F32P, C.c_int64, _F32P, C.c_int64, C.c_int, C.c_int,
                                          C.c_int, C.c_int64, C.c_int, _I32P, _F32P]
        L.orc_core_from_knn.argtypes = [_F32P, C.c_int64, C.c_int, C.c_int, _F32P]
        L.orc_init_from_knn.argtypes = [_F32P, _I32P, _F32P, C.c_int64, C.c_int, _U32P, _U32P,
                                        _F32P, _I64P, _I32P]
        L.orc_boruvka_candidates.argtypes = [_F32P, _F32P, _I32P, C.c_int64, C.c_int, _F32P, _I32P]
        L.orc_boruvka_candidates_rows.argtypes = [_F32P, _F32P, _I32P, C.c_int64, C.c_int,
                                                  C.c_int64, C.c_int64, _F32P, _I32P]
        L.orc_component_plan.argtypes = [_I32P, C.c_int64, C.c_int, _I32P, _I32P, _I32P, _I32P,
                                         _I32P, _I64P, _I64P]
        L.orc_component_reduce.argtypes = [_F32P, _I32P, _I32P, _I32P, C.c_int64, C.c_int64,
                                           _F32P, _I32P]
        L.orc_fit_core.argtypes = [_F32P, C.c_int64, C.c_int, C.c_int, _I32P, _F32P, _F32P,
                                   _U32P, _U32P, _F32P, _I64P, C.POINTER(_FitStats)]
        L.orc_brute_force_mst.argtypes = [_F32P, C.c_int64, C.c_int, C.c_int, C.c_int, _U32P,
                                          _U32P, _F32P, _I64P]
        L.orc_finalize_mst.argtypes = [_U32P, _U32P, _F32P, C.c_int64, _F64P]
        L.orc_pair_distances.argtypes = [_F32P, _F32P, C.c_int64, C.c_int, C.c_int, _F32P]
        L.orc_set_threads.argtypes = [C.c_int]
        L.orc_set_blocked.argtypes = [C.c_int]
        L.orc_exact_neighbors_blocked.argtypes = L.orc_exact_neighbors.argtypes
        L.orc_boruvka_candidates_blocked.argtypes = L.orc_boruvka_candidates.argtypes
        L.orc_prediction_cores.argtypes = [_F32P, C.c_int64, C.c_int, C.c_int, _F64P]
        L.orc_predict_candidates.argtypes = [_I64P, _I64P, _F32P, _F32P, C.c_int64, _I32P,
                                             C.c_int64, _U32P, C.c_int64, C.c_int, _F64P, _I32P,
                                             _F64P, C.c_int64, _I32P, _F64P, _I32P,
                                             C.POINTER(C.c_int)]
        L.orc_max_threads.restype = C.c_int
        _LIB = L
    return _LIB


def _p(a: np.ndarray, t):
    return a.ctypes.data_as(t)


def _check(code: int, what: str) -> None:
    if code != 0:
        raise OracleError(code, what)


def set_threads(threads: int) -> None:
    lib().orc_set_threads(int(threads))


def max_threads() -> int:
    return int(lib().orc_max_threads())


def set_blocked(on: bool) -> None:
    """Whether fit_core runs the blocked all-pairs loops (the default; bit-identical to the
    row-at-a-time loops, several times faster where the compiler vectorises them)."""
    lib().orc_set_blocked(int(bool(on)))


def exact_neighbors(query, reference, k, *, exclude_self=True, query_offset=0, squared=True,
                    blocked=False):
    """Exact kNN rows; `blocked` selects the blocked loop (same bits), otherwise the
    row-at-a-time loop that the CPU baseline times."""
    q = np.ascontiguousarray(query, dtype=np.float32)
    r = np.ascontiguousarray(reference, dtype=np.float32)
    nq, d = q.shape
    ids = np.empty((nq, k), np.int32)
    dist = np.empty((nq, k), np.float32)
    fn = lib().orc_exact_neighbors_blocked if blocked else lib().orc_exact_neighbors
    _check(fn(_p(q, _F32P), nq, _p(r, _F32P), r.shape[0], d, k, int(exclude_self), query_offset,
              int(squared), _p(ids, _I32P), _p(dist, _F32P)), "exact_neighbors")
    return ids, dist


def core_from_knn(knn_sq: np.ndarray, min_samples: int) -> np.ndarray:
    knn_sq = np.ascontiguousarray(knn_sq, dtype=np.float32)
    n, k = knn_sq.shape
    core = np.empty(n, np.float32)
    lib().orc_core_from_knn(_p(knn_sq, _F32P), n, k, min_samples, _p(core, _F32P))
    return core


def init_from_knn(core_sq, neighbors, knn_sq):
    core_sq = np.ascontiguousarray(core_sq, np.float32)
    neighbors = np.ascontiguousarray(neighbors, np.int32)
    knn_sq = np.ascontiguousarray(knn_sq, np.float32)
    n, k = neighbors.shape
    src = np.empty(max(n, 1), np.uint32)
    dst = np.empty(max(n, 1), np.uint32)
    w = np.empty(max(n, 1), np.float32)
    m = np.zeros(1, np.int64)
    labels = np.empty(n, np.int32)
    _check(lib().orc_init_from_knn(_p(core_sq, _F32P), _p(neighbors, _I32P), _p(knn_sq, _F32P), n,
                                   k, _p(src, _U32P), _p(dst, _U32P), _p(w, _F32P), _p(m, _I64P),
                                   _p(labels, _I32P)), "init_from_knn")
    e = int(m[0])
    return src[:e].copy(), dst[:e].copy(), w[:e].copy(), labels


def boruvka_candidates(x, core_sq, components, *, blocked=False):
    x = np.ascontiguousarray(x, np.float32)
    core_sq = np.ascontiguousarray(core_sq, np.float32)
    components = np.ascontiguousarray(components, np.int32)
    n, d = x.shape
    w = np.empty(n, np.float32)
    dst = np.empty(n, np.int32)
    fn = lib().orc_boruvka_candidates_blocked if blocked else lib().orc_boruvka_candidates
    _check(fn(_p(x, _F32P), _p(core_sq, _F32P), _p(components, _I32P), n, d, _p(w, _F32P),
              _p(dst, _I32P)), "boruvka_candidates")
    return w, dst


def boruvka_candidate_rows(x, core_sq, components, row_begin, row_end):
    """Candidates of rows [row_begin, row_end) against all rows (bounded timing sample)."""
    x = np.ascontiguousarray(x, np.float32)
    core_sq = np.ascontiguousarray(core_sq, np.float32)
    components = np.ascontiguousarray(components, np.int32)
    n, d = x.shape
    m = row_end - row_begin
    w = np.empty(max(m, 1), np.float32)
    dst = np.empty(max(m, 1), np.int32)
    _check(lib().orc_boruvka_candidates_rows(_p(x, _F32P), _p(core_sq, _F32P),
                                             _p(components, _I32P), n, d, row_begin, row_end,
                                             _p(w, _F32P), _p(dst, _I32P)), "candidate rows")
    return w[:m], dst[:m]


@dataclass
class ComponentPlan:
    members: np.ndarray
    offsets: np.ndarray
    tile_starts: np.ndarray
    tile_ends: np.ndarray
    partial_offsets: np.ndarray


def component_plan(labels, tile_width: int = 512) -> ComponentPlan:
    labels = np.ascontiguousarray(labels, np.int32)
    n = labels.shape[0]
    members = np.empty(max(n, 1), np.int32)
    offsets = np.empty(n + 1, np.int32)
    ts = np.empty(max(n, 1), np.int32)
    te = np.empty(max(n, 1), np.int32)
    po = np.empty(n + 1, np.int32)
    c = np.zeros(1, np.int64)
    p = np.zeros(1, np.int64)
    _check(lib().orc_component_plan(_p(labels, _I32P), n, tile_width, _p(members, _I32P),
                                    _p(offsets, _I32P), _p(ts, _I32P), _p(te, _I32P), _p(po, _I32P),
                                    _p(c, _I64P), _p(p, _I64P)), "component_plan")
    c, p = int(c[0]), int(p[0])
    return ComponentPlan(members[:n].copy(), offsets[:c + 1].copy(), ts[:p].copy(), te[:p].copy(),
                         po[:c + 1].copy())


def component_reduce(weights, indices, plan: ComponentPlan):
    weights = np.ascontiguousarray(weights, np.float32)
    indices = np.ascontiguousarray(indices, np.int32)
    n = weights.shape[0]
    c = plan.offsets.shape[0] - 1
    ww = np.empty(max(c, 1), np.float32)
    wm = np.empty((max(c, 1), 5), np.int32)
    members = np.ascontiguousarray(plan.members, np.int32)
    offsets = np.ascontiguousarray(plan.offsets, np.int32)
    _check(lib().orc_component_reduce(_p(weights, _F32P), _p(indices, _I32P), _p(members, _I32P),
                                      _p(offsets, _I32P), n, c, _p(ww, _F32P), _p(wm, _I32P)),
           "component_reduce")
    return ww[:c].copy(), wm[:c].copy()


@dataclass
class FitCore:
    knn_ids: np.ndarray
    knn_sq: np.ndarray
    core_sq: np.ndarray
    src: np.ndarray
    dst: np.ndarray
    wsq: np.ndarray
    rounds: int
    seed_edges: int
    components_after_seed: int
    round_components: list = field(default_factory=list)
    round_cross_pairs: list = field(default_factory=list)


def fit_core(x, min_samples: int) -> FitCore:
    """Exact brute-force fit core with production (kNN-seeded) semantics."""
    x = np.ascontiguousarray(x, np.float32)
    n, d = x.shape
    k = min(min_samples, n - 1)
    ids = np.empty((n, k), np.int32)
    ksq = np.empty((n, k), np.float32)
    core = np.empty(n, np.float32)
    src = np.empty(n, np.uint32)
    dst = np.empty(n, np.uint32)
    w = np.empty(n, np.float32)
    m = np.zeros(1, np.int64)
    maxr = 256
    rc_arr = np.zeros(maxr, np.int64)
    rp_arr = np.zeros(maxr, np.float64)
    st = _FitStats(0, 0, 0, _p(rc_arr, _I64P), _p(rp_arr, _F64P), maxr)
    _check(lib().orc_fit_core(_p(x, _F32P), n, d, min_samples, _p(ids, _I32P), _p(ksq, _F32P),
                              _p(core, _F32P), _p(src, _U32P), _p(dst, _U32P), _p(w, _F32P),
                              _p(m, _I64P), C.byref(st)), "fit_core")
    e = int(m[0])
    r = int(st.rounds)
    return FitCore(ids, ksq, core, src[:e].copy(), dst[:e].copy(), w[:e].copy(), r,
                   int(st.seed_edges), int(st.components_after_seed),
                   rc_arr[:min(r, maxr)].tolist(), rp_arr[:min(r, maxr)].tolist())


def brute_force_mst(x, min_samples: int, *, fused: bool = True):
    x = np.ascontiguousarray(x, np.float32)
    n, d = x.shape
    src = np.empty(max(n, 1), np.uint32)
    dst = np.empty(max(n, 1), np.uint32)
    w = np.empty(max(n, 1), np.float32)
    m = np.zeros(1, np.int64)
    _check(lib().orc_brute_force_mst(_p(x, _F32P), n, d, min_samples, int(fused), _p(src, _U32P),
                                     _p(dst, _U32P), _p(w, _F32P), _p(m, _I64P)), "brute_force_mst")
    e = int(m[0])
    return src[:e].copy(), dst[:e].copy(), w[:e].copy()


def finalize_mst(src, dst, wsq) -> np.ndarray:
    """Sorted [m, 3] float64 (src, dst, sqrt(w_sq)) by (weight, src, dst)."""
    src = np.ascontiguousarray(src, np.uint32)
    dst = np.ascontiguousarray(dst, np.uint32)
    wsq = np.ascontiguousarray(wsq, np.float32)
    m = src.shape[0]
    out = np.empty((max(m, 1), 3), np.float64)
    _check(lib().orc_finalize_mst(_p(src, _U32P), _p(dst, _U32P), _p(wsq, _F32P), m,
                                  _p(out, _F64P)), "finalize_mst")
    return out[:m].copy()


def pair_distances(x, y, *, fused: bool = True) -> np.ndarray:
    x = np.ascontiguousarray(x, np.float32)
    y = np.ascontiguousarray(y, np.float32)
    m, d = x.shape
    out = np.empty(m, np.float32)
    lib().orc_pair_distances(_p(x, _F32P), _p(y, _F32P), m, d, int(fused), _p(out, _F32P))
    return out


def prediction_cores(train, min_samples: int) -> np.ndarray:
    """Training prediction cores (self-inclusive rank s - 1, Euclidean f64)."""
    train = np.ascontiguousarray(train, np.float32)
    out = np.empty(train.shape[0], np.float64)
    _check(lib().orc_prediction_cores(_p(train, _F32P), train.shape[0], train.shape[1],
                                      int(min_samples), _p(out, _F64P)), "prediction_cores")
    return out


def predict_candidates(tree, labels, finite_index, min_samples: int, cores, ids, distances):
    """(labels, strengths, connecting points, no_cluster_tree) from candidate rows of width
    2 * min_samples (compact ids, Euclidean distances). ``tree`` has the condensed-tree fields
    parent, child, lambda_val, child_size (raw ids)."""
    parent = np.ascontiguousarray(tree["parent"], np.int64)
    child = np.ascontiguousarray(tree["child"], np.int64)
    lam = np.ascontiguousarray(tree["lambda_val"], np.float32)
    size = np.ascontiguousarray(tree["child_size"], np.float32)
    labels = np.ascontiguousarray(labels, np.int32)
    fi = np.ascontiguousarray(finite_index, np.uint32)
    cores = np.ascontiguousarray(cores, np.float64)
    ids = np.ascontiguousarray(ids, np.int32)
    distances = np.ascontiguousarray(distances, np.float64)
    m = ids.shape[0]
    out_l = np.empty(m, np.int32)
    out_s = np.empty(m, np.float64)
    out_c = np.empty(m, np.int32)
    nc = C.c_int(0)
    _check(lib().orc_predict_candidates(
        _p(parent, _I64P), _p(child, _I64P), _p(lam, _F32P), _p(size, _F32P), parent.shape[0],
        _p(labels, _I32P), labels.shape[0], _p(fi, _U32P), fi.shape[0], int(min_samples),
        _p(cores, _F64P), _p(ids, _I32P), _p(distances, _F64P), m, _p(out_l, _I32P),
        _p(out_s, _F64P), _p(out_c, _I32P), C.byref(nc)), "predict_candidates")
    return out_l, out_s, out_c, bool(nc.value)


def approximate_predict(tree, labels, finite_index, min_samples: int, train, queries,
                        cores=None):
    """The whole prediction on the CPU: exact self-inclusive candidates of width 2 s against the
    finite training rows, then the hierarchy math."""
    s = int(min_samples)
    train = np.ascontiguousarray(train, np.float32)
    queries = np.ascontiguousarray(queries, np.float32)
    if cores is None:
        cores = prediction_cores(train, s)
    ids, sq = exact_neighbors(queries, train, 2 * s, exclude_self=False)
    return predict_candidates(tree, labels, finite_index, s, cores, ids,
                              np.sqrt(sq.astype(np.float64)))
