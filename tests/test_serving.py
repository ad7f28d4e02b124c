"""Fit-request server: admission by memory budget and queue order on the scheduling test double
(CPU), and on the GPU that every result equals the same fit run alone."""
from __future__ import annotations

import numpy as np
import pytest

from cuscan_gb300 import _lib, synthetic
from cuscan_gb300.serving import FitServer


def bound(n, d, ms=5, precision=_lib.PRECISION_BF16_REFINED):
    return _lib.fit_workspace_bytes(n, d, ms, precision)


def drain(server, ids, timeout=30.0):
    infos = {}
    for rid in ids:
        info = server.wait(rid, timeout)
        assert info is not None, f"request {rid} did not finish"
        infos[rid] = info
    return infos


def test_usable_bytes_follows_the_reference_admission_rule():
    """usable = min(9/10 free (exact integer form) + live, limit, total) - 64 MiB, saturating
    at 0 (crates/cuscan-common/src/memory.rs:17-40)."""
    from cuscan_gb300.serving import MEMORY_RESERVE_BYTES, usable_bytes

    mib, gib = 1 << 20, 1 << 30
    assert MEMORY_RESERVE_BYTES == 64 * mib
    # 9/10 of 100 GiB less the reserve
    assert usable_bytes(100 * gib, 200 * gib) == 90 * gib - 64 * mib
    # rounding of the tenth: (19 // 10) * 9 + (19 % 10) * 9 // 10 = 9 + 8
    assert usable_bytes(19 + 64 * mib * 10, 1 << 62) == (64 * mib * 9 + 17) - 64 * mib
    # bytes already held count on top of the free share; the total and the limit cap the sum
    assert usable_bytes(10 * gib, 100 * gib, live_bytes=5 * gib) == 14 * gib - 64 * mib
    assert usable_bytes(10 * gib, 8 * gib, live_bytes=5 * gib) == 8 * gib - 64 * mib
    assert usable_bytes(10 * gib, 100 * gib, limit_bytes=2 * gib) == 2 * gib - 64 * mib
    # below the reserve nothing is usable
    assert usable_bytes(0, 100 * gib) == 0
    assert usable_bytes(70 * mib, 100 * gib) == 0
    with pytest.raises(ValueError):
        usable_bytes(-1, 100 * gib)


def test_workspace_bound_grows_with_shape():
    small, big = bound(1000, 16), bound(50000, 128)
    assert 0 < small < big
    assert bound(5000, 64, precision=_lib.PRECISION_PLAIN) < bound(5000, 64)
    assert _lib.fit_workspace_bytes(1, 4, 5, 0) == 0


def test_budget_is_never_exceeded_and_admission_is_fifo():
    budget = 3 * bound(20000, 64) + (1 << 20)
    rng = np.random.default_rng(0)
    shapes = [(int(rng.integers(500, 20000)), int(rng.choice([16, 32, 64]))) for _ in range(40)]
    with FitServer(slots=4, budget_bytes=budget, simulated_us_per_kpoint=200.0) as srv:
        ids = [srv.submit(np.zeros((1, d), np.float32).repeat(n, 0), min_cluster_size=5)
               for n, d in shapes]
        infos = drain(srv, ids)
        st = srv.stats()
    assert st["completed"] == 40 and st["failed"] == 0
    assert st["peak_committed_bytes"] <= budget
    admitted = [infos[r]["submit_ms"] + infos[r]["queued_ms"] for r in ids]
    assert all(b >= a - 1e-6 for a, b in zip(admitted, admitted[1:])), "admission out of order"
    assert all(infos[r]["status"] == _lib.OK for r in ids)
    assert {infos[r]["slot"] for r in ids} <= {0, 1, 2, 3}


def test_request_larger_than_budget_fails_with_memory_error():
    with FitServer(slots=2, budget_bytes=bound(2000, 16), simulated_us_per_kpoint=1.0) as srv:
        rid = srv.submit(np.zeros((100000, 64), np.float32), min_cluster_size=5)
        with pytest.raises(MemoryError):
            srv.result(rid, timeout=5.0)
        ok = srv.submit(np.zeros((1000, 16), np.float32), min_cluster_size=5)
        info = srv.wait(ok, 5.0)
        assert info["status"] == _lib.OK


def test_idle_workspace_is_released_for_a_large_request():
    big = bound(40000, 128)
    budget = big + bound(4000, 64) // 2
    with FitServer(slots=3, budget_bytes=budget, simulated_us_per_kpoint=50.0) as srv:
        small = [srv.submit(np.zeros((4000, 64), np.float32), min_cluster_size=5)
                 for _ in range(6)]
        drain(srv, small)
        assert srv.stats()["committed_bytes"] > 0  # idle slots keep their workspace
        rid = srv.submit(np.zeros((40000, 128), np.float32), min_cluster_size=5)
        assert srv.wait(rid, 10.0)["status"] == _lib.OK
        st = srv.stats()
    assert st["workspace_releases"] >= 1
    assert st["peak_committed_bytes"] <= budget


def test_wait_times_out_and_wait_any_reports_each_request_once():
    with FitServer(slots=1, budget_bytes=1 << 34, simulated_us_per_kpoint=20000.0) as srv:
        slow = srv.submit(np.zeros((20000, 4), np.float32), min_cluster_size=2)   # ~0.4 s
        queued = srv.submit(np.zeros((10, 4), np.float32), min_cluster_size=2)
        assert srv.wait(queued, 0.01) is None
        seen = [srv.wait_any(5.0), srv.wait_any(5.0)]
        assert seen == [slow, queued]
        assert srv.wait_any(0.01) is None
        with pytest.raises(ValueError):  # the test double computes no result
            srv.result(slow)
        again = srv.submit(np.zeros((10, 4), np.float32), min_cluster_size=2)
        srv.wait(again, 5.0)
        srv.release(again)                 # released before wait_any saw it
        assert srv.wait_any(0.01) is None


def test_close_with_queued_requests_returns():
    srv = FitServer(slots=1, budget_bytes=1 << 34, simulated_us_per_kpoint=5000.0)
    for _ in range(5):
        srv.submit(np.zeros((20000, 4), np.float32), min_cluster_size=2)  # 0.1 s each
    srv.close()


def test_invalid_server_and_request_arguments():
    with pytest.raises(ValueError):
        FitServer(slots=0, budget_bytes=1 << 30, simulated_us_per_kpoint=1.0)
    with FitServer(slots=1, budget_bytes=1 << 30, simulated_us_per_kpoint=1.0) as srv:
        with pytest.raises(ValueError):
            srv.submit(np.zeros((0, 3), np.float32))
        with pytest.raises(ValueError):
            srv.submit(np.zeros((10, 3), np.float32), precision="fp16")
        with pytest.raises(ValueError):
            srv.submit(np.zeros((10, 3), np.float32), min_cluster_size=0)
        for prec in ("fp32", "bf16_refined", "fp16_refined"):
            rid = srv.submit(np.zeros((10, 3), np.float32), precision=prec)
            assert srv.wait(rid, 5.0)["status"] == _lib.OK


def test_small_fits_behind_a_small_head_run_as_one_pack():
    with FitServer(slots=1, budget_bytes=1 << 34, pack_limit=8,
                   simulated_us_per_kpoint=2000.0) as srv:
        blocker = srv.submit(np.zeros((20000, 8), np.float32))  # occupies the slot ~40 ms
        sizes = [1000] * 10 + [30000] + [500] * 3
        ids = [srv.submit(np.zeros((n, 8), np.float32)) for n in sizes]
        infos = drain(srv, [blocker] + ids)
        st = srv.stats()
    packs = [infos[r]["pack_size"] for r in ids]
    # the first eight small fits form one pack, the next two a second one (the large request
    # behind them is never overtaken), the last three a third one
    assert packs == [8] * 8 + [2] * 2 + [1] + [3] * 3, packs
    assert st["packs"] == 3 and st["packed_requests"] == 13
    assert infos[blocker]["pack_size"] == 1
    admitted = [infos[r]["submit_ms"] + infos[r]["queued_ms"] for r in ids]
    assert all(b >= a - 1e-6 for a, b in zip(admitted, admitted[1:])), "admission out of order"
    assert len({infos[r]["slot"] for r in ids[:8]}) == 1


def test_fits_outside_the_packed_limits_run_on_their_own():
    with FitServer(slots=1, budget_bytes=1 << 34, pack_limit=8,
                   simulated_us_per_kpoint=2000.0) as srv:
        blocker = srv.submit(np.zeros((20000, 8), np.float32))
        wide = _lib.PACK_MAX_FEATURES + 1
        shapes = [(1000, 8), (1000, wide), (1000, 8), (1000, 8)]
        ids = [srv.submit(np.zeros(s, np.float32)) for s in shapes]
        infos = drain(srv, [blocker] + ids)
    assert [infos[r]["pack_size"] for r in ids] == [1, 1, 2, 2]


def test_pack_stays_within_the_budget():
    small = bound(2000, 64)
    budget = 3 * small + (1 << 20)
    with FitServer(slots=1, budget_bytes=budget, pack_limit=16,
                   simulated_us_per_kpoint=2000.0) as srv:
        blocker = srv.submit(np.zeros((2000, 64), np.float32))
        ids = [srv.submit(np.zeros((2000, 64), np.float32)) for _ in range(9)]
        infos = drain(srv, [blocker] + ids)
        st = srv.stats()
    assert st["peak_committed_bytes"] <= budget
    assert max(infos[r]["pack_size"] for r in ids) <= 2  # held workspace + two bounds fit
    assert st["completed"] == 10 and st["failed"] == 0


def test_pack_limit_one_runs_every_fit_alone():
    with FitServer(slots=1, budget_bytes=1 << 34, pack_limit=1,
                   simulated_us_per_kpoint=2000.0) as srv:
        ids = [srv.submit(np.zeros((1000, 8), np.float32)) for _ in range(6)]
        infos = drain(srv, ids)
        assert srv.stats()["packs"] == 0
    assert all(infos[r]["pack_size"] == 1 for r in ids)
    for bad in (0, _lib.PACK_MAX_FITS + 1):
        with pytest.raises(ValueError):
            FitServer(slots=1, budget_bytes=1 << 30, pack_limit=bad, simulated_us_per_kpoint=1.0)


def host_predictor():
    from cuscan_gb300.prediction import Predictor
    labels = np.array([0, 0, 0, 1, 1, 1], np.int32)
    rows = [(6, 7, 1.0, 3.0), (6, 8, 1.0, 3.0)] + [(7, i, 2.0, 1.0) for i in range(3)] + \
           [(8, i, 2.0, 1.0) for i in range(3, 6)]
    t = np.array(rows, dtype=[("parent", np.int64), ("child", np.int64),
                              ("lambda_val", np.float64), ("child_size", np.float64)])
    return Predictor(condensed_tree=t, labels=labels, finite_index=np.arange(6, dtype=np.uint32),
                     min_samples=2, n_features=3, prediction_core=np.zeros(6))


def test_predict_requests_share_the_queue_with_fits():
    pred = host_predictor()
    with FitServer(slots=2, budget_bytes=1 << 32, simulated_us_per_kpoint=100.0) as srv:
        ids = []
        for i in range(20):
            if i % 2:
                ids.append(srv.submit_predict(pred, np.zeros((1 + 50 * i, 3), np.float32)))
            else:
                ids.append(srv.submit(np.zeros((2000, 3), np.float32), min_cluster_size=5))
        infos = drain(srv, ids)
        assert [infos[r]["kind"] for r in ids] == [i % 2 for i in range(20)]
        assert all(infos[r]["status"] == _lib.OK for r in ids)
        with pytest.raises(ValueError):  # the test double computes no result
            srv.result(ids[1])
        with pytest.raises(ValueError):
            srv.submit_predict(pred, np.zeros((4, 2), np.float32))   # wrong feature count
        with pytest.raises(ValueError):
            srv.submit_predict(pred, np.full((4, 3), np.nan, np.float32))


# ---------------------------------------------------------------- GPU ----------------------

def request_mix():
    rng = np.random.default_rng(21)
    out = []
    for i, (n, d) in enumerate([(600, 16), (2500, 32), (9000, 64), (4000, 128), (12000, 16),
                                (3000, 64), (800, 128), (20000, 32)]):
        x = synthetic.blobs_with_noise(n=n, d=d, centers=int(rng.integers(2, 30)), seed=100 + i)
        out.append((x, max(5, n // 200), "bf16_refined" if i % 3 else "fp32"))
    x = synthetic.blobs_with_noise(n=3000, d=16, centers=6, seed=7)
    x[::97, 3] = np.nan
    x[5, 0] = np.inf
    out.append((x, 15, "bf16_refined"))
    return out


@pytest.mark.gpu
def test_results_in_the_mix_equal_fits_alone():
    import cuscan_gb300 as cg
    mix = request_mix()
    alone = []
    for x, mcs, prec in mix:
        m = cg.HDBSCAN(min_cluster_size=mcs, min_samples=5, precision=prec).fit(x)
        alone.append(m)
    with FitServer(slots=4, budget_bytes=8 << 30) as srv:
        ids = [srv.submit(x, min_cluster_size=mcs, min_samples=5, precision=prec)
               for x, mcs, prec in mix]
        results = [srv.result(r, timeout=120.0) for r in ids]
        st = srv.stats()
    assert st["completed"] == len(mix) and st["failed"] == 0
    assert max(r["info"]["slot"] for r in results) > 0  # more than one slot was used
    for m, r in zip(alone, results):
        np.testing.assert_array_equal(r["labels"], m.labels_)
        np.testing.assert_array_equal(r["probabilities"].view(np.uint32),
                                      np.asarray(m.probabilities_, np.float32).view(np.uint32))
        np.testing.assert_array_equal(r["core_distances"].view(np.uint32),
                                      np.asarray(m.core_distances_, np.float32).view(np.uint32))
        np.testing.assert_array_equal(r["minimum_spanning_tree"], m.minimum_spanning_tree_)


@pytest.mark.gpu
def test_packed_small_fits_equal_fits_alone():
    import cuscan_gb300 as cg
    rng = np.random.default_rng(33)
    mix = []
    for i in range(24):
        n = int(np.exp(rng.uniform(np.log(40), np.log(2047))))
        d = int(rng.choice([16, 32, 64, 128]))
        x = synthetic.gaussian_mixture(n, d, int(rng.integers(2, 30)), seed=500 + i)
        if i == 5:
            x[::7, 1] = np.nan  # rows set aside before the packed fit core
        mix.append((x, max(5, n // 200), ("bf16_refined", "fp16_refined", "fp32")[i % 3]))
    alone = [cg.HDBSCAN(min_cluster_size=mcs, min_samples=5, precision=prec).fit(x)
             for x, mcs, prec in mix]
    with FitServer(slots=2, budget_bytes=8 << 30, pack_limit=8) as srv:
        ids = [srv.submit(x, min_cluster_size=mcs, min_samples=5, precision=prec)
               for x, mcs, prec in mix]
        results = [srv.result(r, timeout=120.0) for r in ids]
        st = srv.stats()
    assert st["completed"] == len(mix) and st["failed"] == 0
    assert st["packs"] > 0 and max(r["info"]["pack_size"] for r in results) > 1
    for m, r in zip(alone, results):
        np.testing.assert_array_equal(r["labels"], m.labels_)
        np.testing.assert_array_equal(r["probabilities"].view(np.uint32),
                                      np.asarray(m.probabilities_, np.float32).view(np.uint32))
        np.testing.assert_array_equal(r["core_distances"].view(np.uint32),
                                      np.asarray(m.core_distances_, np.float32).view(np.uint32))
        np.testing.assert_array_equal(r["minimum_spanning_tree"], m.minimum_spanning_tree_)


@pytest.mark.gpu
def test_results_repeat_across_submissions():
    x, mcs, _ = request_mix()[2]
    with FitServer(slots=3, budget_bytes=4 << 30) as srv:
        ids = [srv.submit(x, min_cluster_size=mcs, min_samples=5) for _ in range(6)]
        res = [srv.result(r, timeout=120.0) for r in ids]
    for r in res[1:]:
        np.testing.assert_array_equal(r["labels"], res[0]["labels"])
        np.testing.assert_array_equal(r["minimum_spanning_tree"], res[0]["minimum_spanning_tree"])


@pytest.mark.gpu
@pytest.mark.parametrize("n,d,ms,prec", [(500, 16, 5, 0), (3000, 128, 15, 1), (20000, 64, 10, 1),
                                         (50000, 128, 5, 1), (7000, 32, 40, 0)])
def test_workspace_bound_covers_a_fit(n, d, ms, prec):
    ctx = _lib.Context(0)
    try:
        x = synthetic.blobs_with_noise(n=n, d=d, seed=n)
        ctx.fit_core(x, ms, prec)
        held = ctx.reserved_bytes()
        assert 0 < held <= _lib.fit_workspace_bytes(n, d, ms, prec)
        ctx.release_workspace()
        assert ctx.reserved_bytes() == 0
    finally:
        ctx.close()


@pytest.mark.gpu
def test_predictions_in_the_mix_equal_predictions_alone():
    import cuscan_gb300 as cg
    models, queries = [], []
    for i, (n, d) in enumerate([(6000, 16), (9000, 64)]):
        x = synthetic.gaussian_mixture(n, d, 12, seed=300 + i)
        models.append(cg.HDBSCAN(min_cluster_size=30, min_samples=5,
                                 precision="fp16_refined").fit(x))
        queries.append([synthetic.gaussian_mixture(m, d, 12, seed=300 + i) + np.float32(0.05)
                        for m in (1, 17, 400, 3000)])
    alone = [[m.approximate_predict(q, return_connecting_points=True) for q in qs]
             for m, qs in zip(models, queries)]
    preds = [m.to_predictor() for m in models]
    mix = request_mix()
    with FitServer(slots=4, budget_bytes=8 << 30) as srv:
        ids = []
        for j in range(4):
            for i in range(2):
                ids.append(("p", i, j, srv.submit_predict(preds[i], queries[i][j])))
            x, mcs, prec = mix[j]
            ids.append(("f", j, None, srv.submit(x, min_cluster_size=mcs, min_samples=5,
                                                 precision=prec)))
        results = [(kind, i, j, srv.result(r, timeout=120.0)) for kind, i, j, r in ids]
    for kind, i, j, r in results:
        if kind != "p":
            continue
        lab, st, conn = alone[i][j]
        np.testing.assert_array_equal(r["labels"], lab)
        np.testing.assert_array_equal(r["strengths"].view(np.uint64), st.view(np.uint64))
        np.testing.assert_array_equal(r["connecting_points"], conn)
