"""Benchmark of the exact HDBSCAN fit core (kNN core distances + Borůvka MST) on one GB300.

One step = one complete fit core (exact kNN sweep, core distances, kNN seed, every Borůvka round
until a single component) over one synthetic point set of the named workload.

  value  : fit Mpts/s with the points already resident in HBM (device pointers)
  e2e    : the same metric through the host-pointer C ABI call cuscan_fit_core, with the
           host->device copy of the points and the device->host copy of every output inside
           the timed region (pinned host buffers)

Multi-GPU: the fit is not partitioned across devices here; under torchrun every rank fits its
own replica (seed + rank) and `value` is total points over the slowest rank's time ("replicas
only", scaling "weak").

`--impl reference` times the reference's CPU semantics (the C oracle restatement, all host
threads) on a bounded, extrapolated sample of the same workload.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "fit Mpts/s (core-dist+MST) BF16-refined vs FP32 vs CPU; serve p50/p99 at ARI=1"


def pinned_empty(shape, dtype):
    """An uninitialised numpy array of `dtype` in pinned (page-locked) host memory."""
    import torch
    count = int(np.prod(shape))
    raw = torch.empty(max(count, 1) * np.dtype(dtype).itemsize, dtype=torch.uint8,
                      pin_memory=True)
    return raw.numpy().view(dtype)[:count].reshape(shape)
L2_BYTES = 129 * 1024 * 1024


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=3)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--workload", default="vmf_500k_d128")
    p.add_argument("--n", type=int, default=None, help="override the workload's row count")
    p.add_argument("--precision", default="bf16_refined",
                   choices=["fp32", "bf16_refined", "fp16_refined"])
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-fp32-compare", action="store_true",
                   help="skip the plain f32 fit timed beside the bf16-refined one")
    p.add_argument("--cpu-seconds", type=float, default=15.0,
                   help="target CPU time of the bounded oracle sample")
    p.add_argument("--no-serve", action="store_true", help="skip the fit-request serving run")
    p.add_argument("--serve-only", action="store_true", help="run only the serving benchmark")
    p.add_argument("--serve-requests", type=int, default=10000)
    p.add_argument("--serve-pool", type=int, default=256,
                   help="distinct point sets the request stream cycles through")
    p.add_argument("--serve-slots", type=int, default=8)
    p.add_argument("--serve-precisions", default="bf16_refined,fp16_refined,fp32")
    p.add_argument("--mixed-predictors", type=int, default=64,
                   help="resident predictors of the mixed fit/predict stream (0: skip it)")
    p.add_argument("--mixed-requests", type=int, default=4000)
    p.add_argument("--mixed-precisions", default="fp16_refined,bf16_refined")
    p.add_argument("--serve-load", type=float, default=0.7,
                   help="Poisson arrival rate as a fraction of the measured saturation rate")
    return p.parse_args()


def dist_env():
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")),
            int(os.environ.get("LOCAL_RANK", "0")))


def algorithmic_flops(n: int, d: int, cross_pairs: float) -> tuple[float, float]:
    """GEMM-equivalent work: 2*d per ordered pair for the kNN sweep (n^2 pairs) and for every
    ordered cross-component pair of every Borůvka round."""
    return 2.0 * d * n * n, 2.0 * d * cross_pairs


class ClockSampler:
    """nvidia-smi SM clock and throttle reasons sampled every 200 ms while running."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines: list[str] = []
        self.thread = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            if self.thread:
                self.thread.join(timeout=2)

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx = float(parts[2])
            except ValueError:
                continue
            for name, flag in zip(names, parts[5:9]):
                if flag.lower() == "active":
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peaks():
    path = ROOT / "MEASURED_PEAKS.json"
    if path.exists():
        d = json.loads(path.read_text())
        return d.get("bf16_tflops"), d.get("hbm_gbs"), "measured"
    return 1900.0, 6800.0, "fallback"


# DRAM bytes (read + write) per launch of each screen kernel, from a one-pass ncu capture of
# the full-size workload (dram__bytes_read.sum + dram__bytes_write.sum): the kNN sweep (one
# launch per fit) and the mean over the Borůvka screen launches of one fit.
NCU_TRAFFIC = {"vmf_500k_d128:bf16_refined": {"knn_screen": 4888804352.0,
                                              "boruvka_candidates": 1182957504.0}}
NCU_TRAFFIC_SCOPE = {"knn_screen": "ncu dram read+write bytes of the kNN screen launch",
                     "boruvka_candidates": "ncu dram read+write bytes, mean per Borůvka screen "
                                           "launch"}


def ncu_traffic(workload: str, precision: str, n_override, kernel: str):
    """DRAM bytes per launch of `kernel` measured by ncu for this workload (at its own size),
    if any."""
    if n_override is not None:
        return None
    return NCU_TRAFFIC.get(f"{workload}:{precision}", {}).get(kernel)


class CpuSampler:
    """Times the oracle (the reference's CPU semantics, all host threads) on bounded samples of
    a workload and projects a full fit: kNN rows against all n points, and Borůvka candidate
    rows against the other half of the points, each extrapolated by the pairs the full fit
    evaluates (n^2 kNN pairs plus the fit's ordered cross-component pairs).

    The first call of each loop pays for thread start-up and page faults, so an untimed warm
    block runs first; the per-row cost is then calibrated on a block of several rows per
    thread, and every sample times at least `min_rows` rows per loop."""

    def __init__(self, x: np.ndarray, ms: int, cross_pairs: float, *, blocked: bool = False,
                 min_rows: int = 256):
        from oracle import oracle as O

        self.O = O
        self.x = x
        self.n, self.d = x.shape
        self.k = min(ms, self.n - 1)
        self.cross = cross_pairs
        self.blocked = blocked
        self.threads = O.max_threads()
        self.min_rows = min(self.n, max(min_rows, 2 * self.threads))
        self.labels = (np.arange(self.n) % 2).astype(np.int32)
        self.core = np.zeros(self.n, np.float32)
        warm = min(self.n, 2 * self.threads)
        self._knn(0, warm)
        self._cand(0, warm)
        calib = min(self.n, 4 * self.threads)
        t0 = time.perf_counter()
        self._knn(warm % self.n, calib)
        self.knn_row_s = (time.perf_counter() - t0) / calib

    def _knn(self, r0: int, rows: int):
        r0 = min(r0, self.n - rows)
        self.O.exact_neighbors(self.x[r0:r0 + rows], self.x, self.k, exclude_self=True,
                               query_offset=r0, blocked=self.blocked)

    def _cand(self, r0: int, rows: int):
        r0 = min(r0, self.n - rows)
        if self.blocked:
            # the blocked candidate loop runs whole point sets; rows against the other half of
            # the points through the blocked kNN loop with k = 1 have the same pair arithmetic
            other = self.x[1::2] if r0 % 2 == 0 else self.x[0::2]
            self.O.exact_neighbors(self.x[r0:r0 + rows], other, 1, exclude_self=False,
                                   blocked=True)
        else:
            self.O.boruvka_candidate_rows(self.x, self.core, self.labels, r0, r0 + rows)

    def rows_for(self, seconds: float) -> int:
        """Rows per loop so that one sample takes about `seconds` (at least min_rows)."""
        per_row = self.knn_row_s * 1.5  # kNN row plus a candidate row (half the pairs)
        return int(min(self.n, max(self.min_rows, seconds / max(per_row, 1e-9))))

    def sample(self, rows: int, offset: int = 0) -> dict:
        n = self.n
        r0 = (offset * rows) % max(n - rows, 1)
        t_start = time.perf_counter()
        t0 = time.perf_counter()
        self._knn(r0, rows)
        t_knn_row = (time.perf_counter() - t0) / rows
        t0 = time.perf_counter()
        self._cand(r0, rows)
        t_cand_pair = (time.perf_counter() - t0) / (rows * (n - n // 2))
        wall = time.perf_counter() - t_start
        t_total = t_knn_row * n + t_cand_pair * self.cross
        return {
            "value": n / t_total / 1e6,
            "unit": "Mpts/s",
            "cores": self.threads,
            "kind": "port",
            "loop": "blocked" if self.blocked else "row-at-a-time (the reference's loop)",
            "sample": (f"oracle kNN of {rows} rows vs all {n} and Borůvka candidates of {rows} "
                       f"rows vs the other half of the points (after an untimed warm block), "
                       f"extrapolated to n^2 kNN pairs + {self.cross:.4g} cross-component "
                       f"pairs ({t_total:.1f} s projected fit)"),
            "projected_fit_s": t_total,
            "sample_s": wall,
        }


def cpu_baseline(x: np.ndarray, ms: int, cross_pairs: float, target_s: float,
                 blocked: bool = False) -> dict:
    """One bounded, extrapolated sample of about `target_s` seconds of CPU work."""
    sampler = CpuSampler(x, ms, cross_pairs, blocked=blocked)
    return sampler.sample(sampler.rows_for(target_s))


# Ordered cross-component pairs summed over the Borůvka rounds of the exact fit of each named
# workload at its full size (from the fit statistics; the exact fit is deterministic and the
# same on every arithmetic path). The CPU reference arm extrapolates its per-pair cost with it.
CROSS_PAIRS = {
    "vmf_500k_d128": 942672776158.0,
    "aniso_100k_d64": 31806079898.0,
}


def serving_run(args, precision: str) -> dict:
    """Fit-request serving: a stream of Gaussian-mixture fits (n log-uniform in [500, 50000],
    d in {16, 32, 64, 128}) through the continuous-batching server. First the saturation rate
    (every request queued at once), then Poisson arrivals at `serve_load` times that rate with
    latency = arrival -> labels ready on the host."""
    import torch

    from cuscan_gb300 import synthetic
    from cuscan_gb300.serving import FitServer, default_budget

    specs = synthetic.fit_request_stream(args.serve_requests)
    pool_n = min(args.serve_pool, len(specs))
    pool = [synthetic.request_points(specs[i]) for i in range(pool_n)]
    budget = default_budget()  # 9/10 of free device memory less 64 MiB

    def kwargs(i):
        sp = specs[i % pool_n]
        return dict(min_cluster_size=sp["min_cluster_size"], min_samples=sp["min_samples"],
                    precision=precision)

    def run(count, rate, srv):
        """Submit `count` requests (all at once if rate is None, else Poisson arrivals) and
        collect every completion; returns per-request latency (ms) and the makespan (s)."""
        rng = np.random.default_rng(7)
        arrivals = (np.zeros(count) if rate is None
                    else np.cumsum(rng.exponential(1.0 / rate, size=count)))
        lag = {}
        lat, queued, points, failures, recs = [], [], 0, 0, []
        done = threading.Event()
        errors = []

        def collect():
            nonlocal points, failures
            got = 0
            try:
                while got < count:
                    rid = srv.wait_any(5.0)
                    if rid is None:
                        continue
                    info = srv.wait(rid, 0.0)
                    for _ in range(100000):
                        if rid in lag:
                            break
                        time.sleep(1e-4)
                    lat.append(lag[rid] + info["latency_ms"])
                    queued.append(info["queued_ms"])
                    st = info["stats"]
                    recs.append((info["n"], lat[-1], info["run_ms"], info["prep_ms"],
                                 info["fit_ms"], info["extract_ms"],
                                 st["core_ms"] + st["mst_ms"]))
                    points += info["n"]
                    failures += info["status"] != 0
                    srv.release(rid)
                    got += 1
            except BaseException as exc:  # surfaced by the submitting thread
                errors.append(exc)
            finally:
                done.set()

        th = threading.Thread(target=collect, daemon=True)
        th.start()
        t0 = time.perf_counter()
        for i in range(count):
            if errors:
                break
            target = t0 + arrivals[i]
            now = time.perf_counter()
            if target > now:
                time.sleep(target - now)
            sub = time.perf_counter()
            rid = srv.submit(pool[i % pool_n], **kwargs(i))
            lag[rid] = max(0.0, (sub - target) * 1e3)
        if not done.wait(timeout=600.0):
            raise RuntimeError("serving run did not finish within 600 s")
        makespan = time.perf_counter() - t0
        th.join()
        if errors:
            raise errors[0]
        return np.asarray(lat), np.asarray(queued), points, failures, makespan, np.asarray(recs)

    def by_size(recs):
        """Latency and where a request's time goes, per size class of n."""
        out = {}
        for lo, hi in ((500, 2000), (2000, 10000), (10000, 50001)):
            r = recs[(recs[:, 0] >= lo) & (recs[:, 0] < hi)]
            if len(r) == 0:
                continue
            out[f"n{lo}-{hi - 1}"] = {
                "requests": int(len(r)), "p50_ms": float(np.percentile(r[:, 1], 50)),
                "p99_ms": float(np.percentile(r[:, 1], 99)),
                "mean_run_ms": float(r[:, 2].mean()), "mean_prep_ms": float(r[:, 3].mean()),
                "mean_fit_ms": float(r[:, 4].mean()), "mean_extract_ms": float(r[:, 5].mean()),
                "mean_gpu_event_ms": float(r[:, 6].mean())}
        return out

    with FitServer(slots=args.serve_slots, budget_bytes=budget) as srv:
        warm = [srv.submit(pool[i % pool_n], **kwargs(i)) for i in range(2 * args.serve_slots)]
        for r in warm:
            srv.result(r, timeout=300.0)
        sat_count = min(len(specs), 2000)
        lat_s, _, pts_s, fail_s, span_s, _ = run(sat_count, None, srv)
        capacity = sat_count / span_s
        rate = args.serve_load * capacity
        lat, queued, pts, fails, span, recs = run(len(specs), rate, srv)
        st = srv.stats()
    return {
        "precision": precision, "requests": len(specs), "distinct_point_sets": pool_n,
        "slots": args.serve_slots, "budget_bytes": budget,
        "saturation": {"requests": sat_count, "req_per_s": capacity,
                       "mpts_per_s": pts_s / span_s / 1e6, "failures": int(fail_s)},
        "poisson": {"rate_req_per_s": rate, "load": args.serve_load,
                    "p50_ms": float(np.percentile(lat, 50)),
                    "p99_ms": float(np.percentile(lat, 99)), "max_ms": float(lat.max()),
                    "mean_ms": float(lat.mean()),
                    "queue_p99_ms": float(np.percentile(queued, 99)),
                    "req_per_s": len(specs) / span, "mpts_per_s": pts / span / 1e6,
                    "failures": int(fails), "by_size": by_size(recs)},
        "peak_committed_bytes": st["peak_committed_bytes"],
        "workspace_releases": st["workspace_releases"],
        "packs": st["packs"], "packed_requests": st["packed_requests"],
    }


def small_fit_packing_section(args) -> dict:
    """The small requests of the fit stream (n <= 2047 rows, every d of the stream), all queued
    at once, run with packing off (pack_limit 1: every fit on its own, about 26 launches and a
    host read per round each) and on (pack_limit 8, the default: each step one launch for all
    fits of a pack). Throughput and latency at saturation for both; the results are the same
    bits either way (GPU tests)."""
    import torch

    from cuscan_gb300 import _lib, synthetic
    from cuscan_gb300.serving import FitServer, default_budget

    specs = [sp for sp in synthetic.fit_request_stream(args.serve_requests)
             if sp["n"] <= _lib.PACK_MAX_ROWS][:1000]
    points = [synthetic.request_points(sp) for sp in specs]
    budget = default_budget()  # 9/10 of free device memory less 64 MiB
    out = {"requests": len(specs), "slots": args.serve_slots, "precision": "fp16_refined"}
    for limit in (1, 8):
        with FitServer(slots=args.serve_slots, budget_bytes=budget, pack_limit=limit) as srv:
            for rep_ in range(2):  # the first pass warms the slots' workspaces
                t0 = time.perf_counter()
                ids = [srv.submit(x, min_cluster_size=sp["min_cluster_size"],
                                  min_samples=sp["min_samples"], precision="fp16_refined")
                       for x, sp in zip(points, specs)]
                lat = [srv.wait(r, 300.0)["latency_ms"] for r in ids]
                span = time.perf_counter() - t0
                for r in ids:
                    srv.release(r)
            st = srv.stats()
        out[f"pack_limit_{limit}"] = {
            "req_per_s": len(specs) / span, "p50_ms": float(np.percentile(lat, 50)),
            "p99_ms": float(np.percentile(lat, 99)), "packs": st["packs"],
            "packed_requests": st["packed_requests"]}
    out["packing_speedup"] = (out["pack_limit_8"]["req_per_s"] /
                              out["pack_limit_1"]["req_per_s"])
    return out


def mixed_serving_section(args) -> dict:
    """Fit requests (the stream above) interleaved with approximate_predict batches (size
    log-uniform in [1, 4096]) against resident predictors, each fitted on n=100,000, d=64
    Gaussian mixtures of 40 blobs. Latency per request type; a sample of predictions is
    compared bit for bit with the same predictor's result computed alone."""
    import torch

    import cuscan_gb300 as cg
    from cuscan_gb300 import synthetic
    from cuscan_gb300.serving import FitServer, default_budget

    t_setup = time.perf_counter()
    npred = args.mixed_predictors
    predictors = []
    for i in range(npred):
        x = synthetic.gaussian_mixture(100_000, 64, 40, seed=9000 + i)
        model = cg.HDBSCAN(min_cluster_size=500, min_samples=5,
                           precision="fp16_refined").fit(x)
        predictors.append(model.to_predictor())
        del x
    rng = np.random.default_rng(11)
    pool_n = 256
    qsizes = np.exp(rng.uniform(np.log(1), np.log(4096), size=pool_n)).astype(np.int64)
    qpred = rng.integers(0, npred, size=pool_n)
    qpool = [synthetic.gaussian_mixture(int(qsizes[i]) + 7919, 64, 40,
                                        seed=9000 + int(qpred[i]))[-int(qsizes[i]):]
             for i in range(pool_n)]
    specs = synthetic.fit_request_stream(min(256, args.serve_requests))
    fpool = [synthetic.request_points(sp) for sp in specs]
    setup_s = time.perf_counter() - t_setup
    budget = default_budget()  # 9/10 of free device memory less 64 MiB
    out = {"predictors": npred, "predictor_training": "n=100000, d=64, 40 blobs, fp16_refined",
           "predict_batch": "log-uniform [1, 4096] rows", "setup_s": setup_s}

    def submit(srv, i, prec, kinds):
        if kinds[i]:
            j = i % pool_n
            return srv.submit_predict(predictors[int(qpred[j])], qpool[j])
        sp = specs[i % len(specs)]
        return srv.submit(fpool[i % len(fpool)], min_cluster_size=sp["min_cluster_size"],
                          min_samples=sp["min_samples"], precision=prec)

    def run(srv, count, rate, prec):
        rs = np.random.default_rng(5)
        kinds = rs.random(count) < 0.5
        arrivals = (np.zeros(count) if rate is None
                    else np.cumsum(rs.exponential(1.0 / rate, size=count)))
        lag, recs, errors = {}, [], []
        done = threading.Event()

        def collect():
            try:
                got = 0
                while got < count:
                    rid = srv.wait_any(5.0)
                    if rid is None:
                        continue
                    info = srv.wait(rid, 0.0)
                    for _ in range(100000):
                        if rid in lag:
                            break
                        time.sleep(1e-4)
                    recs.append((info["kind"], lag[rid] + info["latency_ms"], info["n"],
                                 info["status"]))
                    srv.release(rid)
                    got += 1
            except BaseException as exc:
                errors.append(exc)
            finally:
                done.set()

        th = threading.Thread(target=collect, daemon=True)
        th.start()
        t0 = time.perf_counter()
        for i in range(count):
            if errors:
                break
            target = t0 + arrivals[i]
            now = time.perf_counter()
            if target > now:
                time.sleep(target - now)
            sub = time.perf_counter()
            rid = submit(srv, i, prec, kinds)
            lag[rid] = max(0.0, (sub - target) * 1e3)
        if not done.wait(timeout=600.0):
            raise RuntimeError("mixed serving run did not finish within 600 s")
        span = time.perf_counter() - t0
        th.join()
        if errors:
            raise errors[0]
        return np.asarray(recs, dtype=np.float64), span

    for prec in args.mixed_precisions.split(","):
        with FitServer(slots=args.serve_slots, budget_bytes=budget) as srv:
            kinds = np.arange(2 * args.serve_slots) % 2 == 1
            for i in range(2 * args.serve_slots):
                srv.result(submit(srv, i, prec, kinds), timeout=300.0)
            sat, sat_span = run(srv, min(1000, args.mixed_requests), None, prec)
            capacity = sat.shape[0] / sat_span
            rate = args.serve_load * capacity
            recs, span = run(srv, args.mixed_requests, rate, prec)
            # a sample of predictions in the mix against the same predictor alone
            same = True
            for j in range(16):
                rid = srv.submit_predict(predictors[int(qpred[j])], qpool[j])
                r = srv.result(rid, timeout=60.0)
                lab, st, conn = predictors[int(qpred[j])].approximate_predict(
                    qpool[j], return_connecting_points=True)
                same &= (np.array_equal(r["labels"], lab) and np.array_equal(
                    r["strengths"].view(np.uint64), st.view(np.uint64)) and
                    np.array_equal(r["connecting_points"], conn))
        res = {"saturation_req_per_s": capacity, "rate_req_per_s": rate,
               "requests": int(recs.shape[0]), "req_per_s": recs.shape[0] / span,
               "failures": int(np.sum(recs[:, 3] != 0)), "predict_mix_equals_alone": bool(same)}
        for kind, name in ((0, "fit"), (1, "predict")):
            r = recs[recs[:, 0] == kind]
            if len(r):
                res[name] = {"requests": int(len(r)), "p50_ms": float(np.percentile(r[:, 1], 50)),
                             "p99_ms": float(np.percentile(r[:, 1], 99)),
                             "mean_rows": float(r[:, 2].mean())}
        out[prec] = res
    return out


def serving_section(args) -> dict:
    out = {"workload": "gaussian mixtures, n log-uniform [500, 50000], d in {16,32,64,128}, "
                       "2-30 blobs (std U[0.5,2]), min_samples 5, min_cluster_size max(5, n/200)",
           "latency": "arrival -> labels and strengths ready on the host"}
    for prec in args.serve_precisions.split(","):
        out[prec] = serving_run(args, prec)
    out["small_fit_packing"] = small_fit_packing_section(args)
    if args.mixed_predictors > 0:
        out["mixed"] = mixed_serving_section(args)
    return out


def serving_summary(serving: dict) -> dict:
    """The compact serving figures, kept in `config` (which survives truncation of the line):
    per precision the Poisson stream's p50/p99, the p99 of fits with n >= 10,000 and the
    saturation rate; the mixed stream's fit and predict p99; the packing speed-up."""
    out = {}
    for prec, res in serving.items():
        if not isinstance(res, dict) or "poisson" not in res:
            continue
        po = res["poisson"]
        big = po["by_size"].get("n10000-50000", {})
        out[prec] = {"p50_ms": round(po["p50_ms"], 2), "p99_ms": round(po["p99_ms"], 2),
                     "p99_n_ge_10000_ms": round(big.get("p99_ms", float("nan")), 2),
                     "saturation_req_per_s": round(res["saturation"]["req_per_s"], 1),
                     "poisson_req_per_s": round(po["req_per_s"], 1)}
    for prec, res in serving.get("mixed", {}).items():
        if isinstance(res, dict) and "fit" in res:
            out[f"mixed_{prec}"] = {
                "fit_p99_ms": round(res["fit"]["p99_ms"], 2),
                "predict_p99_ms": round(res.get("predict", {}).get("p99_ms", float("nan")), 2),
                "req_per_s": round(res["req_per_s"], 1),
                "predict_mix_equals_alone": res["predict_mix_equals_alone"]}
    pack = serving.get("small_fit_packing")
    if pack:
        out["packing_speedup"] = round(pack["packing_speedup"], 3)
    return out


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    from cuscan_gb300 import synthetic
    from oracle import oracle as O

    x, ms, mcs = synthetic.workload(args.workload, n=args.n)
    n, d = x.shape
    cross = CROSS_PAIRS.get(args.workload) if args.n is None else None
    cross_note = "recorded"
    if cross is None:  # unrecorded size: the recorded workloads sum to about 3.8 n^2
        cross, cross_note = 3.8 * n * n, "estimated as 3.8 n^2"
    # One sampler for the run: an untimed warm block and a calibration first, then the warm-up
    # steps untimed and every timed step the same number of rows (at least 256 per loop), so
    # that each step is a like-for-like bounded sample of the fit and not a cold start.
    sampler = CpuSampler(x, ms, cross)
    rows = sampler.rows_for(max(1.0, args.cpu_seconds / max(args.steps, 1)))
    for w in range(args.warmup):
        sampler.sample(sampler.min_rows, offset=w)
    samples = [sampler.sample(rows, offset=args.warmup + i) for i in range(args.steps)]
    values = [c["value"] for c in samples]
    value = float(np.median(values))
    cb = samples[len(samples) // 2]
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "Mpts/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        # a step is one bounded sample (wall time measured); the value projects a full fit
        "ms_per_step": float(np.median([c["sample_s"] for c in samples])) * 1e3,
        "projected": True,
        "projected_fit_ms": float(np.median([c["projected_fit_s"] for c in samples])) * 1e3,
        "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": args.workload, "n": n, "d": d, "min_samples": ms,
                   "min_cluster_size": mcs, "parallelism": "single",
                   "cross_pairs": cross, "cross_pairs_source": cross_note,
                   "rows_per_step": rows,
                   "value_spread": [float(min(values)), float(max(values))]},
        "cpu_baseline": {"value": value, "unit": "Mpts/s", "cores": O.max_threads(),
                         "kind": "port", "loop": cb["loop"], "sample": cb["sample"]},
        "e2e": {"value": value, "unit": "Mpts/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_ours(args):
    import torch

    import cuscan_gb300 as cg
    from cuscan_gb300 import _lib, replicas, synthetic

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")

    def barrier():
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()

    if args.serve_only:
        if rank == 0:
            print(json.dumps({"serving": serving_section(args)}), flush=True)
        return
    x, ms, mcs = synthetic.workload(args.workload, n=args.n)
    if world > 1 and rank > 0:  # independent replica per rank
        gen, kw, _, _ = synthetic.WORKLOADS[args.workload]
        kw = dict(kw, seed=replicas.replica_seed(kw["seed"], rank))
        if args.n:
            kw["n"] = args.n
        x = gen(**kw)
    n, d = x.shape
    k = min(ms, n - 1)
    prec = _lib.PRECISIONS[args.precision]
    ctx = cg.context(local)

    xd = torch.from_numpy(x).cuda()
    ids = torch.empty((n, k), dtype=torch.int32, device="cuda")
    ksq = torch.empty((n, k), dtype=torch.float32, device="cuda")
    core = torch.empty(n, dtype=torch.float32, device="cuda")
    src = torch.empty(n, dtype=torch.int32, device="cuda")
    dst = torch.empty(n, dtype=torch.int32, device="cuda")
    wsq = torch.empty(n, dtype=torch.float32, device="cuda")
    flush = torch.empty(2 * L2_BYTES // 4, dtype=torch.float32, device="cuda")
    stream = torch.cuda.ExternalStream(ctx.stream)

    def fit_once():
        return ctx.fit_core_device(xd.data_ptr(), n, d, ms, prec, ids.data_ptr(), ksq.data_ptr(),
                                   core.data_ptr(), src.data_ptr(), dst.data_ptr(),
                                   wsq.data_ptr(), ctx.stream)

    for _ in range(args.warmup):
        fit_once()
    torch.cuda.synchronize()

    step_ms = []
    screen_ms = []  # the kNN screen launch of every timed step
    stats = None
    launches0 = _lib.launch_count()
    barrier()
    with ClockSampler(local) as clocks:
        for _ in range(args.steps):
            flush.zero_()                      # evict the L2 between steps
            torch.cuda.synchronize()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            m, st = fit_once()
            e1.record(stream)
            e1.synchronize()
            step_ms.append(e0.elapsed_time(e1))
            stats = st.as_dict()
            screen_ms.append(stats["knn_screen_ms"])
            assert m == n - 1
        barrier()
    launches = _lib.launch_count() - launches0
    # per Borůvka round of the last timed fit: rows screened, tensor-core tiles run and their
    # share of a dense round's tiles (every query block against every tile)
    dense_tiles = -(-n // 128) * -(-n // 256)
    round_detail = [{"rows": r["rows"], "tiles": r["tiles"], "ms": round(r["ms"], 3),
                     "executed_tile_frac": round(r["tiles"] / dense_tiles, 4),
                     "cross_pair_frac": round(r["cross_pairs"] / (float(n) * n), 4)}
                    for r in ctx.round_stats()]
    pts_per_s, worst_s = replicas.aggregate_throughput(n, args.steps, float(np.sum(step_ms)) / 1e3,
                                                       device="cuda")
    ms_per_step = worst_s * 1e3 / args.steps
    value = pts_per_s / 1e6

    # end to end through the host-pointer C ABI (pinned host input and outputs)
    xh = torch.from_numpy(x).pin_memory().numpy()
    pinned = ctx.fit_core_outputs(n, ms, pinned_empty)
    ctx.fit_core(xh, ms, prec, out=pinned)
    torch.cuda.synchronize()
    e2e_t = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        ctx.fit_core(xh, ms, prec, out=pinned)
        e2e_t.append(time.perf_counter() - t0)
    e2e_pts_per_s, e2e_s = replicas.aggregate_throughput(n, args.steps, float(np.sum(e2e_t)),
                                                         device="cuda")
    h2d = n * d * 4
    d2h = n * k * 8 + n * 4 + (n - 1) * 12

    # the plain f32 form of the same fit, timed the same way (one step), for the comparison
    fp32 = None
    if args.precision != "fp32" and not args.no_fp32_compare:
        # the refined fit's outputs (the buffers are reused), compared bit for bit below
        outs = {"knn_ids": ids, "knn_sq": ksq, "core_sq": core, "src": src, "dst": dst,
                "wsq": wsq}
        refined_out = {key: t.clone() for key, t in outs.items()}
        flush.zero_()
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        _, st32 = ctx.fit_core_device(xd.data_ptr(), n, d, ms, _lib.PRECISION_PLAIN,
                                      ids.data_ptr(), ksq.data_ptr(), core.data_ptr(),
                                      src.data_ptr(), dst.data_ptr(), wsq.data_ptr(), ctx.stream)
        e1.record(stream)
        e1.synchronize()
        f_ms = e0.elapsed_time(e1)
        fp32 = {"value": n / (f_ms / 1e3) / 1e6, "unit": "Mpts/s", "ms_per_step": f_ms,
                "steps": 1, f"{args.precision}_speedup": f_ms / ms_per_step,
                # both forms emit the same edge list, so the f64 totals are the same bits
                "mst_weight_f64_equal": st32.mst_weight == stats["mst_weight"]}
        # kNN lists, core distances and the MST in merge order, bit for bit: equal edges give
        # equal labels (ARI 1.0) through the unchanged extraction
        fp32["outputs_bit_identical"] = all(
            torch.equal(refined_out[key].view(torch.int32), t.view(torch.int32))
            for key, t in outs.items())

    # roofline of the dominant kernel (CUDA events inside the fit, on its stream)
    bf16_peak, hbm_peak, peak_src = measured_peaks()
    w_knn, w_cand = algorithmic_flops(n, d, stats["cross_pairs"])
    t_knn = stats["knn_kernel_ms"] / 1e3
    t_cand = stats["candidate_kernel_ms"] / 1e3
    if stats["knn_screen_ms"] > 0:
        # the refined forms: the kNN screen launch, the largest kernel of the fit by device
        # time (ncu launch list), timed alone with CUDA events on the fit's stream
        dom, t_dom, w_dom = "knn_screen", float(np.mean(screen_ms)) / 1e3, w_knn
        achieved = w_dom / t_dom / 1e12
    elif t_knn >= t_cand:
        dom, achieved, t_dom, w_dom = "knn_sweep", w_knn / t_knn / 1e12, t_knn, w_knn
    else:
        dom = "boruvka_candidates"
        achieved, t_dom, w_dom = w_cand / t_cand / 1e12, t_cand, w_cand
    roof = {"bound": "tensor", "kernel": dom, "achieved": achieved, "peak": bf16_peak,
            "unit": "TFLOP/s", "frac": achieved / bf16_peak, "peak_source": f"{peak_src} bf16",
            "traffic": ncu_traffic(args.workload, args.precision, args.n, dom),
            "kernel_ms": t_dom * 1e3, "algorithmic_tflop": w_dom / 1e12,
            "knn_stage_ms": stats["knn_kernel_ms"]}
    if roof["traffic"] is not None:
        roof["traffic_scope"] = NCU_TRAFFIC_SCOPE[dom]
    if args.precision != "fp32":
        d_pad = -(-d // 64) * 64
        tiles = int(stats["screen_tile_pairs"])
        roof["tensor_tiles"] = tiles
        roof["tensor_tflop_executed"] = tiles * 2.0 * 128 * 256 * d_pad / 1e12
        roof["executed_frac_fit"] = (roof["tensor_tflop_executed"] * 1e12 / (t_knn + t_cand)
                                     / 1e12 / bf16_peak)
        roof["work_note"] = ("achieved is the named kernel's algorithmic work (the kNN screen: "
                             "2 d n^2, every ordered pair) over its mean launch time in the timed "
                             "steps; tensor_tflop_executed is what all screens of one fit ran "
                             "on the tensor cores, executed_frac_fit that work over the kNN and "
                             "Borůvka stage time against the same peak")
    if args.precision == "fp32":
        roof["note"] = ("plain form runs f32 direct differences on the SIMT pipes; the fraction "
                        "is against the measured bf16 tensor peak")

    line = {
        "metric": METRIC, "value": value, "unit": "Mpts/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_per_step,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": {"fp32": "f32", "bf16_refined": "bf16+f32", "fp16_refined": "fp16+f32"}[args.precision],
        "data": "synthetic",
        "config": {"workload": args.workload, "n": n, "d": d, "min_samples": ms,
                   "min_cluster_size": mcs, "precision": args.precision,
                   "parallelism": "replicas" if world > 1 else "single",
                   "l2": "flushed between steps (256 MiB write)",
                   "rounds": stats["rounds"], "components_after_seed":
                       stats["components_after_seed"],
                   "core_ms": stats["core_ms"], "mst_ms": stats["mst_ms"],
                   "knn_kernel_ms": stats["knn_kernel_ms"],
                   "knn_screen_ms": stats["knn_screen_ms"],
                   "candidate_kernel_ms": stats["candidate_kernel_ms"],
                   "knn_fallback_rows": stats["fallback_rows"],
                   "boruvka_fallback_rows": stats["boruvka_fallback_rows"],
                   "rescreened_rows": stats["rescreened_rows"],
                   "boruvka_screened_rows": stats["boruvka_screened_rows"],
                   "mst_weight_f64": stats["mst_weight"],
                   "operand_format": {-1: "none", 0: "bf16", 1: "fp16", 2: "split bf16"}[
                       int(stats["operand_format"])],
                   "boruvka_rounds": round_detail,
                   "algorithmic_tflop_per_step": (w_knn + w_cand) / 1e12},
        "clocks": clocks.summary(),
        "e2e": {"value": e2e_pts_per_s / 1e6, "unit": "Mpts/s",
                "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
        "gpu_launches": launches,
        "roofline": roof,
    }
    if fp32 is not None:
        line["fp32_plain"] = fp32
    if fp32 is not None:
        line["config"]["fp32_plain"] = {k2: fp32[k2] for k2 in (
            "ms_per_step", f"{args.precision}_speedup", "outputs_bit_identical",
            "mst_weight_f64_equal")}
    if rank == 0 and world == 1 and not args.no_serve:
        del xd, ids, ksq, core, src, dst, wsq, flush
        torch.cuda.empty_cache()
        line["serving"] = serving_section(args)
        line["config"]["serving_summary"] = serving_summary(line["serving"])
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = {k2: v for k2, v in cpu_baseline(
            x, ms, stats["cross_pairs"], args.cpu_seconds).items()
            if k2 not in ("projected_fit_s", "sample_s")}
        # context only: the oracle's blocked loops (same arithmetic, vectorised across
        # reference rows) on the same host cores; the baseline above is the reference's loop
        blk = cpu_baseline(x, ms, stats["cross_pairs"], args.cpu_seconds / 3, blocked=True)
        line["cpu_blocked"] = {"value": blk["value"], "unit": "Mpts/s", "cores": blk["cores"],
                               "sample": blk["sample"]}
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
