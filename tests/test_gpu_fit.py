"""Parity of the fused device fit core (kNN core distances + seeded Borůvka MST) with the CPU
oracle, through the C ABI, and of the estimator's labels with the reference fixtures.

Small and medium cases compare every output bit for bit, including the MST edge order (the
reference's merge order). The full-size case checks size-independent properties instead.
"""
from __future__ import annotations

import numpy as np
import pytest

import cuscan_gb300 as cg
from cuscan_gb300 import _lib, synthetic
from oracle import oracle as O
from tests.conftest import load_case

pytestmark = pytest.mark.gpu

PRECISIONS = [_lib.PRECISION_PLAIN, _lib.PRECISION_BF16_REFINED, _lib.PRECISION_FP16_REFINED]


def bits(a):
    return np.ascontiguousarray(a, np.float32).view(np.uint32)


def tree_sum(v: np.ndarray) -> np.ndarray:
    """Shared-memory tree of 256 lanes (lane t adds lane t + off for off = 128, 64, ..., 1)."""
    v = v.copy()
    off = v.shape[-1] // 2
    while off:
        v[..., :off] = v[..., :off] + v[..., off:2 * off]
        off //= 2
    return v[..., 0]


def device_order_weight(wsq: np.ndarray) -> float:
    """The f64 total MST weight summed in the device reduction's order: sqrt((double) w_sq)
    per edge, grid-stride accumulation over at most 256 blocks of 256 threads, a tree per
    block, then one tree over the partials."""
    w = np.sqrt(np.asarray(wsq, np.float32).astype(np.float64))
    m, lanes = w.size, 256
    grid = min(256, -(-m // lanes))
    stride = grid * lanes
    padded = np.zeros(-(-m // stride) * stride)
    padded[:m] = w
    acc = np.zeros((grid, lanes))
    for j in range(padded.size // stride):
        acc = acc + padded[j * stride:(j + 1) * stride].reshape(grid, lanes)
    partial = np.zeros(lanes)
    partial[:grid] = tree_sum(acc)
    return float(tree_sum(partial))


def assert_fit_equal(got, exp):
    np.testing.assert_array_equal(got["knn_ids"], exp.knn_ids)
    np.testing.assert_array_equal(bits(got["knn_sq"]), bits(exp.knn_sq))
    np.testing.assert_array_equal(bits(got["core_sq"]), bits(exp.core_sq))
    np.testing.assert_array_equal(got["src"], exp.src)
    np.testing.assert_array_equal(got["dst"], exp.dst)
    np.testing.assert_array_equal(bits(got["wsq"]), bits(exp.wsq))
    assert got["stats"]["rounds"] == exp.rounds
    assert got["stats"]["seed_edges"] == exp.seed_edges
    assert got["stats"]["mst_weight"] == device_order_weight(exp.wsq)


CASES = ["blobs_d2", "blobs_d10", "blobs_d50", "moons_leaf", "varying_density",
         "single_cluster", "duplicates_ties", "mixed_nonfinite", "overflow_finite",
         "persistence_equal", "selection_interactions", "all_noise", "two_finite", "padding",
         "n_below_min_samples"]


@pytest.mark.parametrize("precision", PRECISIONS)
@pytest.mark.parametrize("cid", CASES)
def test_fit_core_matches_oracle_on_fixtures(gpu_ctx, manifest, cid, precision):
    p = {c["id"]: c for c in manifest["cases"]}[cid]["params"]
    x = load_case(cid)["input"]
    x = np.ascontiguousarray(x[np.isfinite(x).all(axis=1)])
    got = gpu_ctx.fit_core(x, p["min_samples"], precision)
    assert_fit_equal(got, O.fit_core(x, p["min_samples"]))


def random_sets():
    rng = np.random.default_rng(7)
    yield "gauss", rng.normal(size=(500, 8)).astype(np.float32), 5
    yield "lattice_ties", rng.integers(0, 5, size=(800, 3)).astype(np.float32), 4
    base = rng.normal(size=(200, 6)).astype(np.float32)
    yield "duplicates", np.concatenate([base, base, base[:50]]), 3
    yield "ms1", rng.normal(size=(300, 4)).astype(np.float32), 1
    yield "ms_ge_n", rng.normal(size=(20, 4)).astype(np.float32), 25
    yield "line", np.arange(1000, dtype=np.float32)[:, None], 2
    yield "blobs_5k", synthetic.blobs_with_noise(n=5000, d=16, centers=12, seed=3), 10
    yield "aniso_8k", synthetic.anisotropic_mixture(n=8000, d=64, components=20, seed=4), 10
    yield "vmf_6k", synthetic.vmf_like(n=6000, d=128, clusters=30, seed=5), 15


@pytest.mark.parametrize("precision", PRECISIONS)
@pytest.mark.parametrize("name,x,ms", list(random_sets()), ids=lambda v: v if isinstance(v, str) else "")
def test_fit_core_matches_oracle_on_random_sets(gpu_ctx, name, x, ms, precision):
    got = gpu_ctx.fit_core(x, ms, precision)
    assert_fit_equal(got, O.fit_core(x, ms))


def test_fit_core_repeatable_and_buffers_reused(gpu_ctx):
    x = synthetic.blobs_with_noise(n=3000, d=10, seed=9)
    a = gpu_ctx.fit_core(x, 5)
    small = gpu_ctx.fit_core(x[:100], 5)
    b = gpu_ctx.fit_core(x, 5)
    for key in ("knn_ids", "src", "dst"):
        np.testing.assert_array_equal(a[key], b[key])
    np.testing.assert_array_equal(bits(a["wsq"]), bits(b["wsq"]))
    assert small["src"].shape[0] == 99


def test_c1_workload_labels_equal_oracle_labels():
    """blobs_2k_d10 (n=2000, d=10, 8 blobs + 5% noise, min_samples=5, mcs=5): labels, MST
    and core distances of the estimator equal those derived from the oracle's MST."""
    x, ms, mcs = synthetic.workload("blobs_2k_d10")
    model = cg.HDBSCAN(min_cluster_size=mcs, min_samples=ms).fit(x)
    fc = O.fit_core(x, ms)
    mst = O.finalize_mst(fc.src, fc.dst, fc.wsq)
    np.testing.assert_array_equal(model.minimum_spanning_tree_, mst)
    host = cg.clusters_from_spanning_tree(mst[:, 0].astype(np.uint32), mst[:, 1].astype(np.uint32),
                                          mst[:, 2], min_cluster_size=mcs)
    np.testing.assert_array_equal(model.labels_, host["labels"])
    np.testing.assert_array_equal(model.core_distances_, np.sqrt(fc.core_sq))
    assert len(set(model.labels_.tolist()) - {-1}) >= 2


@pytest.mark.parametrize("cid", ["blobs_d2", "blobs_d10", "blobs_d50", "moons_leaf",
                                 "varying_density", "single_cluster", "mixed_nonfinite",
                                 "overflow_finite", "persistence_equal",
                                 "selection_interactions"])
def test_estimator_matches_fixture_labels(manifest, cid):
    p = {c["id"]: c for c in manifest["cases"]}[cid]["params"]
    case = load_case(cid)
    model = cg.HDBSCAN(min_cluster_size=p["min_cluster_size"], min_samples=p["min_samples"],
                       cluster_selection_method=p["selection"],
                       allow_single_cluster=p["allow_single_cluster"],
                       max_cluster_size=p["max_cluster_size"],
                       cluster_selection_epsilon=float(p["epsilon"]),
                       cluster_selection_persistence=float(p["persistence"])).fit(case["input"])
    np.testing.assert_array_equal(model.labels_, case["labels"])
    assert np.all(np.abs(model.probabilities_ - case["probabilities"]) <= 1e-5)
    np.testing.assert_array_equal(model.minimum_spanning_tree_[:, :2], case["mst"][:, :2])
    np.testing.assert_array_equal(model.finite_index_, case["finite_index"])


def test_one_finite_row_contract():
    x = np.array([[np.nan, 1.0], [0.5, 0.5], [np.inf, 0.0]], np.float32)
    model = cg.HDBSCAN(min_cluster_size=2).fit(x)
    assert model.labels_.tolist() == [-1, -1, -1]
    assert model.finite_index_.tolist() == [1]


def check_tree_properties(x, out, ms):
    """Size-independent checks: n-1 edges forming a spanning tree, every edge weight the exact
    mutual reachability of its endpoints, core = kNN column, sampled kNN rows exact."""
    n = x.shape[0]
    src, dst, w = out["src"], out["dst"], out["wsq"]
    assert src.shape[0] == n - 1
    parent = np.arange(n)

    def find(a):
        while parent[a] != a:
            parent[a] = parent[parent[a]]
            a = parent[a]
        return a

    for a, b in zip(src.tolist(), dst.tolist()):
        ra, rb = find(a), find(b)
        assert ra != rb, "cycle"
        parent[ra] = rb
    d2 = O.pair_distances(x[src], x[dst])
    core = out["core_sq"]
    mrd = np.maximum(np.maximum(d2, core[src]), core[dst])
    np.testing.assert_array_equal(bits(w), bits(mrd))
    k = out["knn_ids"].shape[1]
    if ms < n:
        np.testing.assert_array_equal(bits(core), bits(out["knn_sq"][:, ms - 1]))
    rng = np.random.default_rng(0)
    rows = rng.choice(n, size=min(n, 256), replace=False)
    for r in rows[:64]:
        ids, ds = O.exact_neighbors(x[r:r + 1], x, k, exclude_self=True, query_offset=int(r))
        np.testing.assert_array_equal(out["knn_ids"][r], ids[0])
        np.testing.assert_array_equal(bits(out["knn_sq"][r]), bits(ds[0]))


def test_full_size_fp32_workload_properties(gpu_ctx):
    """aniso_100k_d64 (n=100000, d=64, min_samples=10) at full size."""
    x, ms, _ = synthetic.workload("aniso_100k_d64")
    out = gpu_ctx.fit_core(x, ms)
    check_tree_properties(x, out, ms)


@pytest.mark.parametrize("precision", PRECISIONS)
def test_medium_workload_matches_oracle_exactly(gpu_ctx, precision):
    x, ms, _ = synthetic.workload("aniso_100k_d64", n=20000)
    got = gpu_ctx.fit_core(x, ms, precision)
    assert_fit_equal(got, O.fit_core(x, ms))


def test_refined_vmf_matches_oracle_and_uses_tensor_screen(gpu_ctx):
    """vMF-like unit vectors (d=128, min_samples=15) at n=30000: the bf16 screen handles the
    rows and the result equals the oracle bit for bit."""
    x = synthetic.vmf_like(n=30000, d=128, clusters=40, seed=12)
    got = gpu_ctx.fit_core(x, 15, _lib.PRECISION_BF16_REFINED)
    assert got["stats"]["refined_rows"] == x.shape[0]
    assert got["stats"]["fallback_rows"] < 0.05 * x.shape[0] * (1 + got["stats"]["rounds"])
    assert_fit_equal(got, O.fit_core(x, 15))


@pytest.mark.parametrize("precision", [_lib.PRECISION_BF16_REFINED, _lib.PRECISION_FP16_REFINED])
def test_far_blobs_match_oracle(gpu_ctx, precision):
    """Gaussian blobs far from the origin (centres in [-10, 10]^64, std 0.5-2): norms are large
    against the neighbour distances. The plain bf16 bound leaves most kNN rows inconclusive, so
    the bf16-refined fit screens again with split-bf16 operands and keeps them for its rounds;
    the fp16 screen leaves hundreds of rows to the threshold re-screen. Both equal the oracle
    bit for bit."""
    x = synthetic.gaussian_mixture(20000, 64, 25, seed=20064)
    got = gpu_ctx.fit_core(x, 5, precision)
    if precision == _lib.PRECISION_BF16_REFINED:
        assert got["stats"]["operand_format"] == 2
    else:
        assert got["stats"]["operand_format"] == 1
        assert got["stats"]["rescreened_rows"] >= 256
        assert got["stats"]["fallback_rows"] < got["stats"]["rescreened_rows"]
    assert_fit_equal(got, O.fit_core(x, 5))


def test_wide_far_blobs_tighten_to_fp16_and_match_oracle(gpu_ctx):
    """The same kind of data at d = 128, where a split tile does not fit the pipeline: the
    bf16-refined fit tightens to scaled fp16 operands and equals the oracle bit for bit."""
    x = synthetic.gaussian_mixture(12000, 128, 20, seed=12128)
    got = gpu_ctx.fit_core(x, 5, _lib.PRECISION_BF16_REFINED)
    assert got["stats"]["operand_format"] == 1
    assert_fit_equal(got, O.fit_core(x, 5))


def test_full_size_refined_equals_plain(gpu_ctx):
    """vmf_500k_d128 reduced to n=150000 (large enough for the symmetric Borůvka screen):
    bf16-refined and plain fits agree bit for bit."""
    x, ms, _ = synthetic.workload("vmf_500k_d128", n=150000)
    a = gpu_ctx.fit_core(x, ms, _lib.PRECISION_PLAIN)
    b = gpu_ctx.fit_core(x, ms, _lib.PRECISION_BF16_REFINED)
    # the headline kind of data keeps bf16 operands; the rows its lists leave inconclusive go
    # through the bf16 threshold re-screen
    print(f"[vmf 150k] rescreened {b['stats']['rescreened_rows']}, "
          f"exact {b['stats']['fallback_rows']}")
    assert b["stats"]["operand_format"] == 0
    assert b["stats"]["rescreened_rows"] >= 256
    for key in ("knn_ids", "src", "dst"):
        np.testing.assert_array_equal(a[key], b[key])
    for key in ("knn_sq", "core_sq", "wsq"):
        np.testing.assert_array_equal(bits(a[key]), bits(b[key]))
    check_tree_properties(x, b, ms)


def test_large_blobs_fp16_equals_plain(gpu_ctx):
    """Gaussian blobs far from the origin at n=140000 (symmetric screen where the rows have
    bounds, one-sided rounds where many do not): fp16-refined and plain agree bit for bit."""
    x = synthetic.gaussian_mixture(140000, 32, 30, seed=140032)
    a = gpu_ctx.fit_core(x, 5, _lib.PRECISION_PLAIN)
    b = gpu_ctx.fit_core(x, 5, _lib.PRECISION_FP16_REFINED)
    for key in ("knn_ids", "src", "dst"):
        np.testing.assert_array_equal(a[key], b[key])
    for key in ("knn_sq", "core_sq", "wsq"):
        np.testing.assert_array_equal(bits(a[key]), bits(b[key]))
    check_tree_properties(x, b, 5)


@pytest.mark.parametrize("failure", ["invalid", "unsupported", "overflow", "native"])
def test_failed_refit_preserves_fitted_state(failure, monkeypatch):
    """A refit that fails leaves every fitted attribute as it was (the reference's
    python/tests/test_hdbscan.py:585-637)."""
    import cuscan_gb300.hdbscan as hmod
    x = load_case("blobs_d2")["input"]
    model = cg.HDBSCAN(min_cluster_size=5, min_samples=5).fit(x)
    names = ("labels_", "probabilities_", "condensed_tree_", "single_linkage_tree_",
             "minimum_spanning_tree_", "core_distances_")
    before = {name: np.array(getattr(model, name), copy=True) for name in names}
    cut_before = model.dbscan_clustering(0.2).copy()
    refit = x
    if failure == "invalid":
        model.min_cluster_size = 0
        error = ValueError
    elif failure == "unsupported":
        model.metric = "manhattan"
        error = NotImplementedError
    elif failure == "overflow":
        refit = np.array([[1e100, 0.0], [0.0, 0.0]])
        error = ValueError
    else:
        def injected(*args, **kwargs):
            raise RuntimeError("injected fit-core failure")
        monkeypatch.setattr(hmod, "fit_hdbscan", injected)
        error = RuntimeError
    with pytest.raises(error):
        model.fit(refit)
    for name, value in before.items():
        np.testing.assert_array_equal(getattr(model, name), value)
    np.testing.assert_array_equal(model.dbscan_clustering(0.2), cut_before)


def test_reused_context_buffers_carry_no_state_between_fits():
    """A context keeps its device buffers between fits. Per-fit state in them (row lower
    bounds and component bounds of the Borůvka screens, the fp16 operand scale, split-kNN
    partials) must not leak from one point set into the next: fits of new data of the same
    size on a used context equal the same fits on a fresh context, bit for bit."""
    first = synthetic.vmf_like(n=30000, d=128, clusters=40, seed=41)
    blobs = synthetic.gaussian_mixture(30000, 128, 25, seed=42)
    vmf = synthetic.vmf_like(n=30000, d=128, clusters=25, seed=43)
    used = _lib.Context(0)
    try:
        used.fit_core(first, 15, _lib.PRECISION_BF16_REFINED)
        got = [used.fit_core(blobs, 5, _lib.PRECISION_FP16_REFINED),
               used.fit_core(vmf, 15, _lib.PRECISION_BF16_REFINED),
               used.fit_core(blobs, 5, _lib.PRECISION_BF16_REFINED)]
    finally:
        used.close()
    cases = [(blobs, 5, _lib.PRECISION_FP16_REFINED), (vmf, 15, _lib.PRECISION_BF16_REFINED),
             (blobs, 5, _lib.PRECISION_BF16_REFINED)]
    for (x, ms, prec), a in zip(cases, got):
        fresh = _lib.Context(0)
        try:
            b = fresh.fit_core(x, ms, prec)
        finally:
            fresh.close()
        for key in ("knn_ids", "src", "dst"):
            np.testing.assert_array_equal(a[key], b[key])
        for key in ("knn_sq", "core_sq", "wsq"):
            np.testing.assert_array_equal(bits(a[key]), bits(b[key]))
        assert a["stats"]["mst_weight"] == b["stats"]["mst_weight"]


def refined_edge_sets():
    """Point sets that reach the tensor-core screens (n >= 2048) with the cases the reference's
    tie and padding rules decide: exact duplicate rows, integer lattices (massive distance ties
    across tiles), feature counts that are not multiples of the 64-feature K block, ragged last
    tiles, min_samples of 1 and above the list capacity, and magnitudes at the ends of the fp16
    operand scale."""
    rng = np.random.default_rng(2048)
    base = rng.normal(size=(1200, 24)).astype(np.float32)
    yield "duplicates", np.concatenate([base, base, base[:700]]), 5
    yield "lattice_d3", rng.integers(0, 12, size=(4000, 3)).astype(np.float32), 6
    yield "lattice_d70", rng.integers(0, 3, size=(2500, 70)).astype(np.float32), 4
    yield "odd_d100", synthetic.blobs_with_noise(n=3001, d=100, centers=9, seed=8), 7
    yield "ms1", synthetic.blobs_with_noise(n=2600, d=16, centers=5, seed=9), 1
    yield "ms40", synthetic.blobs_with_noise(n=2600, d=32, centers=5, seed=10), 40
    yield "tiny", (synthetic.blobs_with_noise(n=3000, d=20, seed=11) * np.float32(1e-30)), 5
    yield "identical", np.ones((2500, 12), np.float32), 5
    two = np.zeros((3000, 8), np.float32)
    two[1::2] = 3.0
    yield "two_points", two, 7
    yield "line_d1", np.arange(3000, dtype=np.float32)[:, None], 3
    yield "n2048_ms32", synthetic.vmf_like(n=2048, d=128, clusters=8, seed=14), 32
    # just inside the screens' range (d max|x|^2 about FLT_MAX / 64): the screens run
    big = synthetic.blobs_with_noise(n=3000, d=20, seed=13)
    yield "large", big * np.float32(np.sqrt(3.4e38 / 64 / 20) / np.abs(big).max()), 5
    # squared norms and distances overflow f32: exact weights tie at +inf, so the refined
    # forms hand the fit to the exact kernels
    yield "huge", (synthetic.blobs_with_noise(n=3000, d=20, seed=12) * np.float32(1e18)), 5


@pytest.mark.parametrize("precision", PRECISIONS)
@pytest.mark.parametrize("name,x,ms", list(refined_edge_sets()),
                         ids=lambda v: v if isinstance(v, str) else "")
def test_refined_edge_cases_match_oracle(gpu_ctx, name, x, ms, precision):
    got = gpu_ctx.fit_core(x, ms, precision)
    assert_fit_equal(got, O.fit_core(x, ms))
    if precision != _lib.PRECISION_PLAIN:
        on_screens = name not in ("huge", "ms40")  # ms40: k above the screens' list capacity
        assert (got["stats"]["refined_rows"] > 0) == on_screens


def test_symmetric_boruvka_screen_equals_plain(gpu_ctx):
    """Every point three times (n = 150,000, min_samples 5): each kNN row holds two exact
    duplicates and three points of other groups, so every component has a bound from a
    crossing kNN edge and every row's core is below it. The first round screens every row with
    the symmetric screen (each unordered pair once, column-side appends). Both refined forms
    equal the plain form bit for bit."""
    rng = np.random.default_rng(3)
    x = np.repeat(rng.random((50000, 8), dtype=np.float32), 3, axis=0)
    a = gpu_ctx.fit_core(x, 5, _lib.PRECISION_PLAIN)
    for precision in (_lib.PRECISION_BF16_REFINED, _lib.PRECISION_FP16_REFINED):
        b = gpu_ctx.fit_core(x, 5, precision)
        assert b["stats"]["symmetric_rounds"] >= 1, "no round ran the symmetric screen"
        for key in ("knn_ids", "src", "dst"):
            np.testing.assert_array_equal(a[key], b[key])
        for key in ("knn_sq", "core_sq", "wsq"):
            np.testing.assert_array_equal(bits(a[key]), bits(b[key]))


def test_fit_core_into_caller_outputs(gpu_ctx):
    """fit_core writes into caller-allocated outputs (pinned memory in the bench) exactly what it
    returns in fresh arrays, and rejects arrays too small for the fit."""
    x = synthetic.blobs_with_noise(n=3000, d=16, seed=21)
    fresh = gpu_ctx.fit_core(x, 5, _lib.PRECISION_BF16_REFINED)
    out = gpu_ctx.fit_core_outputs(3000, 5)
    got = gpu_ctx.fit_core(x, 5, _lib.PRECISION_BF16_REFINED, out=out)
    for key in ("knn_ids", "src", "dst"):
        np.testing.assert_array_equal(got[key], fresh[key])
    for key in ("knn_sq", "core_sq", "wsq"):
        np.testing.assert_array_equal(bits(got[key]), bits(fresh[key]))
    assert got["core_sq"] is out["core_sq"]
    with pytest.raises(ValueError):
        gpu_ctx.fit_core(x, 5, out=gpu_ctx.fit_core_outputs(2999, 5))


@pytest.mark.parametrize("precision", [_lib.PRECISION_PLAIN, _lib.PRECISION_BF16_REFINED])
def test_round_stats_and_row_selection(gpu_ctx, precision):
    """cuscan_fit_round_stats reports one entry per Borůvka round of the last fit. From 2048
    rows both the screened and the exact rounds scan only the rows that can hold their
    component's cheapest edge: the per-round rows add up to boruvka_screened_rows, stay within
    n, fall below n in a later round, and the fit still equals the oracle."""
    x = synthetic.blobs_with_noise(n=20_000, d=16, centers=40, seed=12)
    got = gpu_ctx.fit_core(x, 5, precision)
    assert_fit_equal(got, O.fit_core(x, 5))
    st = got["stats"]
    rounds = gpu_ctx.round_stats()
    assert len(rounds) == st["rounds"] >= 2
    rows = [r["rows"] for r in rounds]
    assert all(0 <= r <= x.shape[0] for r in rows)
    assert sum(rows) == st["boruvka_screened_rows"]
    assert min(rows[1:]) < x.shape[0]
    cross = [r["cross_pairs"] for r in rounds]
    assert all(a >= b for a, b in zip(cross, cross[1:]))
    if precision == _lib.PRECISION_PLAIN:
        assert all(r["tiles"] == 0 for r in rounds)
