"""Parity of the three backend operations (exact kNN, Borůvka candidates, component reduce)
with the CPU oracle, called through the C ABI on device buffers. Integer and float results are
compared bit for bit."""
from __future__ import annotations

import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def ptr(t):
    return t.data_ptr()


def stream():
    return torch.cuda.current_stream().cuda_stream


def gpu_knn(ctx, q, r, k, exclude_self=True, offset=0, squared=True):
    q = np.ascontiguousarray(q, np.float32)
    r = np.ascontiguousarray(r, np.float32)
    tq, tr = dev(q), dev(r)
    ids = torch.empty((q.shape[0], k), dtype=torch.int32, device="cuda")
    ds = torch.empty((q.shape[0], k), dtype=torch.float32, device="cuda")
    ctx.exact_knn(ptr(tq), q.shape[0], ptr(tr), r.shape[0], q.shape[1], k, exclude_self, offset,
                  squared, ptr(ids), ptr(ds), stream())
    torch.cuda.synchronize()
    return ids.cpu().numpy(), ds.cpu().numpy()


def bits(a):
    return np.ascontiguousarray(a, np.float32).view(np.uint32)


@pytest.mark.parametrize("n,d,k,seed", [(1, 3, 1, 0), (2, 2, 3, 1), (37, 3, 5, 2),
                                        (300, 10, 8, 3), (1000, 64, 10, 4), (2050, 128, 15, 5),
                                        (700, 17, 16, 6), (513, 33, 32, 7), (400, 9, 40, 8),
                                        (3000, 20, 1, 9)])
def test_exact_knn_matches_oracle(gpu_ctx, n, d, k, seed):
    rng = np.random.default_rng(seed)
    x = rng.normal(size=(n, d)).astype(np.float32)
    ids, ds = gpu_knn(gpu_ctx, x, x, k)
    eids, eds = O.exact_neighbors(x, x, k)
    np.testing.assert_array_equal(ids, eids)
    np.testing.assert_array_equal(bits(ds), bits(eds))


def _self_knn_sets():
    from cuscan_gb300 import synthetic

    yield "vmf_6k_d128", synthetic.vmf_like(n=6000, d=128, seed=3), 15
    yield "blobs_far_5k_d64", (synthetic.blobs_with_noise(n=5000, d=64, seed=4) + 200.0).astype(
        np.float32), 10
    yield "normal_4k_d20_k1", np.random.default_rng(5).normal(size=(4000, 20)).astype(np.float32), 1
    yield "normal_3k_d33_k32", np.random.default_rng(6).normal(size=(3000, 33)).astype(np.float32), 32


@pytest.mark.parametrize("name,x,k", list(_self_knn_sets()), ids=lambda v: v if isinstance(v, str) else "")
def test_exact_knn_of_a_set_against_itself_takes_the_screen_and_stays_exact(gpu_ctx, name, x, k):
    """From 2048 rows the kNN of a point set against itself runs the tensor-core screen with
    exact re-rank (falling back to the exact sweep where the screen cannot decide); its ids and
    squared distances equal the oracle's bit for bit, including far-from-origin data that needs
    the tightened operands."""
    ids, ds = gpu_knn(gpu_ctx, x, x, k)
    eids, eds = O.exact_neighbors(x, x, k)
    np.testing.assert_array_equal(ids, eids)
    np.testing.assert_array_equal(bits(ds), bits(eds))


def test_exact_knn_ties_duplicates_and_lattice(gpu_ctx):
    rng = np.random.default_rng(11)
    base = rng.integers(0, 4, size=(300, 3)).astype(np.float32)   # many exact ties
    x = np.concatenate([base, base[:50]])                          # exact duplicates
    for k in (1, 5, 16, 33):
        ids, ds = gpu_knn(gpu_ctx, x, x, k)
        eids, eds = O.exact_neighbors(x, x, k)
        np.testing.assert_array_equal(ids, eids)
        np.testing.assert_array_equal(bits(ds), bits(eds))


def test_exact_knn_padding_offset_and_unsquared(gpu_ctx):
    # crates/cuscan-common/src/neighbors.rs:440-465
    q = np.array([[10.0], [20.0]], np.float32)
    r = np.array([[0.0], [10.0], [20.0]], np.float32)
    ids, ds = gpu_knn(gpu_ctx, q, r, 3, True, 1, True)
    assert ids.ravel().tolist() == [0, 2, 3, 1, 0, 3]
    np.testing.assert_array_equal(ds.ravel(),
                                  np.array([100, 100, np.inf, 100, 400, np.inf], np.float32))
    ids, ds = gpu_knn(gpu_ctx, np.zeros((1, 1)), np.zeros((1, 1)), 2)
    assert ids.ravel().tolist() == [1, 1] and np.all(np.isinf(ds))
    rng = np.random.default_rng(5)
    x = rng.normal(size=(64, 4)).astype(np.float32)
    ids, ds = gpu_knn(gpu_ctx, x, x, 70, True, 0, False)
    eids, eds = O.exact_neighbors(x, x, 70, squared=False)
    np.testing.assert_array_equal(ids, eids)
    np.testing.assert_array_equal(bits(ds), bits(eds))


def test_exact_knn_overflow_tail(gpu_ctx):
    # neighbors.rs:407-438 (k = 1300 takes the wide path)
    query = (np.arange(701) % 17).astype(np.float32)
    query[700] = np.finfo(np.float32).max
    ref = ((np.arange(763) * 7) % 23).astype(np.float32)
    ref[12:713] = query
    ids, ds = gpu_knn(gpu_ctx, query[:, None], ref[:, None], 1300, True, 12)
    eids, eds = O.exact_neighbors(query[:, None], ref[:, None], 1300, exclude_self=True,
                                  query_offset=12)
    np.testing.assert_array_equal(ids, eids)
    np.testing.assert_array_equal(bits(ds), bits(eds))


def gpu_candidates(ctx, x, core, comp):
    n, d = x.shape
    tx, tc, tl = dev(x.astype(np.float32)), dev(core.astype(np.float32)), dev(comp.astype(np.int32))
    w = torch.empty(n, dtype=torch.float32, device="cuda")
    j = torch.empty(n, dtype=torch.int32, device="cuda")
    ctx.boruvka_candidates(ptr(tx), ptr(tc), ptr(tl), n, d, ptr(w), ptr(j), stream())
    torch.cuda.synchronize()
    return w.cpu().numpy(), j.cpu().numpy()


@pytest.mark.parametrize("n,comps", [(1, 1), (2, 2), (257, 2), (513, 7)])
def test_candidates_reference_cases(gpu_ctx, n, comps):
    # crates/hdbscan/tests/test_candidates.rs:8-77
    i = np.arange(n)
    x = np.stack([((i * 17 + i // 7) % 97) * 0.125, ((i * 11) % 53) * 0.25,
                  (i % 13).astype(np.float64)], 1).astype(np.float32)
    core = ((i % 9) * 0.125).astype(np.float32)
    comp = ((i * 7 + i // 19) % comps).astype(np.int32)
    w, j = gpu_candidates(gpu_ctx, x, core, comp)
    ew, ej = O.boruvka_candidates(x, core, comp)
    np.testing.assert_array_equal(bits(w), bits(ew))
    np.testing.assert_array_equal(j, ej)


@pytest.mark.parametrize("n,d,comps,seed", [(1000, 16, 3, 0), (3000, 64, 40, 1),
                                            (2048, 128, 1000, 2), (5000, 10, 2, 3)])
def test_candidates_random(gpu_ctx, n, d, comps, seed):
    rng = np.random.default_rng(seed)
    x = rng.normal(size=(n, d)).astype(np.float32)
    core = rng.uniform(0, 2 * d, size=n).astype(np.float32)
    core[rng.random(n) < 0.3] = 0.0
    comp = rng.integers(0, comps, size=n).astype(np.int32)
    w, j = gpu_candidates(gpu_ctx, x, core, comp)
    ew, ej = O.boruvka_candidates(x, core, comp)
    np.testing.assert_array_equal(bits(w), bits(ew))
    np.testing.assert_array_equal(j, ej)


def test_candidates_infinite_cores_pick_lowest_index(gpu_ctx):
    x = np.random.default_rng(3).normal(size=(100, 5)).astype(np.float32)
    core = np.full(100, np.inf, np.float32)
    comp = (np.arange(100) % 4).astype(np.int32)
    w, j = gpu_candidates(gpu_ctx, x, core, comp)
    ew, ej = O.boruvka_candidates(x, core, comp)
    np.testing.assert_array_equal(j, ej)
    assert np.all(np.isinf(w))


def gpu_reduce(ctx, w, dst, plan, n):
    c = plan.offsets.shape[0] - 1
    p = plan.tile_starts.shape[0]
    t = [dev(a) for a in (w.astype(np.float32), dst.astype(np.int32), plan.members,
                          plan.tile_starts if p else np.zeros(1, np.int32),
                          plan.tile_ends if p else np.zeros(1, np.int32), plan.partial_offsets)]
    ww = torch.empty(max(c, 1), dtype=torch.float32, device="cuda")
    wm = torch.empty((max(c, 1), 5), dtype=torch.int32, device="cuda")
    ctx.component_reduce(*[ptr(a) for a in t], n, p, c, ptr(ww), ptr(wm), stream())
    torch.cuda.synchronize()
    return ww.cpu().numpy()[:c], wm.cpu().numpy()[:c]


@pytest.mark.parametrize("n,comps,tile,seed", [(4, 2, 2, 0), (600, 7, 512, 1), (5000, 3, 512, 2),
                                               (3000, 900, 64, 3), (10000, 1, 512, 4)])
def test_component_reduce_matches_oracle(gpu_ctx, n, comps, tile, seed):
    rng = np.random.default_rng(seed)
    labels = rng.integers(0, comps, size=n).astype(np.int32)
    plan = O.component_plan(labels, tile)
    w = rng.integers(0, 50, size=n).astype(np.float32)       # heavy key ties
    w[rng.random(n) < 0.05] = -0.0
    w[rng.random(n) < 0.05] = np.inf
    dst = rng.integers(0, n, size=n).astype(np.int32)
    dst[rng.random(n) < 0.05] = -1
    if seed % 2:
        w[rng.random(n) < 0.01] = np.nan
        dst[rng.random(n) < 0.01] = n + 3
    ww, wm = gpu_reduce(gpu_ctx, w, dst, plan, n)
    eww, ewm = O.component_reduce(w, dst, plan)
    np.testing.assert_array_equal(wm, ewm)
    np.testing.assert_array_equal(bits(ww), bits(eww))


@pytest.mark.parametrize("n,d,seed", [(512, 128, 0), (600, 64, 1), (300, 10, 2), (1000, 100, 3)])
def test_tensor_core_tile_matches_bf16_products(gpu_ctx, n, d, seed):
    """The tcgen05 screen's raw accumulator for query rows 0..127 x reference rows 0..255
    equals the dot products of the bf16-rounded rows (f32 accumulation tolerance)."""
    rng = np.random.default_rng(seed)
    x = rng.normal(size=(n, d)).astype(np.float32)
    tx = dev(x)
    out = torch.zeros((128, 256), dtype=torch.float32, device="cuda")
    gpu_ctx.debug_screen_tile(ptr(tx), n, d, ptr(out), stream())
    torch.cuda.synchronize()
    got = out.cpu().numpy().astype(np.float64)
    xb = torch.from_numpy(x).to(torch.bfloat16).to(torch.float64).numpy()
    cols = min(256, n)
    exp = xb[:128] @ xb[:cols].T
    scale = np.abs(xb[:128]) @ np.abs(xb[:cols]).T
    err = np.abs(got[:, :cols] - exp)
    assert np.all(err <= 1e-5 * scale + 1e-30), float(np.max(err / np.maximum(scale, 1e-30)))


def _chunk_max_data(kind: str, n: int, d: int) -> np.ndarray:
    rng = np.random.default_rng(d + len(kind))
    if kind == "normal":
        return rng.normal(size=(n, d)).astype(np.float32)
    if kind == "negative_dots":  # queries and references on opposite sides: all dots < 0
        x = np.abs(rng.normal(size=(n, d))) + 0.1
        x[:128] *= -1.0
        return x.astype(np.float32)
    if kind == "ties":  # few distinct values: many equal dots, signed zeros
        return rng.integers(-1, 2, size=(n, d)).astype(np.float32)
    if kind == "wide_range":
        return (rng.normal(size=(n, d)) * np.exp2(rng.integers(-20, 20, size=(n, 1)))).astype(
            np.float32)
    raise ValueError(kind)


@pytest.mark.parametrize("d", [64, 128])
@pytest.mark.parametrize("kind", ["normal", "negative_dots", "ties", "wide_range"])
def test_chunk_maxima_equal_the_tile_maxima(gpu_ctx, kind, d):
    """The screens take each row's largest dot product per 32-column chunk from the TMEM load
    itself (tcgen05.ld.red .max): it must equal the maximum of the 32 loaded accumulator values
    bit for bit, for every row of the 128-row block and every chunk of the 256-column tile
    (lane r holds row r, chunk h covers columns 32 h .. 32 h + 31)."""
    n = 512
    x = _chunk_max_data(kind, n, d)
    tx = dev(x)
    out = torch.zeros((128, 256), dtype=torch.float32, device="cuda")
    chunks = torch.full((128, 8), float("nan"), dtype=torch.float32, device="cuda")
    gpu_ctx.debug_screen_tile(ptr(tx), n, d, ptr(out), stream(), chunk_out=ptr(chunks))
    torch.cuda.synchronize()
    tile = out.cpu().numpy()
    got = chunks.cpu().numpy()
    expect = tile.reshape(128, 8, 32).max(axis=2)
    assert not np.isnan(got).any()
    np.testing.assert_array_equal(bits(np.abs(got)), bits(np.abs(expect)))
    np.testing.assert_array_equal(got, expect)


def test_component_reduce_clamps_a_malformed_plan(gpu_ctx):
    """Plan arrays that overrun their buffers (partial offsets past p, tile ends past n, member
    ids >= n) are clamped instead of read out of bounds: the result equals the same call on
    the clamped plan."""
    rng = np.random.default_rng(21)
    n = 3000
    labels = rng.integers(0, 40, size=n).astype(np.int32)
    plan = O.component_plan(labels, 64)
    w = rng.integers(0, 50, size=n).astype(np.float32)
    dst = rng.integers(0, n, size=n).astype(np.int32)
    p = plan.tile_starts.shape[0]
    bad = O.ComponentPlan(plan.members.copy(), plan.offsets, plan.tile_starts.copy(),
                          plan.tile_ends.copy(), plan.partial_offsets.copy())
    bad.partial_offsets[-1] = p + 1000          # past the last partial
    bad.tile_ends[-1] = n + 77                  # past the member array
    bad.members[5] = n + 9                      # a member id outside the points
    fixed = O.ComponentPlan(bad.members.copy(), bad.offsets, bad.tile_starts,
                            np.minimum(bad.tile_ends, n).astype(np.int32),
                            np.minimum(bad.partial_offsets, p).astype(np.int32))
    fixed.members[5] = 0
    w_fixed = w.copy()
    # member 5's slot now names point 0; give point 0 a weight that cannot win so that skipping
    # the bad id and reading point 0 give the same reduction
    w_fixed[0] = np.inf
    w[0] = np.inf
    ww_bad, wm_bad = gpu_reduce(gpu_ctx, w, dst, bad, n)
    ww_fix, wm_fix = gpu_reduce(gpu_ctx, w_fixed, dst, fixed, n)
    np.testing.assert_array_equal(wm_bad, wm_fix)
    np.testing.assert_array_equal(bits(ww_bad), bits(ww_fix))
