"""Packed small fits (cuscan_fit_core_packed): several fit cores together, each step of every
fit in one launch, the Borůvka rounds of finished fits skipped on the device.

Every fit of a pack must equal the same fit run alone through cuscan_fit_core, and the oracle,
bit for bit: kNN ids and distances, core distances, MST edges in merge order, round and seed
counts, and the f64 total weight.
"""
from __future__ import annotations

import numpy as np
import pytest

from cuscan_gb300 import _lib, synthetic
from oracle import oracle as O
from tests.conftest import load_case
from tests.test_gpu_fit import assert_fit_equal, bits

pytestmark = pytest.mark.gpu


def small_sets():
    rng = np.random.default_rng(11)
    yield rng.normal(size=(500, 8)).astype(np.float32), 5, _lib.PRECISION_PLAIN
    yield rng.integers(0, 5, size=(800, 3)).astype(np.float32), 4, _lib.PRECISION_BF16_REFINED
    base = rng.normal(size=(200, 6)).astype(np.float32)
    yield np.concatenate([base, base, base[:50]]), 3, _lib.PRECISION_FP16_REFINED
    yield rng.normal(size=(300, 4)).astype(np.float32), 1, _lib.PRECISION_PLAIN
    yield rng.normal(size=(20, 4)).astype(np.float32), 25, _lib.PRECISION_PLAIN
    yield np.arange(1000, dtype=np.float32)[:, None], 2, _lib.PRECISION_PLAIN
    yield rng.normal(size=(2, 5)).astype(np.float32), 5, _lib.PRECISION_PLAIN
    yield synthetic.blobs_with_noise(n=2047, d=128, centers=12, seed=3), 10, \
        _lib.PRECISION_BF16_REFINED
    yield synthetic.blobs_with_noise(n=1500, d=10, seed=42), 5, _lib.PRECISION_PLAIN
    x = load_case("blobs_d50")["input"]
    yield np.ascontiguousarray(x[np.isfinite(x).all(axis=1)]), 5, _lib.PRECISION_PLAIN


def test_pack_equals_alone_and_oracle(gpu_ctx):
    fits = list(small_sets())
    packed = gpu_ctx.fit_core_packed(fits)
    for (x, ms, prec), got in zip(fits, packed):
        assert got["status"] == _lib.OK
        alone = gpu_ctx.fit_core(x, ms, prec)
        for key in ("knn_ids", "src", "dst"):
            np.testing.assert_array_equal(got[key], alone[key])
        for key in ("knn_sq", "core_sq", "wsq"):
            np.testing.assert_array_equal(bits(got[key]), bits(alone[key]))
        for key in ("rounds", "seed_edges", "components_after_seed", "cross_pairs",
                    "mst_weight"):
            assert got["stats"][key] == alone["stats"][key], key
        assert_fit_equal(got, O.fit_core(x, ms))


def test_consecutive_packs_reuse_the_workspace(gpu_ctx):
    rng = np.random.default_rng(5)
    for sizes in ([1800, 40, 700], [64, 2000, 9, 1200, 333], [2047] * 16):
        fits = [(synthetic.blobs_with_noise(n=n, d=int(rng.choice([16, 32, 64])),
                                            centers=int(rng.integers(2, 30)),
                                            seed=int(rng.integers(1 << 30))), 5,
                 _lib.PRECISION_BF16_REFINED) for n in sizes]
        packed = gpu_ctx.fit_core_packed(fits)
        assert len(packed) == len(fits)
        for (x, ms, _), got in zip(fits, packed):
            assert_fit_equal(got, O.fit_core(x, ms))


def test_pack_launches_each_step_once_for_all_fits():
    """A pack launches each step once for all of its fits: the kNN lists (and their merge), the
    seed, four launches per round and the weight, with one host read of the round counter
    after the first three rounds and after every two more. The counts do not grow with the
    number of fits, and every result still equals the oracle."""
    ctx = _lib.Context(0)
    rng = np.random.default_rng(9)
    for count in (1, 5, 16):
        fits = [(synthetic.blobs_with_noise(n=int(rng.integers(300, 2048)),
                                            d=int(rng.choice([8, 32, 64])),
                                            centers=int(rng.integers(2, 20)),
                                            seed=int(rng.integers(1 << 30))), 5,
                 _lib.PRECISION_FP16_REFINED) for _ in range(count)]
        packed = ctx.fit_core_packed(fits)
        rounds = max(got["stats"]["rounds"] for got in packed)
        for (x, ms, _), got in zip(fits, packed):
            assert_fit_equal(got, O.fit_core(x, ms))
        st = ctx.packed_launch_stats()
        launched = 3 if rounds <= 3 else 3 + 2 * ((rounds - 2) // 2)
        assert st["host_reads"] == 1 + (launched - 3) // 2, (st, rounds)
        # kNN (+ merge), seed, four per round launched, weight
        assert st["launches"] in (3 + 4 * launched, 4 + 4 * launched), (st, rounds)


def test_pack_with_wide_lists_and_tiny_fits(gpu_ctx):
    """k > 32 takes the per-fit kNN launch inside the pack; fits of 2 and 3 rows, and a fit
    whose min_samples exceeds its rows, sit beside ordinary ones."""
    rng = np.random.default_rng(21)
    fits = [(rng.normal(size=(400, 6)).astype(np.float32), 40, _lib.PRECISION_PLAIN),
            (rng.normal(size=(2, 3)).astype(np.float32), 5, _lib.PRECISION_PLAIN),
            (rng.normal(size=(3, 3)).astype(np.float32), 2, _lib.PRECISION_BF16_REFINED),
            (rng.normal(size=(30, 2)).astype(np.float32), 50, _lib.PRECISION_PLAIN),
            (synthetic.blobs_with_noise(n=1200, d=40, centers=7, seed=8), 5,
             _lib.PRECISION_FP16_REFINED)]
    packed = gpu_ctx.fit_core_packed(fits)
    for (x, ms, prec), got in zip(fits, packed):
        alone = gpu_ctx.fit_core(x, ms, prec)
        for key in ("knn_ids", "src", "dst"):
            np.testing.assert_array_equal(got[key], alone[key])
        for key in ("knn_sq", "core_sq", "wsq"):
            np.testing.assert_array_equal(bits(got[key]), bits(alone[key]))
        assert got["stats"]["mst_weight"] == alone["stats"]["mst_weight"]
        assert_fit_equal(got, O.fit_core(x, ms))


def test_pack_limits(gpu_ctx):
    x = np.zeros((2048, 4), np.float32)
    with pytest.raises(ValueError):
        gpu_ctx.fit_core_packed([(x, 5, _lib.PRECISION_PLAIN)])
    small = np.random.default_rng(0).normal(size=(50, 4)).astype(np.float32)
    with pytest.raises(ValueError):
        gpu_ctx.fit_core_packed([(small, 5, _lib.PRECISION_PLAIN)] * (_lib.PACK_MAX_FITS + 1))
    with pytest.raises(ValueError):
        gpu_ctx.fit_core_packed([(small, 0, _lib.PRECISION_PLAIN)])
    # the context stays usable after a rejected pack
    got = gpu_ctx.fit_core_packed([(small, 5, _lib.PRECISION_PLAIN)])[0]
    assert_fit_equal(got, O.fit_core(small, 5))
