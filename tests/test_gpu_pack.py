"""Packed small fits (cuscan_fit_core_packed): several fit cores in one CUDA graph launch, the
Borůvka rounds of each as a device-controlled while loop.

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


def test_packs_of_one_size_update_one_instantiated_graph():
    """Packs of the same size share one graph topology: the first is instantiated, the later
    ones (other row counts, dimensions and point sets) update it in place, and every result
    still equals the oracle. Row counts stay above 256, where the exact kNN always splits the
    reference range (at most 256 rows take the unsplit launch, another topology, and such a pack
    is instantiated anew)."""
    ctx = _lib.Context(0)
    rng = np.random.default_rng(9)
    rounds = 4
    for r in range(rounds):
        fits = [(synthetic.blobs_with_noise(n=int(rng.integers(300, 2048)),
                                            d=int(rng.choice([8, 32, 64])),
                                            centers=int(rng.integers(2, 20)),
                                            seed=int(rng.integers(1 << 30))), 5,
                 _lib.PRECISION_FP16_REFINED) for _ in range(3)]
        packed = ctx.fit_core_packed(fits)
        for (x, ms, _), got in zip(fits, packed):
            assert_fit_equal(got, O.fit_core(x, ms))
    st = ctx.packed_graph_stats()
    assert st == {"instantiations": 1, "updates": rounds - 1}, st


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
