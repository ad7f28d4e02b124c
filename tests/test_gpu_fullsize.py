"""Oracle parity at the full size of the 100,000-point workloads.

Two configurations state a CPU-checked result at their own size:

* the anisotropic mixture, n = 100,000, d = 64, min_samples 10, min_cluster_size 50 (labels
  against the reference CPU semantics, MST weight against the FP64 total);
* the vMF-like unit vectors, d = 128, min_samples 15, min_cluster_size 100, here at
  n = 100,000 (the 500,000-point fit is compared with the plain f32 form bit for bit by the
  benchmark instead; its oracle run would take several minutes).

For each, the oracle's fit core (production semantics: kNN seed, then Borůvka rounds in merge
order; crates/hdbscan/src/estimator.rs:524-874) runs once on the host and every precision's
device fit must equal it bit for bit: kNN ids and squared distances, core distances, the MST
edges in merge order, the f64 total weight in the device's summation order, and the labels of
the unchanged extraction. The oracle uses its blocked loops (bit-identical to the row-at-a-time
loops, checked on the CPU in test_oracle_consistency.py).
"""
from __future__ import annotations

import numpy as np
import pytest

import cuscan_gb300 as cg
from cuscan_gb300 import _lib, synthetic
from oracle import oracle as O
from tests.test_gpu_fit import PRECISIONS, assert_fit_equal

pytestmark = pytest.mark.gpu


def _oracle_labels(fc, mcs):
    mst = O.finalize_mst(fc.src, fc.dst, fc.wsq)
    host = cg.clusters_from_spanning_tree(mst[:, 0].astype(np.uint32),
                                          mst[:, 1].astype(np.uint32), mst[:, 2],
                                          min_cluster_size=mcs)
    return mst, host["labels"]


@pytest.fixture(scope="module")
def aniso_full():
    x, ms, mcs = synthetic.workload("aniso_100k_d64")
    assert x.shape == (100_000, 64)
    fc = O.fit_core(x, ms)
    mst, labels = _oracle_labels(fc, mcs)
    return x, ms, mcs, fc, mst, labels


@pytest.fixture(scope="module")
def vmf_100k():
    x, ms, mcs = synthetic.workload("vmf_500k_d128", n=100_000)
    assert x.shape == (100_000, 128)
    fc = O.fit_core(x, ms)
    mst, labels = _oracle_labels(fc, mcs)
    return x, ms, mcs, fc, mst, labels


def _check(gpu_ctx, case, precision):
    x, ms, mcs, fc, mst, labels = case
    got = gpu_ctx.fit_core(x, ms, precision)
    assert_fit_equal(got, fc)
    model = cg.HDBSCAN(min_cluster_size=mcs, min_samples=ms,
                       precision={v: k for k, v in _lib.PRECISIONS.items()}[precision]).fit(x)
    np.testing.assert_array_equal(model.minimum_spanning_tree_, mst)
    np.testing.assert_array_equal(model.labels_, labels)
    return got


@pytest.mark.parametrize("precision", PRECISIONS)
def test_aniso_100k_d64_full_size_equals_oracle(gpu_ctx, aniso_full, precision):
    got = _check(gpu_ctx, aniso_full, precision)
    assert len(set(aniso_full[5].tolist()) - {-1}) >= 2
    if precision != _lib.PRECISION_PLAIN:
        assert got["stats"]["refined_rows"] == aniso_full[0].shape[0]


@pytest.mark.parametrize("precision", PRECISIONS)
def test_vmf_100k_d128_equals_oracle(gpu_ctx, vmf_100k, precision):
    got = _check(gpu_ctx, vmf_100k, precision)
    if precision != _lib.PRECISION_PLAIN:
        assert got["stats"]["screen_tile_pairs"] > 0
