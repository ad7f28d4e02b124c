"""The C-ABI library builds, loads without a GPU and exports every declared symbol; the
estimator surface validates like the reference's (no device calls)."""
from __future__ import annotations

import re
import subprocess
from pathlib import Path

import numpy as np
import pytest

import cuscan_gb300 as cg
from cuscan_gb300 import _lib

HEADER = Path(__file__).resolve().parent.parent / "include" / "cuscan_gb300.h"


def declared_functions():
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(cuscan_[a-z_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol():
    path = _lib.library_path()
    cg.load()
    out = subprocess.run(["nm", "-D", "--defined-only", str(path)], capture_output=True,
                         text=True, check=True).stdout
    exported = set(re.findall(r"\b(cuscan_[a-z_]+)\b", out))
    declared = declared_functions()
    assert declared, "header declares no functions"
    missing = [f for f in declared if f not in exported]
    assert not missing, f"declared but not exported: {missing}"
    assert set(declared) == set(_lib.SIGNATURES), "ctypes signatures out of sync with the header"


def test_library_is_built_for_sm_103a_only():
    # every translation unit is compiled with this one target (cuscan_gb300/build.py)
    from cuscan_gb300 import build
    assert build.ARCH == ["-gencode", "arch=compute_103a,code=sm_103a"]


def test_version_string():
    assert b"sm_103a" in cg.load().cuscan_version()


def test_error_mapping_matches_reference():
    # crates/cuscan-python/src/hdbscan.rs:956-968
    for code, exc in [(1, ValueError), (2, ValueError), (3, RuntimeError), (4, RuntimeError),
                      (5, OverflowError), (6, OverflowError), (7, MemoryError)]:
        with pytest.raises(exc):
            _lib.raise_for(code, "x")
    _lib.raise_for(0, "ok")


@pytest.mark.parametrize("kwargs,exc", [
    (dict(min_cluster_size=0), ValueError),
    (dict(min_samples=0), ValueError),
    (dict(min_cluster_size=True), ValueError),
    (dict(cluster_selection_epsilon=-1.0), ValueError),
    (dict(cluster_selection_epsilon=1), ValueError),
    (dict(cluster_selection_method="x"), ValueError),
    (dict(allow_single_cluster=1), ValueError),
    (dict(max_cluster_size=0), ValueError),
    (dict(backend="tpu"), ValueError),
    (dict(metric="manhattan"), NotImplementedError),
    (dict(semi_supervised=True), NotImplementedError),
    (dict(backend="cpu"), NotImplementedError),
    (dict(precision="fp16"), ValueError),
])
def test_estimator_validation(kwargs, exc):
    with pytest.raises(exc):
        cg.HDBSCAN(**kwargs).fit(np.zeros((4, 2), np.float32))


def test_input_validation():
    with pytest.raises(ValueError):
        cg.HDBSCAN().fit(np.zeros(4))
    with pytest.raises(ValueError):
        cg.HDBSCAN().fit(np.full((3, 2), np.nan))
    with pytest.raises(ValueError):
        cg.HDBSCAN().fit(np.array([[1e300, 0.0]]))
    with pytest.raises(ValueError):
        cg.HDBSCAN().labels_


def test_no_gpu_context_raises_without_fallback():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(RuntimeError):
        cg.Context(0)
    with pytest.raises(RuntimeError):
        cg.HDBSCAN().fit(np.random.default_rng(0).normal(size=(20, 3)))
