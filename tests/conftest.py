"""pytest configuration: the `gpu` marker and shared fixtures.

Tests marked `gpu` need a CUDA device of the Blackwell generation and call the CUDA path
through the library's C ABI; every other test runs on the CPU only.
"""
from __future__ import annotations

import json
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
GOLDEN = ROOT / "tests" / "golden"
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a kernels)")


@pytest.fixture(scope="session")
def manifest():
    return json.loads((GOLDEN / "manifest.json").read_text())


def load_case(case_id: str):
    return dict(np.load(GOLDEN / f"{case_id}.npz"))


@pytest.fixture(scope="session")
def gpu_ctx():
    import cuscan_gb300 as cg
    return cg.context(0)
