"""Shared fixtures.  `gpu` tests need a CUDA device and the native runner;
everything else runs on CPU (the oracle, host logic, library exports)."""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the native runner")


def _has_gpu() -> bool:
    try:
        import torch

        return torch.cuda.is_available()
    except Exception:  # noqa: BLE001
        return False


HAS_GPU = _has_gpu()


def pytest_collection_modifyitems(config, items):
    if HAS_GPU:
        return
    skip = pytest.mark.skip(reason="no CUDA device")
    for it in items:
        if "gpu" in it.keywords:
            it.add_marker(skip)


@pytest.fixture(scope="session")
def orc():
    from oracle import orc as o

    o.lib()
    return o


@pytest.fixture(scope="session")
def ocs_lib():
    import occastft_gb300 as ocs

    if not os.path.exists(ocs.LIB_PATH):
        from occastft_gb300 import build

        build.build()
    return ocs


@pytest.fixture(scope="session")
def golden():
    import json

    here = os.path.join(ROOT, "tests", "golden")
    with open(os.path.join(here, "manifest.json")) as f:
        manifest = json.load(f)
    arrays = np.load(os.path.join(here, "reference_outputs.npz"))
    return manifest, arrays


def signal(seed: int, n: int) -> np.ndarray:
    return np.random.default_rng(seed).uniform(-1.0, 1.0, n).astype(np.float32)
