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


def sweep_signal(n: int, seed: int = 1, fs: float = 48000.0) -> np.ndarray:
    """The window sweep's signal: 8 sinusoids (frequencies uniform in
    [20 Hz, 20 kHz] at fs, amplitudes in [0.05, 0.5], random phases) plus
    Gaussian noise of sigma 0.01, evaluated in float64 and stored as float32."""
    rng = np.random.default_rng(seed)
    f = rng.uniform(20.0, 20000.0, 8)
    a = rng.uniform(0.05, 0.5, 8)
    ph = rng.uniform(0.0, 2 * np.pi, 8)
    noise = np.random.default_rng(seed + 1000)
    out = np.empty(n, dtype=np.float32)
    chunk = 1 << 22
    for s in range(0, n, chunk):
        e = min(n, s + chunk)
        t = np.arange(s, e, dtype=np.float64) / fs
        acc = 0.01 * noise.standard_normal(e - s)
        for k in range(8):
            acc += a[k] * np.sin(2 * np.pi * f[k] * t + ph[k])
        out[s:e] = acc.astype(np.float32)
    return out


def to_quot_f32(n: int, window: int, overlap: float) -> int:
    """toQuot (GLOBAL/RunnerInterface.hpp:26-35) in float32 arithmetic, each
    operation rounded to float32, truncated to an integer."""
    f32 = np.float32
    full, win, ov = f32(n), f32(window), f32(overlap)
    if ov == f32(0):
        q = full / win + f32(1)
    else:
        q = full / (win * (f32(1) - ov)) + f32(1)
    return int(q)
