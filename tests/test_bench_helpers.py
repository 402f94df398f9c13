"""bench.py's host-side arithmetic, on CPU: the algorithmic bytes behind the
roofline fraction and the FP32-pipe bound reported beside it."""
import math

import numpy as np

import pytest

import bench


class _Geo:
    def __init__(self, n_window, hop, frames, out_floats):
        self.n_window, self.hop, self.frames, self.out_floats = n_window, hop, frames, out_floats


def test_algorithmic_bytes_counts_covered_samples_and_output(ocs_lib):
    g = ocs_lib.geometry(100_000_000, 10, 0.5, "--hamming_window")
    # every sample is read once (the last frame runs past the end), every output float written once
    assert bench.algorithmic_bytes(100_000_000, g, False, False) == 4 * 100_000_000 + 4 * g.out_floats
    # a compat half-complex request computes only the frames its output needs
    short = _Geo(1024, 512, 10, 10 * 1024)
    assert bench.algorithmic_bytes(1_000_000, short, True, False) == 4 * (9 * 512 + 1024) + 4 * 10 * 1024


def test_fp32_pipe_bound():
    # 5 (N/2) log2(N/2) flops per frame against lanes x 2 x clock per SM
    r = bench.fp32_pipe_bound(1024, 1000, 1e-3, 152, 2000.0)
    flops = 5 * 512 * 9 * 1000
    peak = 152 * bench.FP32_LANES_PER_SM * 2 * 2000e6
    assert r["gflop_s"] == round(flops / 1e-3 / 1e9, 1)
    assert r["peak_gflop_s"] == round(peak / 1e9, 1)
    assert r["frac"] == pytest.approx(flops / 1e-3 / peak, abs=1e-4)
    # doubling the window at a fixed frame count adds one radix-2 level
    a = bench.fp32_pipe_bound(1024, 10**6, 1e-3, 152, 2000.0)
    b = bench.fp32_pipe_bound(2048, 10**6, 1e-3, 152, 2000.0)
    assert b["gflop_s"] / a["gflop_s"] == pytest.approx(2 * 10 / 9, rel=1e-6)
    assert math.isclose(bench.NOMINAL_SM_MAX_MHZ, 2070.0)


@pytest.mark.parametrize("have_reference_build", [True, False])
def test_serial_one_core_baseline(monkeypatch, have_reference_build):
    """cpu_baseline's single-core Serial figure: the reference's own Serial code
    where it was built from source, else the bit-exact port on one thread
    (on machines without the reference checkout)."""
    from oracle import orc

    if not have_reference_build:
        monkeypatch.setattr(orc.RefLib, "available", staticmethod(lambda name="libref_serial.so": False))
    elif not orc.RefLib.available("libref_serial.so"):
        pytest.skip("oracle/_ref not built")
    r = bench.cpu_serial_baseline(sample_n=1 << 16, budget_s=0.2)
    assert r["cores"] == 1 and r["unit"] == bench.METRIC and r["value"] > 0
    assert r["kind"] == ("reference" if have_reference_build else "port")
    assert "one thread" in r["sample"]


def test_reference_arm_prints_its_line():
    """`bench.py --impl reference` (the reference's CPU implementation of the
    path, timed on the host cores) prints one JSON line with the keys of the
    bench contract; warm-up is never below three steps."""
    import json
    import os
    import subprocess
    import sys

    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    r = subprocess.run([sys.executable, os.path.join(root, "bench.py"), "--impl", "reference", "--steps", "1",
                        "--warmup", "0"], capture_output=True, text=True, timeout=600, cwd=root)
    assert r.returncode == 0, r.stderr[-3000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, r.stdout
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["metric"] == bench.METRIC and d["unit"] == bench.METRIC
    assert d["value"] > 0 and d["higher_is_better"] is True and d["n_gpus"] == 1
    assert d["steps"] == 1 and d["warmup"] >= 3
    cb = d["cpu_baseline"]
    assert cb["value"] == d["value"] and cb["kind"] in ("reference", "port") and cb["cores"] >= 1 and cb["sample"]
    assert d["e2e"] == {"value": d["value"], "unit": d["unit"], "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
    assert d["config"]["window"] == 1024 and d["config"]["overlap"] == 0.5


def test_reference_arm_other_ranks_exit_quietly():
    """Under torchrun with N > 1 only rank 0 runs the reference arm; the
    other ranks exit 0 without work or output."""
    import os
    import subprocess
    import sys

    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    env = dict(os.environ, WORLD_SIZE="2", RANK="1", LOCAL_RANK="1")
    r = subprocess.run([sys.executable, os.path.join(root, "bench.py"), "--impl", "reference", "--steps", "1"],
                       capture_output=True, text=True, timeout=300, cwd=root, env=env)
    assert r.returncode == 0 and "{" not in r.stdout, r.stdout + r.stderr[-2000:]


@pytest.mark.parametrize("opts", ["--hanning_window", "--hamming_window", "--blackman_window"])
def test_accuracy_window_is_independent_and_agrees(orc, opts):
    """The bench's accuracy check evaluates its window in float64 from the
    formula, not from the library's table; the two agree to float rounding."""
    N = 1024
    kind = opts[2:].split("_")[0]
    ref = orc.window(kind, N).astype(np.float64)
    w = bench.window_fp64(opts, N)
    assert np.max(np.abs(w - ref)) <= 2e-7


def test_cpu_baseline_uses_the_reference_arms_sample():
    """cpu_baseline and the reference arm time the same slice of the signal."""
    import inspect

    assert inspect.signature(bench.cpu_baseline).parameters["sample_n"].default == bench.CPU_SAMPLE
    r = bench.cpu_baseline(sample_n=1 << 16, budget_s=0.2)
    assert r["value"] > 0 and r["kind"] in ("reference", "port") and r["cores"] >= 1
    assert r["serial_1core"]["cores"] == 1


def test_cpu_leg_subprocess_prints_its_line(monkeypatch):
    """The CPU baseline runs as `bench.py --cpu-leg` in a fresh process; the
    options string (which starts with "--") reaches it intact."""
    monkeypatch.setattr(bench, "CPU_SAMPLE", 1 << 16)
    import subprocess
    import sys

    real = subprocess.run

    def small(cmd, **kw):
        # the child times a small sample so that the test stays short
        return real(cmd + ["--cpu-sample", str(1 << 16)], **kw) if "--cpu-leg" in cmd else real(cmd, **kw)

    monkeypatch.setattr(subprocess, "run", small)
    r = bench.cpu_baseline_subprocess()
    assert "unavailable" not in r, r
    assert r["value"] > 0 and r["kind"] in ("reference", "port") and r["serial_1core"]["cores"] == 1
