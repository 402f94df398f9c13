"""The C ABI's host logic on the CPU: occastft_gb300/csrc/ocs_api.cpp compiled
unchanged against a host-only CUDA stand-in (tests/fake_cuda/) whose streams
are FIFO worker threads ordered by events as CUDA's are, and whose stand-in
kernels read each frame's samples and write the floats the layout gives that
frame.  Built with ThreadSanitizer where the compiler has it.

Covers what the GPU tests cannot make happen on purpose or often enough:
- a set-up, a window table upload, a request slot or a kernel-variant timing
  whose allocation, copy, streams or events fail (nothing may leak);
- the chunked copy/compute pipeline of ocs_activate under random delays on
  every stream and slow input copies, with the result written over the
  signal in three placements;
- four threads calling ocs_activate at once;
- ocs_plan_tune ahead of a request (its scratch released, the choice kept);
- uneven batches, the tile-length tuning of a new mix (timed once, then kept;
  none with a fixed length), the per-capture descriptor buffers, and a full
  release at ocs_shutdown."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
FAKE = os.path.join(ROOT, "tests", "fake_cuda")
CSRC = os.path.join(ROOT, "occastft_gb300", "csrc")
SOURCES = [os.path.join(CSRC, "ocs_api.cpp"), os.path.join(CSRC, "ocs_host.cpp"),
           os.path.join(FAKE, "fake_runtime.cpp"), os.path.join(FAKE, "fake_kernels.cpp"),
           os.path.join(FAKE, "api_stress.cpp")]
CHECKS = ["setup_fail", "table_fail", "slot_fail", "tune_fail", "capture_tune", "plan_tune", "activate",
          "concurrent", "batch", "batch_tune", "capture", "shutdown"]


def _build(out, sanitize):
    cxx = os.environ.get("CXX", "g++")
    cmd = [cxx, "-std=c++17", "-O1", "-g", "-pthread", "-I" + FAKE, "-I" + CSRC] + sanitize + SOURCES + ["-o", out]
    return subprocess.run(cmd, capture_output=True, text=True, timeout=300)


@pytest.fixture(scope="module")
def api_bin(tmp_path_factory):
    if not shutil.which(os.environ.get("CXX", "g++")):
        pytest.skip("no C++ compiler")
    out = str(tmp_path_factory.mktemp("api_stress") / "api_stress")
    r = _build(out, ["-fsanitize=thread"])
    tsan = r.returncode == 0
    if not tsan:
        r = _build(out, [])
    assert r.returncode == 0, r.stderr[-4000:]
    return out, tsan


def _env():
    env = dict(os.environ, TSAN_OPTIONS="halt_on_error=1 exitcode=66")
    env.pop("OCS_TUNE_CACHE", None)
    return env


@pytest.fixture(scope="module")
def run(api_bin):
    exe, tsan = api_bin
    p = subprocess.run([exe], capture_output=True, text=True, timeout=900, env=_env())
    return p, tsan


@pytest.mark.parametrize("check", CHECKS)
def test_c_abi_host_logic(run, check):
    p, tsan = run
    assert f"ok {check}" in p.stdout, (p.stdout + p.stderr)[-4000:]
    if tsan:
        assert "ThreadSanitizer" not in p.stderr, p.stderr[-4000:]


def test_c_abi_host_logic_exit(run):
    p, _ = run
    assert p.returncode == 0 and "all ok" in p.stdout, (p.stdout + p.stderr)[-4000:]


def test_tuning_cache_round_trip(api_bin, tmp_path):
    """OCS_TUNE_CACHE: one process tunes a request and appends its choice
    ("gpu|exp|outk|dense|bucket|variant"); a second process, in which no
    event can be created, runs the same request on the cached choice alone.
    Lines for other GPUs and malformed lines are skipped."""
    exe, _ = api_bin
    cache = tmp_path / "tune.txt"
    cache.write_text("not a cache line\nanother gpu|10|0|0|9|1\n")
    w = subprocess.run([exe, "tune-cache-write", str(cache)], capture_output=True, text=True, timeout=300, env=_env())
    assert w.returncode == 0 and "ok tune-cache-write" in w.stdout, w.stdout + w.stderr
    lines = cache.read_text().splitlines()
    assert lines[:2] == ["not a cache line", "another gpu|10|0|0|9|1"]
    mine = [ln.split("|") for ln in lines[2:]]
    assert mine and all(len(f) == 6 and f[0] == "host stand-in" for f in mine), lines
    r = subprocess.run([exe, "tune-cache-read", str(cache)], capture_output=True, text=True, timeout=300, env=_env())
    assert r.returncode == 0 and "ok tune-cache-read" in r.stdout, r.stdout + r.stderr
    # without the cached line the same run has to time the variants, and cannot
    cache.write_text("not a cache line\n")
    r = subprocess.run([exe, "tune-cache-read", str(cache)], capture_output=True, text=True, timeout=300, env=_env())
    assert r.returncode != 0 and "kernel variant timing" in r.stdout
