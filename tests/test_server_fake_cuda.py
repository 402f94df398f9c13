"""The request server's control logic on the CPU: occastft_gb300/csrc/ocs_server.cpp
compiled unchanged against a host-only CUDA stand-in (tests/fake_cuda/) whose
streams are FIFO worker threads and whose batch launch writes a known function
of each input.  Built with ThreadSanitizer where the compiler has it, so the
start/submit/wait/stop interleavings are checked for data races as well.

Covers what the GPU server tests cannot make happen on purpose: a copy that
cannot be issued, a start that fails part-way (leak check), a stop racing six
submitting and waiting threads, plus admission through a small pool,
coalescing and cancellation."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
FAKE = os.path.join(ROOT, "tests", "fake_cuda")
CSRC = os.path.join(ROOT, "occastft_gb300", "csrc")
SOURCES = [os.path.join(CSRC, "ocs_server.cpp"), os.path.join(CSRC, "ocs_host.cpp"),
           os.path.join(FAKE, "fake_runtime.cpp"), os.path.join(FAKE, "fake_server_internal.cpp"),
           os.path.join(FAKE, "server_stress.cpp")]


def _build(out, sanitize):
    cxx = os.environ.get("CXX", "g++")
    cmd = [cxx, "-std=c++17", "-O1", "-g", "-pthread", "-I" + FAKE, "-I" + CSRC] + sanitize + SOURCES + ["-o", out]
    return subprocess.run(cmd, capture_output=True, text=True, timeout=300)


@pytest.fixture(scope="module")
def stress_bin(tmp_path_factory):
    if not shutil.which(os.environ.get("CXX", "g++")):
        pytest.skip("no C++ compiler")
    d = tmp_path_factory.mktemp("server_stress")
    out = str(d / "server_stress")
    r = _build(out, ["-fsanitize=thread"])
    tsan = r.returncode == 0
    if not tsan:
        r = _build(out, [])
    assert r.returncode == 0, r.stderr[-4000:]
    return out, tsan


@pytest.mark.parametrize("check", ["admission", "copy_error", "cancel", "stop_race", "start_fail"])
def test_server_control_logic(stress_bin, check):
    exe, tsan = stress_bin
    env = dict(os.environ, TSAN_OPTIONS="halt_on_error=1 exitcode=66")
    r = subprocess.run([exe, check], capture_output=True, text=True, timeout=300, env=env)
    assert r.returncode == 0, (r.stdout + r.stderr)[-4000:]
    assert f"ok {check}" in r.stdout
    if tsan:
        assert "ThreadSanitizer" not in r.stderr, r.stderr[-4000:]


@pytest.fixture(scope="module")
def served_bin(tmp_path_factory):
    """The server on the C ABI's real batch path (ocs_api.cpp) and the
    stand-in kernels (tests/fake_cuda/server_api_stress.cpp)."""
    if not shutil.which(os.environ.get("CXX", "g++")):
        pytest.skip("no C++ compiler")
    srcs = [os.path.join(CSRC, "ocs_server.cpp"), os.path.join(CSRC, "ocs_api.cpp"), os.path.join(CSRC, "ocs_host.cpp"),
            os.path.join(FAKE, "fake_runtime.cpp"), os.path.join(FAKE, "fake_kernels.cpp"),
            os.path.join(FAKE, "server_api_stress.cpp")]
    out = str(tmp_path_factory.mktemp("served") / "server_api_stress")
    cxx = os.environ.get("CXX", "g++")
    base = [cxx, "-std=c++17", "-O1", "-g", "-pthread", "-I" + FAKE, "-I" + CSRC]
    r = subprocess.run(base + ["-fsanitize=thread"] + srcs + ["-o", out], capture_output=True, text=True, timeout=300)
    tsan = r.returncode == 0
    if not tsan:
        r = subprocess.run(base + srcs + ["-o", out], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr[-4000:]
    return out, tsan


def test_server_on_the_batch_path(served_bin):
    """Six threads x 40 mixed requests through a 4 MiB pool and three slots,
    each slot reusing its descriptor staging, with random stream delays:
    every result as the stand-in kernels define it, statistics consistent,
    everything released at stop and shutdown."""
    exe, tsan = served_bin
    env = dict(os.environ, TSAN_OPTIONS="halt_on_error=1 exitcode=66")
    env.pop("OCS_TUNE_CACHE", None)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=600, env=env)
    assert r.returncode == 0 and "all ok" in r.stdout, (r.stdout + r.stderr)[-4000:]
    if tsan:
        assert "ThreadSanitizer" not in r.stderr, r.stderr[-4000:]
