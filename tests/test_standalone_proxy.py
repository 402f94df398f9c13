"""The proxy's runtime fallback (StandAlone/src/STFTProxy.cpp:83-154), on CPU:
unavailable runtimes are skipped, a local runner is launched as
`<exe> <port>` and fed through POSIX shared memory, and a runner that dies
is replaced by the next runtime of the list.  The runners here are the
oracle's serial runner (tests/oracle_runner.py) behind `serialRun` shims."""
import os
import stat
import sys

import numpy as np

from occastft_gb300 import proxy
from tests.conftest import ROOT, signal


def make_serial_runner(d):
    exe = os.path.join(d, "serialRun")
    with open(exe, "w") as f:
        f.write(f"#!/bin/sh\nexec {sys.executable} {os.path.join(ROOT, 'tests', 'oracle_runner.py')} \"$@\"\n")
    os.chmod(exe, os.stat(exe).st_mode | stat.S_IEXEC)
    return d


def test_skips_unavailable_runtimes(tmp_path, orc):
    d = make_serial_runner(str(tmp_path))
    errs = []
    p = proxy.STFTProxy([("CUDA", "/nonexistent/dir"), ("HIP", "/nonexistent"), ("SERIAL", d)], errs.append)
    try:
        assert p.gpu_type == "SERIAL" and p.status == "OK"
        x = signal(3, 20000)
        got = p.request_stft(x, 10, 0.5, "--hanning_window --remove_dc")
        ref = orc.serial_pipeline(x, 10, 0.5, "--hanning_window --remove_dc")
        assert got.shape == ref.shape and np.array_equal(got, ref)
    finally:
        assert p.kill_runner()


def test_runner_failure_falls_back(tmp_path, orc):
    (tmp_path / "a").mkdir()
    (tmp_path / "b").mkdir()
    d1 = make_serial_runner(str(tmp_path / "a"))
    d2 = make_serial_runner(str(tmp_path / "b"))
    errs = []
    p = proxy.STFTProxy([("SERIAL", d1), ("SERIAL", d2)], errs.append)
    try:
        x = signal(4, 30000)
        first = p.runner
        assert p.request_stft(x, 9, 0.75, "--blackman_window") is not None
        first.kill()  # injected failure: the runner dies between requests
        first.wait()
        got = p.request_stft(x, 9, 0.75, "--blackman_window")
        assert p.runner is not first and errs
        assert np.array_equal(got, orc.serial_pipeline(x, 9, 0.75, "--blackman_window"))
    finally:
        p.kill_runner()


def test_run_out_of_fallbacks(tmp_path):
    p = proxy.STFTProxy([("SERIAL", str(tmp_path))])  # no executable there
    assert p.status == "Run Out Fallback"
    assert p.request_stft(signal(1, 1000), 8) is None


def test_shared_memory_is_unlinked(tmp_path):
    d = make_serial_runner(str(tmp_path))
    p = proxy.STFTProxy([("SERIAL", d)])
    try:
        before = set(os.listdir("/dev/shm"))
        p.request_stft(signal(5, 5000), 8, 0.5, "--hamming_window")
        assert set(os.listdir("/dev/shm")) - before == set()
    finally:
        p.kill_runner()


def test_unreachable_runner_is_not_left_running(tmp_path, orc):
    """A runner executable that starts but never accepts connections is given
    up after the connection attempts, and the proxy ends that process before
    moving on to the next runtime of the list."""
    (tmp_path / "dead").mkdir()
    (tmp_path / "ok").mkdir()
    pidfile = tmp_path / "pid"
    exe = tmp_path / "dead" / "serialRun"
    exe.write_text(f"#!/bin/sh\necho $$ > {pidfile}\nexec sleep 600\n")
    exe.chmod(exe.stat().st_mode | stat.S_IEXEC)
    d2 = make_serial_runner(str(tmp_path / "ok"))
    p = proxy.STFTProxy([("SERIAL", str(tmp_path / "dead")), ("SERIAL", d2)])
    try:
        assert p.status == "OK" and p.gpu_type == "SERIAL"
        pid = int(pidfile.read_text())
        assert not os.path.exists(f"/proc/{pid}") or open(f"/proc/{pid}/stat").read().split()[2] == "Z"
        x = signal(6, 8000)
        assert np.array_equal(p.request_stft(x, 8, 0.5, "--hamming_window"),
                              orc.serial_pipeline(x, 8, 0.5, "--hamming_window"))
    finally:
        p.kill_runner()
