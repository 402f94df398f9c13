"""Helpers for the runner-executable tests: start `occastft_gb300/cudaRun`
on a free port and wait until it accepts connections."""
import os
import socket
import subprocess
import time

from tests.conftest import ROOT

CUDARUN = os.path.join(ROOT, "occastft_gb300", "cudaRun")


def free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def ensure_built():
    if not os.path.exists(CUDARUN):
        from occastft_gb300 import build

        build.build()


def start_cudarun(port: int = 0, env=None) -> tuple:
    ensure_built()
    port = port or free_port()
    e = dict(os.environ)
    if env:
        e.update(env)
    p = subprocess.Popen([CUDARUN, str(port)], env=e, stdout=subprocess.PIPE, stderr=subprocess.PIPE)
    deadline = time.time() + 60
    while time.time() < deadline:
        if p.poll() is not None:
            raise RuntimeError("cudaRun exited: " + p.stderr.read().decode(errors="replace"))
        try:
            with socket.create_connection(("127.0.0.1", port), timeout=0.2):
                return p, port
        except OSError:
            time.sleep(0.05)
    p.kill()
    raise RuntimeError("cudaRun did not start listening")


def stop(p):
    if p.poll() is None:
        p.kill()
    p.wait(timeout=10)
