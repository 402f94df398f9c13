"""Mutation fuzzing of the runner's two parsers of network input, on the CPU,
under AddressSanitizer and UndefinedBehaviorSanitizer:
- the RequestCapnp decoder (tests/fuzz/codec_fuzz.cpp): seeds are valid
  requests written by the Python codec in single-segment, far-pointer and
  double-far-pointer layouts, with and without a data list; each is mutated
  20,000 times (bit flips, words set to extreme pointer values, truncation,
  extension, segment-table entries).  It must never read outside the message.
- the WebSocket server (tests/fuzz/ws_fuzz.cpp): 2,000 connections, each a
  handshake and then a mutated stream of valid client frames (text,
  fragmented binary with a ping inside, close).  The handler reads every
  message byte, and a clean client is served afterwards."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from occastft_gb300 import wire

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SA = os.path.join(ROOT, "occastft_gb300", "standalone")


def _seeds(d):
    x = np.linspace(-1, 1, 37, dtype=np.float32)
    reqs = [
        wire.Request(windowRadix=10, overlapRatio=0.5, mappedID="42", sharedMemory="/STFT42SHAREDMEM", dataLength=1000,
                     overlapdataLength=2048, options="--hanning_window --remove_dc", posixFileDes=-1),
        wire.Request(windowRadix=8, overlapRatio=0.75, mappedID="7", dataLength=x.size, overlapdataLength=256,
                     options="--blackman_window --half_complex_return", data=x),
    ]
    paths = []
    for i, r in enumerate(reqs):
        for layout in ("single", "far", "double-far"):
            p = os.path.join(d, f"seed{i}_{layout}.bin")
            with open(p, "wb") as f:
                f.write(wire.encode(r, layout))
            paths.append(p)
    return paths


def test_request_decoder_survives_mutations(tmp_path):
    cxx = os.environ.get("CXX", "g++")
    if not shutil.which(cxx):
        pytest.skip("no C++ compiler")
    exe = str(tmp_path / "codec_fuzz")
    r = subprocess.run([cxx, "-std=c++17", "-O1", "-g", "-fsanitize=address,undefined", "-fno-sanitize-recover=all",
                        "-I" + SA, os.path.join(SA, "request_codec.cpp"),
                        os.path.join(ROOT, "tests", "fuzz", "codec_fuzz.cpp"), "-o", exe],
                       capture_output=True, text=True, timeout=300)
    if r.returncode != 0 and "sanitize" in r.stderr:
        pytest.skip("the compiler has no AddressSanitizer")
    assert r.returncode == 0, r.stderr[-4000:]
    env = dict(os.environ, ASAN_OPTIONS="detect_leaks=1:abort_on_error=0", UBSAN_OPTIONS="print_stacktrace=1")
    p = subprocess.run([exe, "20000"] + _seeds(str(tmp_path)), capture_output=True, text=True, timeout=600, env=env)
    assert p.returncode == 0, (p.stdout + p.stderr)[-4000:]
    assert "decoded ok:" in p.stdout and "ERROR" not in p.stderr and "runtime error" not in p.stderr, p.stderr[-4000:]
    ok, total = [int(v) for v in p.stdout.split("decoded ok:")[1].split("of")]
    assert total == 6 * 20000 and 0 < ok < total  # some mutants still decode, most are refused


def test_websocket_server_survives_mutated_streams(tmp_path):
    cxx = os.environ.get("CXX", "g++")
    if not shutil.which(cxx):
        pytest.skip("no C++ compiler")
    exe = str(tmp_path / "ws_fuzz")
    r = subprocess.run([cxx, "-std=c++17", "-O1", "-g", "-pthread", "-fsanitize=address,undefined",
                        "-fno-sanitize-recover=all", "-I" + SA, os.path.join(SA, "ws_server.cpp"),
                        os.path.join(ROOT, "tests", "fuzz", "ws_fuzz.cpp"), "-o", exe],
                       capture_output=True, text=True, timeout=300)
    if r.returncode != 0 and "sanitize" in r.stderr:
        pytest.skip("the compiler has no AddressSanitizer")
    assert r.returncode == 0, r.stderr[-4000:]
    env = dict(os.environ, ASAN_OPTIONS="detect_leaks=1", UBSAN_OPTIONS="print_stacktrace=1")
    p = subprocess.run([exe, "2000"], capture_output=True, text=True, timeout=600, env=env)
    assert p.returncode == 0, (p.stdout + p.stderr)[-4000:]
    assert "clean client served: yes" in p.stdout and "ERROR" not in p.stderr and "runtime error" not in p.stderr
