"""The runner executable's success paths on the CPU.  cudaRun is built from its
own sources (occastft_gb300/standalone/) and the C ABI (ocs_api.cpp), against
the host-only CUDA stand-in and stand-in kernels of tests/fake_cuda/, with
ThreadSanitizer where the compiler has it.  It then serves real requests over
the reference's protocol:
- data-list requests in single-segment, far-pointer and fragmented messages;
- shared-memory requests whose result is written over the signal in place;
- four clients at once;
- the proxy launching it and fetching results.
Results must equal what the stand-in kernels define: frame f reads samples
[f*hop, f*hop + N) with zeros past the end, and output float k of its row
takes sample k mod N.  The GPU tests check the same paths against the FP64
oracle."""
import os
import shutil
import subprocess
import threading

import numpy as np
import pytest

from occastft_gb300 import proxy, wire
from tests import cudarun_util as cu
from tests.conftest import ROOT, signal

FAKE = os.path.join(ROOT, "tests", "fake_cuda")
CSRC = os.path.join(ROOT, "occastft_gb300", "csrc")
SA = os.path.join(ROOT, "occastft_gb300", "standalone")
SOURCES = [os.path.join(SA, f) for f in ("cudaRun.cpp", "request_codec.cpp", "ws_server.cpp", "shm_payload.cpp")] + \
          [os.path.join(CSRC, "ocs_api.cpp"), os.path.join(CSRC, "ocs_host.cpp"),
           os.path.join(FAKE, "fake_runtime.cpp"), os.path.join(FAKE, "fake_kernels.cpp")]
CASES = [
    (10, 0.5, "--hamming_window"),
    (8, 0.75, "--hanning_window --remove_dc --half_complex_return"),
    (12, 0.5, "--blackman_window --layout=dense"),
    (6, 0.25, "--flattop_window --serial_power"),
    (9, 0.3, "--hanning_window --half_complex_return --layout=dense"),
    (16, 0.5, "--hanning_window"),
]


def stand_in_out(ocs_lib, x, exp, ov, opts):
    """What the stand-in kernels produce for the whole request."""
    g = ocs_lib.geometry(x.size, exp, ov, opts)
    N = 1 << exp
    half = "--half_complex_return" in opts
    row = (N // 2 + 1) * (2 if half else 1) if "--layout=dense" in opts else (2 * N if half else N)
    F = np.arange(g.frames, dtype=np.int64)[:, None]
    K = np.arange(row, dtype=np.int64)[None, :]
    idx = (F * row + K).ravel()
    s = (F * g.hop + K % N).ravel()
    keep = idx < g.out_floats
    vals = np.where(s < x.size, x[np.minimum(s, x.size - 1)], np.float32(0)).astype(np.float32)
    out = np.full(g.out_floats, np.nan, np.float32)
    out[idx[keep]] = vals[keep]
    return out


@pytest.fixture(scope="module")
def stand_in_runner(tmp_path_factory):
    cxx = os.environ.get("CXX", "g++")
    if not shutil.which(cxx):
        pytest.skip("no C++ compiler")
    d = tmp_path_factory.mktemp("runner")
    exe = str(d / "cudaRun")
    base = [cxx, "-std=c++17", "-O1", "-g", "-pthread", "-I" + FAKE, "-I" + CSRC, "-I" + SA,
            "-I" + os.path.join(ROOT, "include")]
    r = subprocess.run(base + ["-fsanitize=thread"] + SOURCES + ["-o", exe, "-lrt"], capture_output=True, text=True,
                       timeout=300)
    tsan = r.returncode == 0
    if not tsan:
        r = subprocess.run(base + SOURCES + ["-o", exe, "-lrt"], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr[-4000:]
    return exe, tsan


@pytest.fixture(scope="module")
def served(stand_in_runner):
    exe, tsan = stand_in_runner
    port = cu.free_port()
    env = dict(os.environ, TSAN_OPTIONS="halt_on_error=1 exitcode=66", OCS_AUTOTUNE="0")
    p = subprocess.Popen([exe, str(port)], env=env, stdout=subprocess.PIPE, stderr=subprocess.PIPE)
    import socket
    import time

    deadline = time.time() + 60
    while True:
        assert p.poll() is None, p.stderr.read().decode(errors="replace")
        try:
            with socket.create_connection(("127.0.0.1", port), timeout=0.2):
                break
        except OSError:
            assert time.time() < deadline, "the stand-in runner did not start listening"
            time.sleep(0.05)
    yield port
    ws = proxy.WsClient("127.0.0.1", port)
    ws.send_text("CLOSE_REQUEST")
    assert ws.recv(timeout=60) == (1, b"CLOSE_COMPLETE")
    ws.close()
    assert p.wait(timeout=60) == 0
    err = p.stderr.read().decode(errors="replace")
    if tsan:
        assert "ThreadSanitizer" not in err, err[-4000:]


def _ask(port, req, layout="single", fragments=1):
    ws = proxy.WsClient("127.0.0.1", port)
    try:
        ws.send_binary(wire.encode(req, layout), fragments=fragments)
        op, payload = ws.recv(timeout=120)
        assert op == 2
        return wire.decode(payload)
    finally:
        ws.close()


@pytest.mark.parametrize("exp,ov,opts", CASES)
@pytest.mark.parametrize("layout,fragments", [("single", 1), ("far", 1), ("double-far", 5)])
def test_data_list_request(served, ocs_lib, exp, ov, opts, layout, fragments):
    x = signal(exp * 7 + 1, 150_001 if exp < 16 else 400_001)
    req = wire.Request(windowRadix=exp, overlapRatio=ov, mappedID="9", dataLength=x.size,
                       overlapdataLength=proxy.to_overlap_length(x.size, ov, 1 << exp), options=opts, data=x)
    a = _ask(served, req, layout, fragments)
    assert a.sharedMemory == "" and a.mappedID == "9"
    want = stand_in_out(ocs_lib, x, exp, ov, opts)
    assert a.data is not None and a.dataLength == a.data.size == want.size
    assert np.array_equal(a.data, want)


@pytest.mark.parametrize("exp,ov,opts", CASES)
def test_shared_memory_request_in_place(served, ocs_lib, exp, ov, opts):
    """The runner reads the signal from the object and writes the result over
    it: ocs_activate's in-place path, with several copy/compute chunks."""
    x = signal(exp * 11 + 5, 5_000_003 if exp < 16 else 1_000_003)
    olen = proxy.to_overlap_length(x.size, ov, 1 << exp)
    shm = proxy.SharedPayload("fk" + str(exp), olen)
    try:
        shm.floats()[: x.size] = x
        req = wire.Request(windowRadix=exp, overlapRatio=ov, mappedID="fk" + str(exp), sharedMemory=shm.name,
                           dataLength=x.size, overlapdataLength=olen, options=opts, posixFileDes=-1)
        a = _ask(served, req, "double-far")
        want = stand_in_out(ocs_lib, x, exp, ov, opts)
        if want.size > shm.floats().size:
            # the object is sized for the reference layout (toOverlapLength);
            # a larger result is refused, not written past the object
            assert a.sharedMemory == "ERR"
            return
        assert a.sharedMemory == shm.name and a.dataLength == x.size and a.data is None
        assert np.array_equal(shm.floats()[: want.size], want)
    finally:
        shm.release()


def test_concurrent_clients(served, ocs_lib):
    """Four connections at once: one thread each in the runner, all calling
    ocs_activate concurrently."""
    errors = []

    def client(i):
        try:
            exp, ov, opts = CASES[i % 5]
            x = signal(400 + i, 700_001)
            olen = proxy.to_overlap_length(x.size, ov, 1 << exp)
            shm = proxy.SharedPayload(f"fc{i}", olen)
            try:
                shm.floats()[: x.size] = x
                req = wire.Request(windowRadix=exp, overlapRatio=ov, mappedID=f"fc{i}", sharedMemory=shm.name,
                                   dataLength=x.size, overlapdataLength=olen, options=opts, posixFileDes=-1)
                a = _ask(served, req)
                want = stand_in_out(ocs_lib, x, exp, ov, opts)
                if a.sharedMemory != shm.name or not np.array_equal(shm.floats()[: want.size], want):
                    errors.append(i)
            finally:
                shm.release()
        except Exception as e:  # noqa: BLE001
            errors.append((i, repr(e)))

    th = [threading.Thread(target=client, args=(i,)) for i in range(4)]
    for t in th:
        t.start()
    for t in th:
        t.join()
    assert not errors, errors


def test_proxy_drives_the_runner(stand_in_runner, ocs_lib, tmp_path):
    """STFTProxy launches the runner as a local runtime (`<exe> <port>`),
    sends shared-memory requests and stops it with CLOSE_REQUEST."""
    exe, _ = stand_in_runner
    os.symlink(exe, tmp_path / "serialRun")  # a local runtime the proxy launches from this folder
    p = proxy.STFTProxy([("SERIAL", str(tmp_path))])
    try:
        assert p.status == "OK"
        for exp, ov, opts in CASES[:4]:
            x = signal(exp + 70, 123_457)
            got = p.request_stft(x, exp, ov, opts)
            want = stand_in_out(ocs_lib, x, exp, ov, opts)
            assert got is not None and np.array_equal(got[: want.size], want), (exp, ov, opts)
    finally:
        assert p.kill_runner()


def test_proxy_remote_server(served, ocs_lib):
    """A "SERVER" runtime: the proxy connects to a runner that is already
    listening and sends the signal in the data list instead of shared memory
    (STFTProxy.cpp:118-154, FFTStruct.cpp data-list path)."""
    p = proxy.STFTProxy([("SERVER", f"127.0.0.1:{served}")])
    try:
        assert p.status == "OK" and p.gpu_type == "SERVER"
        for exp, ov, opts in CASES[:4]:
            x = signal(exp + 90, 98_765)
            got = p.request_stft(x, exp, ov, opts)
            want = stand_in_out(ocs_lib, x, exp, ov, opts)
            assert got is not None and np.array_equal(got, want), (exp, ov, opts)
    finally:
        p.ws.close()  # the shared runner keeps serving the other tests


def test_foreign_shared_memory_object_is_not_touched(served):
    """A request naming a shared-memory object outside the protocol's
    "/STFT<mappedID>SHAREDMEM" form is answered "ERR" and the object is
    neither read nor written."""
    from multiprocessing import shared_memory

    seg = shared_memory.SharedMemory(name=f"ocs_foreign_{os.getpid()}", create=True, size=1 << 20)
    try:
        view = np.ndarray((1 << 18,), dtype=np.float32, buffer=seg.buf)
        view[:] = 3.25
        x = signal(5, 100_000)
        req = wire.Request(windowRadix=10, overlapRatio=0.5, mappedID="x", sharedMemory="/" + seg.name,
                           dataLength=x.size, overlapdataLength=proxy.to_overlap_length(x.size, 0.5, 1024),
                           options="", posixFileDes=-1)
        a = _ask(served, req)
        assert a.sharedMemory == "ERR"
        assert np.all(view == 3.25)
        del view
    finally:
        seg.close()
        seg.unlink()
