"""The runner executable on the GPU: requests through the WebSocket protocol
(data list and POSIX shared memory, single- and multi-segment messages)
against the FP64 oracle and against the C ABI, the proxy driving cudaRun,
and the proxy falling back to the oracle's serial runner when cudaRun dies."""
import os

import numpy as np
import pytest

from occastft_gb300 import proxy, wire
from tests import cudarun_util as cu
from tests.conftest import signal
from tests.test_standalone_proxy import make_serial_runner

pytestmark = pytest.mark.gpu
REL_L2 = 1e-5

CASES = [
    (10, 0.5, "--hamming_window"),
    (8, 0.75, "--hanning_window --remove_dc --half_complex_return"),
    (12, 0.5, "--blackman_window --layout=dense"),
    (6, 0.25, "--flattop_window --serial_power"),
    (10, 0.75, "--hanning_window --precision=tc-fp16"),
]


@pytest.fixture(scope="module")
def runner():
    p, port = cu.start_cudarun()
    yield p, port
    cu.stop(p)


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
@pytest.mark.parametrize("layout", ["single", "far"])
def test_data_list_request(runner, orc, ocs_lib, exp, ov, opts, layout):
    _, port = runner
    x = signal(exp * 7 + 1, 250_001)
    req = wire.Request(windowRadix=exp, overlapRatio=ov, mappedID="9", dataLength=x.size,
                       overlapdataLength=proxy.to_overlap_length(x.size, ov, 1 << exp), options=opts, data=x)
    a = _ask(port, req, layout)
    assert a.sharedMemory == "" and a.mappedID == "9"
    assert a.data is not None and a.dataLength == a.data.size
    base = opts.replace(" --precision=tc-fp16", "")
    ref = orc.fp64_stft(x, exp, ov, base)
    assert a.data.size == ref.size
    assert orc.rel_l2(a.data, ref) <= REL_L2
    direct = ocs_lib.activate(x, exp, ov, opts)
    assert orc.rel_l2(a.data, direct) <= 1e-6


@pytest.mark.parametrize("exp,ov,opts", CASES)
def test_shared_memory_request(runner, orc, exp, ov, opts):
    _, port = runner
    x = signal(exp * 11 + 5, 400_003)
    olen = proxy.to_overlap_length(x.size, ov, 1 << exp)
    shm = proxy.SharedPayload("gpu" + str(exp), olen)
    try:
        shm.floats()[: x.size] = x
        req = wire.Request(windowRadix=exp, overlapRatio=ov, mappedID="gpu" + str(exp), sharedMemory=shm.name,
                           dataLength=x.size, overlapdataLength=olen, options=opts, posixFileDes=-1)
        a = _ask(port, req, "double-far")
        assert a.sharedMemory == shm.name and a.dataLength == x.size and a.data is None
        base = opts.replace(" --precision=tc-fp16", "")
        ref = orc.fp64_stft(x, exp, ov, base)
        got = shm.floats()[: ref.size].copy()
        assert orc.rel_l2(got, ref) <= REL_L2
    finally:
        shm.release()


def test_fragmented_large_request(runner, orc):
    _, port = runner
    x = signal(99, 3_000_000)
    req = wire.Request(windowRadix=10, overlapRatio=0.5, mappedID="big", dataLength=x.size,
                       overlapdataLength=proxy.to_overlap_length(x.size, 0.5, 1024), options="--hanning_window",
                       data=x)
    a = _ask(port, req, "far", fragments=7)
    assert orc.rel_l2(a.data, orc.fp64_stft(x, 10, 0.5, "--hanning_window")) <= REL_L2


def test_geometry_error_answers_err(runner):
    _, port = runner
    req = wire.Request(windowRadix=10, overlapRatio=1.0, mappedID="bad", dataLength=10, options="",
                       data=np.ones(10, np.float32))
    assert _ask(port, req).sharedMemory == "ERR"


def test_proxy_drives_cudarun(orc):
    cu.ensure_built()
    p = proxy.STFTProxy([("CUDA", os.path.dirname(cu.CUDARUN))])
    try:
        assert p.gpu_type == "CUDA"
        x = signal(12, 1_000_000)
        got = p.request_stft(x, 10, 0.5, "--hanning_window --remove_dc --half_complex_return")
        ref = orc.fp64_stft(x, 10, 0.5, "--hanning_window --remove_dc --half_complex_return")
        assert orc.rel_l2(got[: ref.size], ref) <= REL_L2
    finally:
        assert p.kill_runner()


def test_proxy_falls_back_to_serial_runner(tmp_path, orc):
    """CUDAFallback -> cudaRun; cudaRun dies (injected on the host: the
    process is killed between requests); the next request is served by the
    next runtime of the list, the oracle's serial runner."""
    cu.ensure_built()
    errs = []
    p = proxy.STFTProxy([("CUDA", os.path.dirname(cu.CUDARUN)), ("SERIAL", make_serial_runner(str(tmp_path)))],
                        errs.append)
    try:
        x = signal(13, 200_000)
        opts = "--hamming_window"
        got_gpu = p.request_stft(x, 10, 0.5, opts)
        assert p.gpu_type == "CUDA"
        assert orc.rel_l2(got_gpu, orc.fp64_stft(x, 10, 0.5, opts)) <= REL_L2
        p.runner.kill()
        p.runner.wait()
        got_cpu = p.request_stft(x, 10, 0.5, opts)
        assert p.gpu_type == "SERIAL" and errs
        assert np.array_equal(got_cpu, orc.serial_pipeline(x, 10, 0.5, opts))
    finally:
        p.kill_runner()
