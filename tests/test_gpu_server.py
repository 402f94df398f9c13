"""The continuous-batching server (ocs_server_*): every result equals the same
request served alone (bit for bit, same batch kernel) and the FP64 oracle;
admission under a small device pool; cancel, timeout and statistics."""
import threading

import numpy as np
import pytest

from tests.conftest import signal

REL_L2 = 1e-5
pytestmark = pytest.mark.gpu


def _draw(k, rng):
    exp = int(rng.choice([8, 9, 10, 11, 12]))
    n = int(round(2 ** rng.uniform(12, 18)))
    ov = float(rng.choice([0.25, 0.5, 0.75]))
    win = str(rng.choice(["--hanning_window", "--hamming_window", "--blackman_window"]))
    out = " --half_complex_return" if k % 2 else ""
    return signal(3000 + k, n), exp, ov, win + out


@pytest.fixture
def server(ocs_lib):
    s = ocs_lib.Server(pool_bytes=256 << 20, max_batch=64, slots=3)
    yield s
    s.stop()


def test_alone_equals_in_the_mix(ocs_lib, orc, server):
    rng = np.random.default_rng(11)
    reqs = [_draw(k, rng) for k in range(60)]
    outs_alone = []
    for (x, exp, ov, opts) in reqs[:5]:
        o = np.empty(ocs_lib.geometry(x.size, exp, ov, opts).out_floats, np.float32)
        assert server.wait(server.submit(x, exp, ov, opts, o), 30000) == 0
        outs_alone.append(o)
    # the same five again, in a burst of 60 submitted from 4 threads
    outs = [np.empty(ocs_lib.geometry(x.size, e, ov, op).out_floats, np.float32) for (x, e, ov, op) in reqs]
    tickets = [None] * len(reqs)

    def submit(idx):
        for i in idx:
            x, exp, ov, opts = reqs[i]
            tickets[i] = server.submit(x, exp, ov, opts, outs[i])

    th = [threading.Thread(target=submit, args=(list(range(t, 60, 4)),)) for t in range(4)]
    for t in th:
        t.start()
    for t in th:
        t.join()
    assert all(server.wait(t, 60000) == 0 for t in tickets)
    for i in range(5):
        assert np.array_equal(outs[i], outs_alone[i]), i
    for i in (0, 7, 33, 59):
        x, exp, ov, opts = reqs[i]
        assert orc.rel_l2(outs[i], orc.fp64_stft(x, exp, ov, opts)) <= REL_L2, i
    st = server.stats()
    assert st["completed"] >= 65 and st["p50_ms"] > 0 and st["p99_ms"] >= st["p50_ms"]
    assert st["batches"] < st["completed"]  # requests were coalesced


def test_admission_with_small_pool(ocs_lib, orc):
    s = ocs_lib.Server(pool_bytes=24 << 20, max_batch=64, slots=2)
    try:
        rng = np.random.default_rng(12)
        reqs = [(signal(4000 + k, 600_000), int(rng.choice([9, 10, 11])), 0.5, "--hanning_window") for k in range(24)]
        outs = [np.empty(ocs_lib.geometry(x.size, e, ov, op).out_floats, np.float32) for (x, e, ov, op) in reqs]
        ts = [s.submit(x, e, ov, op, o) for (x, e, ov, op), o in zip(reqs, outs)]
        assert all(s.wait(t, 60000) == 0 for t in ts)
        for (x, e, ov, op), o in list(zip(reqs, outs))[::5]:
            assert orc.rel_l2(o, orc.fp64_stft(x, e, ov, op)) <= REL_L2
        big = signal(1, 8_000_000)
        with pytest.raises(ocs_lib.OcsError) as ei:
            s.submit(big, 10, 0.5, "", np.empty(ocs_lib.geometry(big.size, 10, 0.5, "").out_floats, np.float32))
        assert ei.value.code == ocs_lib.OCS_ENOMEM
        assert s.stats()["rejected"] == 1
    finally:
        s.stop()


def test_cancel_timeout_and_errors(ocs_lib, server):
    x = signal(9, 1 << 20)
    o = np.empty(ocs_lib.geometry(x.size, 10, 0.5, "").out_floats, np.float32)
    with pytest.raises(ocs_lib.OcsError):
        server.submit(x, 5, 0.5, "", o)  # exponent below 6: refused at submit
    ts = [server.submit(x, 10, 0.5, "", np.empty_like(o)) for _ in range(40)]
    cancelled = 0
    for t in ts[::-1][:10]:
        try:
            server.cancel(t)
            cancelled += 1
            with pytest.raises(ocs_lib.OcsError):
                server.wait(t, 0)  # a withdrawn request is gone
        except ocs_lib.OcsError:
            pass  # already admitted to the device: it will finish normally
    for t in ts:
        try:
            assert server.wait(t, 60000) == 0
        except ocs_lib.OcsError:
            pass  # cancelled above
    # a bounded wait on an unfinished request times out without blocking
    t = server.submit(x, 10, 0.5, "", o)
    try:
        server.wait(t, 0)
    except ocs_lib.OcsError as e:
        assert e.code == ocs_lib.OCS_ETIMEDOUT
        assert server.wait(t, 60000) == 0
