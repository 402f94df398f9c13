"""The runner executable's protocol, on CPU: the RequestCapnp codec (single
segment, single- and double-far pointers), the WebSocket handshake and
framing of cudaRun, and CLOSE_REQUEST.  Requests here use a window exponent
the pipeline rejects (2^5, "Operation not supported",
RunnerCommon.cpp:250-253), so every answer is "ERR" with or without a GPU and
the answer's echoed fields show what the runner decoded."""
import socket
import struct

import numpy as np
import pytest

from occastft_gb300 import proxy, wire
from tests import cudarun_util as cu


def _req(**kw):
    base = dict(windowRadix=5, overlapRatio=0.5, mappedID="17", posixFileDes=-1, windowsHandlePTR=2**64 - 1,
                dataLength=3, overlapdataLength=64, options="--hanning_window", memPTR=0x7F00DEADBEEF)
    base.update(kw)
    return wire.Request(**base)


@pytest.mark.parametrize("layout", ["single", "far", "double-far"])
def test_wire_round_trip(layout):
    x = np.arange(1000, dtype=np.float32) * 0.25 - 3
    r = _req(data=x, sharedMemory="/STFT17SHAREDMEM", options="--blackman_window --remove_dc")
    d = wire.decode(wire.encode(r, layout))
    for f in ("windowRadix", "mappedID", "posixFileDes", "windowsHandlePTR", "dataLength", "overlapdataLength",
              "options", "memPTR", "sharedMemory"):
        assert getattr(d, f) == getattr(r, f), f
    assert d.overlapRatio == np.float32(0.5)
    assert np.array_equal(d.data, x)


def test_wire_layout_words():
    """Field placement of the schema: data word 3 holds windowRadix (low) and
    overlapRatio (high); the root struct is 6 data words and 4 pointers."""
    b = wire.encode(_req(windowRadix=10, overlapRatio=0.75, dataLength=7, overlapdataLength=9))
    nseg, w0 = struct.unpack_from("<II", b, 0)
    assert nseg == 0
    root = struct.unpack_from("<Q", b, 8)[0]
    assert root & 3 == 0 and (root >> 32) & 0xFFFF == 6 and root >> 48 == 4
    words = struct.unpack_from("<6Q", b, 16)
    assert words[3] & 0xFFFFFFFF == 10
    assert struct.unpack("<f", struct.pack("<I", words[3] >> 32))[0] == 0.75
    assert words[4] == 7 and words[5] == 9


def test_overlap_length_matches_geometry(ocs_lib):
    """The proxy sizes shared memory with toOverlapLength; the runner writes
    OFullSize floats.  Both use the same float arithmetic."""
    for n, exp, ov in [(2**20, 10, 0.5), (1000003, 8, 0.75), (77777, 12, 0.3), (4096, 6, 0.0)]:
        g = ocs_lib.geometry(n, exp, ov, "--hanning_window")
        assert proxy.to_overlap_length(n, ov, 1 << exp) == g.ofull


@pytest.fixture()
def runner():
    p, port = cu.start_cudarun()
    yield p, port
    cu.stop(p)


def test_handshake_known_answer(runner):
    """RFC 6455 section 1.3 sample key and accept value."""
    _, port = runner
    with socket.create_connection(("127.0.0.1", port), timeout=10) as s:
        s.sendall(b"GET / HTTP/1.1\r\nHost: x\r\nUpgrade: websocket\r\nConnection: Upgrade\r\n"
                  b"Sec-WebSocket-Key: dGhlIHNhbXBsZSBub25jZQ==\r\nSec-WebSocket-Version: 13\r\n\r\n")
        resp = b""
        while b"\r\n\r\n" not in resp:
            resp += s.recv(4096)
    assert resp.startswith(b"HTTP/1.1 101")
    assert b"Sec-WebSocket-Accept: s3pPLMBiTxaQ9kYGzzhZRbK+xOo=" in resp
    assert b"permessage-deflate" not in resp


def test_rejects_plain_http(runner):
    _, port = runner
    with socket.create_connection(("127.0.0.1", port), timeout=10) as s:
        s.sendall(b"GET / HTTP/1.1\r\nHost: x\r\n\r\n")
        assert s.recv(4096).startswith(b"HTTP/1.1 400")


@pytest.mark.parametrize("layout", ["single", "far", "double-far"])
@pytest.mark.parametrize("fragments", [1, 3])
def test_error_answer_echoes_fields(runner, layout, fragments):
    _, port = runner
    ws = proxy.WsClient("127.0.0.1", port)
    x = np.linspace(-1, 1, 300, dtype=np.float32)
    r = _req(data=x, dataLength=x.size, mappedID="4242")
    ws.send_binary(wire.encode(r, layout), fragments=fragments)
    op, payload = ws.recv(timeout=30)
    assert op == 2
    a = wire.decode(payload)
    assert a.sharedMemory == "ERR"
    assert a.mappedID == "4242"
    assert (a.windowRadix, a.dataLength, a.overlapdataLength) == (5, x.size, 64)
    assert (a.posixFileDes, a.windowsHandlePTR, a.memPTR) == (-1, 2**64 - 1, 0x7F00DEADBEEF)
    assert a.overlapRatio == np.float32(0.5)
    assert a.options == ""  # the answer does not carry options (FFTStruct.cpp:95-110)
    assert a.data is None
    ws.close()


def test_undecodable_request(runner):
    _, port = runner
    ws = proxy.WsClient("127.0.0.1", port)
    ws.send_binary(b"\x00\x00\x00\x00\xff\x00\x00\x00garbage!")
    op, payload = ws.recv(timeout=30)
    a = wire.decode(payload)
    assert a.sharedMemory == "ERR" and a.mappedID == ""
    ws.close()


def test_missing_shared_memory_object(runner):
    _, port = runner
    ws = proxy.WsClient("127.0.0.1", port)
    ws.send_binary(wire.encode(_req(windowRadix=10, sharedMemory="/STFTnosuchSHAREDMEM", dataLength=10)))
    a = wire.decode(ws.recv(timeout=30)[1])
    assert a.sharedMemory == "ERR" and a.mappedID == "17"
    ws.close()


def test_ping_and_close_frames(runner):
    _, port = runner
    ws = proxy.WsClient("127.0.0.1", port)
    ws.ping(b"hello")
    assert ws.recv(timeout=30) == (10, b"hello")
    ws._send(8, struct.pack(">H", 1000))
    op, payload = ws.recv(timeout=30)
    assert op == 8 and payload == struct.pack(">H", 1000)
    ws.close()


@pytest.mark.parametrize("length", [2**64 - 5, 2**63, 2**37])
def test_oversized_continuation_frame_is_refused(runner, length):
    """A continuation frame whose 64-bit length is above the message limit
    (including lengths whose sum with the bytes already received would wrap,
    and ones with the most significant bit set, which RFC 6455 5.2 forbids)
    is answered with close code 1009 before any payload is stored; the runner
    keeps serving other connections."""
    _, port = runner
    ws = proxy.WsClient("127.0.0.1", port)
    mask = b"\x01\x02\x03\x04"
    first = bytes(range(10))
    ws.sock.sendall(bytes([0x02, 0x80 | len(first)]) + mask + bytes(b ^ mask[i & 3] for i, b in enumerate(first)))
    ws.sock.sendall(bytes([0x80, 0x80 | 127]) + struct.pack(">Q", length) + mask + bytes(64))
    assert ws.recv(timeout=30) == (8, struct.pack(">H", 1009))
    ws.close()
    other = proxy.WsClient("127.0.0.1", port)
    other.ping(b"still serving")
    assert other.recv(timeout=30) == (10, b"still serving")
    other.close()


def _rss_mb(pid):
    for line in open(f"/proc/{pid}/status"):
        if line.startswith("VmRSS:"):
            return int(line.split()[1]) / 1024
    return 0.0


def test_frame_header_alone_allocates_nothing(runner):
    """A header that states an 8 GB payload, followed by 1 MB of it: the
    runner's buffer grows with the bytes that arrive (64 MB steps), so its
    resident memory stays far below the stated length.  Dropping the
    connection mid-frame ends only that connection."""
    import time

    p, port = runner
    before = _rss_mb(p.pid)
    ws = proxy.WsClient("127.0.0.1", port)
    mask = b"\x05\x06\x07\x08"
    ws.sock.sendall(bytes([0x82, 0x80 | 127]) + struct.pack(">Q", 8 << 30) + mask + bytes(1 << 20))
    time.sleep(0.5)
    grown = _rss_mb(p.pid) - before
    assert grown < 256, f"runner grew by {grown:.0f} MB on a header alone"
    ws.sock.close()
    other = proxy.WsClient("127.0.0.1", port)
    other.ping(b"after")
    assert other.recv(timeout=30) == (10, b"after")
    other.close()


def test_silent_peer_is_dropped_after_the_handshake_deadline(runner):
    """A peer that connects and never sends its opening request is closed
    after the handshake deadline (5 s) instead of holding a thread."""
    import time

    _, port = runner
    with socket.create_connection(("127.0.0.1", port), timeout=30) as s:
        t0 = time.time()
        assert s.recv(16) == b""  # closed by the runner
        assert 3 < time.time() - t0 < 20


def test_trickling_peer_is_dropped_at_the_handshake_deadline(runner):
    """A peer that sends its opening request one byte a second is closed
    about 5 s after the accept: the deadline covers the whole handshake, not
    each read."""
    import time

    _, port = runner
    req = b"GET / HTTP/1.1\r\nHost: x\r\nUpgrade: websocket\r\nConnection: Upgrade\r\n"
    with socket.create_connection(("127.0.0.1", port), timeout=30) as s:
        t0 = time.time()
        closed_at = None
        for b in req:
            try:
                s.sendall(bytes([b]))
            except OSError:
                closed_at = time.time()
                break
            s.settimeout(1.0)
            try:
                if s.recv(16) == b"":
                    closed_at = time.time()
                    break
            except socket.timeout:
                pass
        assert closed_at is not None, "the runner kept a trickling peer past its handshake deadline"
        assert 3 < closed_at - t0 < 9


def test_connections_beyond_the_cap_are_refused(runner):
    """At most 256 connections are open at once: the ones beyond are closed at
    accept, the others stay open, and a clean client is served once they go."""
    _, port = runner
    # upgraded connections: the handshake deadline does not apply to them
    held = [proxy.WsClient("127.0.0.1", port) for _ in range(256)]
    try:
        extra = [socket.create_connection(("127.0.0.1", port), timeout=10) for _ in range(8)]
        for s in extra:
            s.settimeout(3)
            assert s.recv(16) == b""  # refused at once, well before the handshake deadline
            s.close()
        held[0].ping(b"held")
        assert held[0].recv(timeout=10) == (10, b"held")  # still served
    finally:
        for ws in held:
            ws.close()
    import time

    deadline = time.time() + 20
    while True:  # the runner reaps the closed connections' threads
        try:
            ws = proxy.WsClient("127.0.0.1", port)
            break
        except (OSError, ConnectionError):
            assert time.time() < deadline
            time.sleep(0.2)
    ws.ping(b"back")
    assert ws.recv(timeout=30) == (10, b"back")
    ws.close()


def test_close_request_stops_runner():
    p, port = cu.start_cudarun()
    try:
        ws = proxy.WsClient("127.0.0.1", port)
        other = proxy.WsClient("127.0.0.1", port)  # a second client is dropped too
        ws.send_text("CLOSE_REQUEST")
        assert ws.recv(timeout=30) == (1, b"CLOSE_COMPLETE")
        assert p.wait(timeout=30) == 0
        other.close()
        ws.close()
    finally:
        cu.stop(p)


def test_bad_port_argument():
    import subprocess

    cu.ensure_built()
    r = subprocess.run([cu.CUDARUN, "notaport"], capture_output=True, text=True, timeout=60)
    assert r.returncode == 1 and "bad port" in r.stderr
