"""A CPU runner for tests: the reference's Serial runner behind the runner
protocol, computed by the oracle's restatement of the reference's serial
pipeline (oracle/stft_oracle.c).  It plays `serialRun` in the proxy fallback
test (StandAlone/src/runtimeChecker.cpp:19-31 launches `<exe> <port>`):
WebSocket on 0.0.0.0:<port>, RequestCapnp binary messages with the signal in
POSIX shared memory or in the data list, "CLOSE_REQUEST" -> "CLOSE_COMPLETE".

Test infrastructure only: the oracle never serves product requests."""
import base64
import hashlib
import mmap
import os
import socket
import struct
import sys
import threading

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

from occastft_gb300 import proxy, wire  # noqa: E402
from oracle import orc  # noqa: E402

GUID = "258EAFA5-E914-47DA-95CA-C5AB0DC85B11"
stop = threading.Event()


def recv_exact(c, n):
    b = bytearray()
    while len(b) < n:
        k = c.recv(n - len(b))
        if not k:
            raise ConnectionError
        b += k
    return bytes(b)


def send_frame(c, op, payload):
    n = len(payload)
    h = bytes([0x80 | op])
    h += bytes([n]) if n < 126 else (bytes([126]) + struct.pack(">H", n) if n <= 0xFFFF else
                                     bytes([127]) + struct.pack(">Q", n))
    c.sendall(h + payload)


def compute(req):
    exp, ov = req.windowRadix, req.overlapRatio
    if req.sharedMemory:
        path = "/dev/shm" + req.sharedMemory
        nbytes = proxy.page_rounded(req.overlapdataLength * 4)
        fd = os.open(path, os.O_RDWR)
        try:
            m = mmap.mmap(fd, nbytes, mmap.MAP_SHARED, mmap.PROT_READ | mmap.PROT_WRITE)
        finally:
            os.close(fd)
        x = np.frombuffer(m, dtype=np.float32, count=req.dataLength).copy()
        out = orc.serial_pipeline(x, exp, ov, req.options)
        np.frombuffer(m, dtype=np.float32, count=out.size)[:] = out
        del x
        m.close()
        return None
    return orc.serial_pipeline(np.asarray(req.data, dtype=np.float32), exp, ov, req.options)


def serve(c):
    hdr = b""
    while b"\r\n\r\n" not in hdr:
        k = c.recv(4096)
        if not k:
            return
        hdr += k
    key = [ln.split(b":", 1)[1].strip().decode() for ln in hdr.split(b"\r\n")
           if ln.lower().startswith(b"sec-websocket-key:")][0]
    acc = base64.b64encode(hashlib.sha1((key + GUID).encode()).digest()).decode()
    c.sendall(("HTTP/1.1 101 Switching Protocols\r\nUpgrade: websocket\r\nConnection: Upgrade\r\n"
               f"Sec-WebSocket-Accept: {acc}\r\n\r\n").encode())
    parts, first = [], None
    while not stop.is_set():
        h = recv_exact(c, 2)
        op, n = h[0] & 0x0F, h[1] & 0x7F
        if n == 126:
            n = struct.unpack(">H", recv_exact(c, 2))[0]
        elif n == 127:
            n = struct.unpack(">Q", recv_exact(c, 8))[0]
        key = recv_exact(c, 4)
        data = bytearray(recv_exact(c, n))
        for i in range(n):
            data[i] ^= key[i & 3]
        if op == 9:
            send_frame(c, 10, bytes(data))
            continue
        if op == 8:
            send_frame(c, 8, bytes(data[:2]))
            return
        if op != 0:
            first = op
        parts.append(bytes(data))
        if not h[0] & 0x80:
            continue
        msg, parts = b"".join(parts), []
        if first == 1:
            if msg == b"CLOSE_REQUEST":
                send_frame(c, 1, b"CLOSE_COMPLETE")
                stop.set()
                return
            continue
        req = wire.decode(msg)
        ans = wire.Request(windowRadix=req.windowRadix, overlapRatio=req.overlapRatio, mappedID=req.mappedID,
                           sharedMemory=req.sharedMemory, memPTR=req.memPTR, posixFileDes=req.posixFileDes,
                           windowsHandlePTR=req.windowsHandlePTR, dataLength=req.dataLength,
                           overlapdataLength=req.overlapdataLength)
        try:
            out = compute(req)
            if out is not None:
                ans.data = out
                ans.dataLength = out.size
        except Exception:  # noqa: BLE001  (any failure answers ERR, as the reference does)
            ans.sharedMemory = "ERR"
        send_frame(c, 2, wire.encode(ans))


def main():
    port = int(sys.argv[1]) if len(sys.argv) > 1 else 54500
    ls = socket.socket()
    ls.setsockopt(socket.SOL_SOCKET, socket.SO_REUSEADDR, 1)
    ls.bind(("0.0.0.0", port))
    ls.listen(8)
    ls.settimeout(0.2)
    while not stop.is_set():
        try:
            c, _ = ls.accept()
        except socket.timeout:
            continue
        threading.Thread(target=lambda: (serve_safe(c)), daemon=True).start()
    ls.close()


def serve_safe(c):
    try:
        serve(c)
    except (ConnectionError, OSError):
        pass
    finally:
        c.close()


if __name__ == "__main__":
    main()
