"""STFT proxy: the client side of the runner protocol, in Python.

Restates the reference's STFTProxy (StandAlone/src/STFTProxy.cpp:4-211,
StandAlone/include/STFTProxy.hpp) and the parts of FFTRequest a client uses
(StandAlone/src/FFTStruct_linux.cpp:5-100): pick the first available runtime
of a fallback list, launch its runner executable as `<exe> <port>` on a free
port (or connect to a remote "SERVER"), send RequestCapnp messages over a
WebSocket, and stop the runner with "CLOSE_REQUEST".  Local runners receive
the signal through a POSIX shared memory object "/STFT<id>SHAREDMEM" that the
runner overwrites with the result; a remote server gets it in the data list.

Differences from the reference, on purpose: requests are synchronous (the
reference returns a future); when the connection fails during a request the
request is sent again once to the next runtime of the list (the reference
moves to the next runtime but leaves that request's future unfulfilled).
"""
from __future__ import annotations

import base64
import ctypes
import hashlib
import mmap
import os
import random
import socket
import struct
import subprocess
import time
from typing import Callable, List, Optional, Tuple

import numpy as np

from . import wire

RUNNER_NAMES = {"CUDA": "cudaRun", "HIP": "hipRun", "OPENCL": "openclRun", "OPENMP": "openmpRun",
                "SERIAL": "serialRun", "METAL": "metalRun"}
_DRIVER_LIBS = {"CUDA": "libcuda.so.1", "HIP": "libamdhip64.so", "OPENCL": "libOpenCL.so.1"}
_GUID = "258EAFA5-E914-47DA-95CA-C5AB0DC85B11"


def to_overlap_length(data_length: int, overlap_ratio: float, window_size: int) -> int:
    """FFTRequest::toOverlapLength (FFTStruct.cpp:145-157): float arithmetic,
    truncated."""
    f32 = np.float32
    if f32(overlap_ratio) == f32(0.0):
        quot = data_length // window_size + 1
    else:
        q = f32(data_length) / (f32(window_size) * (f32(1.0) - f32(overlap_ratio)))
        quot = int(q) + 1
    return quot * window_size


def page_rounded(nbytes: int) -> int:
    page = mmap.PAGESIZE
    return (nbytes + page - 1) // page * page


# ------------------------------------------------------------ WebSocket client
class WsClosed(ConnectionError):
    pass


class WsClient:
    """Minimal RFC 6455 client: masked frames, ping answers, fragmentation."""

    def __init__(self, host: str, port: int, timeout: float = 5.0):
        self.sock = socket.create_connection((host, port), timeout=timeout)
        self.sock.setsockopt(socket.IPPROTO_TCP, socket.TCP_NODELAY, 1)
        # a runner that is still initialising its device answers the
        # handshake late: give it longer than the connect
        self.sock.settimeout(max(timeout, 60.0))
        key = base64.b64encode(os.urandom(16)).decode()
        req = (f"GET / HTTP/1.1\r\nHost: {host}:{port}\r\nUpgrade: websocket\r\nConnection: Upgrade\r\n"
               f"Sec-WebSocket-Key: {key}\r\nSec-WebSocket-Version: 13\r\n"
               "Sec-WebSocket-Extensions: permessage-deflate; client_max_window_bits\r\n\r\n")
        self.sock.sendall(req.encode())
        resp = b""
        while b"\r\n\r\n" not in resp:
            chunk = self.sock.recv(4096)
            if not chunk:
                raise WsClosed("connection closed during the handshake")
            resp += chunk
        head = resp.split(b"\r\n\r\n", 1)[0].decode(errors="replace")
        if " 101 " not in head.split("\r\n")[0] + " ":
            raise ConnectionError("handshake refused: " + head.split("\r\n")[0])
        want = base64.b64encode(hashlib.sha1((key + _GUID).encode()).digest()).decode()
        accept = [ln.split(":", 1)[1].strip() for ln in head.split("\r\n")[1:]
                  if ln.lower().startswith("sec-websocket-accept:")]
        if accept != [want]:
            raise ConnectionError("bad Sec-WebSocket-Accept")
        self.sock.settimeout(None)

    def _send(self, opcode: int, payload: bytes, fin: bool = True):
        n = len(payload)
        h = bytes([(0x80 if fin else 0) | opcode])
        if n < 126:
            h += bytes([0x80 | n])
        elif n <= 0xFFFF:
            h += bytes([0x80 | 126]) + struct.pack(">H", n)
        else:
            h += bytes([0x80 | 127]) + struct.pack(">Q", n)
        mask = os.urandom(4)
        if n:
            m = np.frombuffer(mask * 2, dtype=np.uint64)[0]
            pad = (-n) % 8
            arr = np.frombuffer(payload + b"\0" * pad, dtype=np.uint64) ^ m
            payload = arr.tobytes()[:n]
        self.sock.sendall(h + mask + payload)

    def send_text(self, s: str):
        self._send(1, s.encode())

    def send_binary(self, b: bytes, fragments: int = 1):
        if fragments <= 1 or len(b) < fragments:
            self._send(2, b)
            return
        step = (len(b) + fragments - 1) // fragments
        parts = [b[i:i + step] for i in range(0, len(b), step)]
        for i, p in enumerate(parts):
            self._send(2 if i == 0 else 0, p, fin=(i == len(parts) - 1))

    def ping(self, payload: bytes = b""):
        self._send(9, payload)

    def close(self, code: int = 1000):
        try:
            self._send(8, struct.pack(">H", code))
        except OSError:
            pass
        try:
            self.sock.close()
        except OSError:
            pass

    def _recv_exact(self, n: int) -> bytes:
        buf = bytearray(n)
        view = memoryview(buf)
        got = 0
        while got < n:
            k = self.sock.recv_into(view[got:], n - got)
            if k == 0:
                raise WsClosed("connection closed")
            got += k
        return bytes(buf)

    def recv(self, timeout: Optional[float] = None) -> Tuple[int, bytes]:
        """Next data message as (opcode, payload); answers pings on the way.
        Returns (10, payload) for a pong and (8, payload) for a close."""
        self.sock.settimeout(timeout)
        try:
            chunks = []
            first_op = None
            while True:
                h = self._recv_exact(2)
                fin, op = h[0] & 0x80, h[0] & 0x0F
                n = h[1] & 0x7F
                if n == 126:
                    n = struct.unpack(">H", self._recv_exact(2))[0]
                elif n == 127:
                    n = struct.unpack(">Q", self._recv_exact(8))[0]
                if h[1] & 0x80:
                    raise ConnectionError("server frames must not be masked")
                payload = self._recv_exact(n) if n else b""
                if op == 9:
                    self._send(10, payload)
                    continue
                if op in (8, 10):
                    return op, payload
                if op != 0:
                    first_op = op
                chunks.append(payload)
                if fin:
                    return first_op, b"".join(chunks)
        finally:
            self.sock.settimeout(None)


# ------------------------------------------------------------ shared memory
class SharedPayload:
    """The proxy's shared memory object for one request (MakeSharedMemory and
    FreeAndGetData, FFTStruct_linux.cpp:5-100)."""

    def __init__(self, mapped_id: str, overlap_floats: int):
        self.name = "/STFT" + mapped_id + "SHAREDMEM"
        self.bytes = page_rounded(overlap_floats * 4)
        self.path = "/dev/shm" + self.name
        fd = os.open(self.path, os.O_CREAT | os.O_RDWR, 0o666)
        try:
            os.ftruncate(fd, self.bytes)
            self.map = mmap.mmap(fd, self.bytes, mmap.MAP_SHARED, mmap.PROT_READ | mmap.PROT_WRITE)
        finally:
            os.close(fd)

    def floats(self) -> np.ndarray:
        return np.frombuffer(self.map, dtype=np.float32)

    def release(self):
        try:
            self.map.close()
        except (BufferError, ValueError):
            pass
        try:
            os.unlink(self.path)
        except FileNotFoundError:
            pass


# ------------------------------------------------------------ proxy
def _free_port() -> int:
    rng = random.Random()
    while True:
        port = rng.randint(49152, 65535)
        with socket.socket() as s:
            try:
                s.setsockopt(socket.SOL_SOCKET, socket.SO_REUSEADDR, 1)
                s.bind(("0.0.0.0", port))
                return port
            except OSError:
                continue


def runtime_available(kind: str, path: str) -> Optional[str]:
    """RuntimeCheck::isAvailable (runtimeChecker.cpp:128-266): the driver
    library loads and the runner executable exists.  Returns the executable
    (or "host:port" for SERVER), else None."""
    if kind == "SERVER":
        return path
    lib = _DRIVER_LIBS.get(kind)
    if lib:
        try:
            ctypes.CDLL(lib)
        except OSError:
            return None
    exe = path
    if kind in RUNNER_NAMES and os.path.basename(path) != RUNNER_NAMES[kind]:
        exe = os.path.join(path, RUNNER_NAMES[kind])
    return os.path.abspath(exe) if os.path.isfile(exe) and os.access(exe, os.X_OK) else None


class STFTProxy:
    def __init__(self, fallback: List[Tuple[str, str]], error_callback: Optional[Callable[[str], None]] = None):
        self.fallback = list(fallback)
        self.error_callback = error_callback or (lambda msg: None)
        self.port_number = _free_port()
        self.status = "OK"
        self.gpu_type: Optional[str] = None
        self.runner: Optional[subprocess.Popen] = None
        self.ws: Optional[WsClient] = None
        self.counter = 0
        self._runtime_fallback()

    def _reap_runner(self):
        """Ends and waits for the runner this proxy launched, so a runner
        that a fallback leaves behind is not left running or unreaped."""
        if self.runner is not None:
            if self.runner.poll() is None:
                self.runner.kill()
            self.runner.wait()
            self.runner = None

    # RuntimeFallback / TryConnect (STFTProxy.cpp:83-154)
    def _runtime_fallback(self):
        if self.ws is not None:
            self.ws.close()
            self.ws = None
        self._reap_runner()
        while self.status == "OK":
            if not self.fallback:
                self.status = "Run Out Fallback"
                return
            kind, path = self.fallback.pop(0)
            if self._try_connect(kind, path):
                self.gpu_type = kind
                return

    def _try_connect(self, kind: str, path: str) -> bool:
        target = runtime_available(kind, path)
        if target is None:
            return False
        if kind == "SERVER":
            host, port = target.rsplit(":", 1)
            port = int(port)
        else:
            self.port_number = _free_port()
            try:
                self.runner = subprocess.Popen([target, str(self.port_number)])
            except OSError:
                return False
            host, port = "127.0.0.1", self.port_number
        for _ in range(5):
            try:
                self.ws = WsClient(host, port, timeout=1.0)
                return True
            except OSError:
                time.sleep(0.5)
        self._reap_runner()  # launched but never reachable
        return False

    def request_stft(self, data, window_size_exp: int, overlap_rate: float = 0.5,
                     options: str = "--hanning_window --remove_dc --half_complex_return") -> Optional[np.ndarray]:
        """RequestSTFT (STFTProxy.cpp:186-211) and the answer's
        FreeAndGetData: the result (OFullSize floats), or None on failure."""
        for attempt in range(2):
            if self.status != "OK" or self.ws is None:
                return None
            try:
                return self._request_once(np.ascontiguousarray(data, dtype=np.float32), window_size_exp,
                                          overlap_rate, options)
            except (OSError, ConnectionError) as e:
                self.error_callback(str(e))
                self._runtime_fallback()
        return None

    def _request_once(self, x: np.ndarray, exp: int, ov: float, options: str) -> Optional[np.ndarray]:
        mapped_id = str(self.counter)
        self.counter += 1
        olen = to_overlap_length(x.size, ov, 1 << exp)
        req = wire.Request(windowRadix=exp, overlapRatio=ov, mappedID=mapped_id, posixFileDes=-1,
                           windowsHandlePTR=2**64 - 1, dataLength=x.size, overlapdataLength=olen, options=options)
        shm = None
        try:
            if self.gpu_type != "SERVER":
                shm = SharedPayload(mapped_id, olen)
                shm.floats()[: x.size] = x
                req.sharedMemory = shm.name
            else:
                req.data = x
            self.ws.send_binary(wire.encode(req))
            while True:
                op, payload = self.ws.recv()
                if op == 2:
                    break
                if op == 8:
                    raise WsClosed("runner closed the connection")
            ans = wire.decode(payload)
            if ans.sharedMemory == "ERR":
                return None
            if shm is not None:
                return shm.floats()[:olen].copy()
            return None if ans.data is None else ans.data.copy()
        finally:
            if shm is not None:
                shm.release()

    def kill_runner(self, no_fallback_any_more: bool = True) -> bool:
        """KillRunner (STFTProxy.cpp:156-184)."""
        if no_fallback_any_more:
            self.status = "NOFALLBACK"
        ok = False
        if self.ws is not None and self.runner is not None:
            try:
                self.ws.send_text("CLOSE_REQUEST")
                deadline = time.time() + 5
                while time.time() < deadline:
                    op, payload = self.ws.recv(timeout=max(0.1, deadline - time.time()))
                    if op == 1 and payload == b"CLOSE_COMPLETE":
                        ok = True
                        break
            except (OSError, ConnectionError):
                ok = False
        if self.ws is not None:
            self.ws.close()
            self.ws = None
        if self.runner is not None:
            try:
                self.runner.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.runner.kill()
                self.runner.wait()
            self.runner = None
        return ok
