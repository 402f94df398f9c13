"""RequestCapnp messages in pure Python (no Cap'n Proto library).

The reference's proxy and runners exchange one Cap'n Proto struct per
WebSocket binary message (StandAlone/include/FFTcapnp.capnp:1-16), written as
a flat array (StandAlone/src/FFTStruct.cpp:41-53).  Layout the capnp compiler
assigns to that schema (6 data words, 4 pointers):

    data word 0 memPTR (u64), 1 posixFileDes (i64), 2 windowsHandlePTR (u64),
    word 3: windowRadix (u32, low half), overlapRatio (f32, high half),
    word 4 dataLength (u64), 5 overlapdataLength (u64);
    pointer 0 sharedMemory (Text), 1 data (List(Float32)), 2 mappedID (Text),
    3 options (Text).

`encode` writes single-segment messages, or (for tests of readers) spreads
the pointed-to objects over extra segments behind single- or double-far
pointers, as Cap'n Proto's builders do for large lists.  `decode` reads any
of these.
"""
from __future__ import annotations

import struct
from dataclasses import dataclass, field
from typing import Optional

import numpy as np

DATA_WORDS = 6
POINTERS = 4
P_SHARED, P_DATA, P_ID, P_OPTIONS = 0, 1, 2, 3


@dataclass
class Request:
    sharedMemory: str = ""  # noqa: N815 (schema field names)
    mappedID: str = ""  # noqa: N815
    options: str = ""
    memPTR: int = 0  # noqa: N815
    posixFileDes: int = 0  # noqa: N815
    windowsHandlePTR: int = 0  # noqa: N815
    windowRadix: int = 0  # noqa: N815
    overlapRatio: float = 0.0  # noqa: N815
    dataLength: int = 0  # noqa: N815
    overlapdataLength: int = 0  # noqa: N815
    data: Optional[np.ndarray] = field(default=None, repr=False)


class WireError(ValueError):
    pass


# ------------------------------------------------------------ pointers
def _struct_ptr(off: int, dw: int, pc: int) -> int:
    return ((off << 2) & 0xFFFFFFFC) | (dw << 32) | (pc << 48)


def _list_ptr(off: int, esize: int, count: int) -> int:
    return 1 | ((off << 2) & 0xFFFFFFFC) | (esize << 32) | (count << 35)


def _far_ptr(pad_word: int, seg: int, double: bool = False) -> int:
    return 2 | (int(double) << 2) | (pad_word << 3) | (seg << 32)


def _text_bytes(s: str) -> bytes:
    b = s.encode() + b"\0"
    return b + b"\0" * ((-len(b)) % 8)


def encode(req: Request, layout: str = "single") -> bytes:
    """Flat-array message.  layout: "single" (one segment), "far" (texts and
    data in segment 1 behind single-far pointers) or "double-far" (content in
    segment 1, two-word landing pads in segment 2)."""
    data = None if req.data is None else np.ascontiguousarray(req.data, dtype=np.float32)
    objs = []  # (pointer slot, kind, payload bytes, count)
    for slot, s in ((P_SHARED, req.sharedMemory), (P_ID, req.mappedID), (P_OPTIONS, req.options)):
        if s:
            objs.append((slot, 2, _text_bytes(s), len(s.encode()) + 1))
    if data is not None and data.size:
        b = data.tobytes()
        objs.append((P_DATA, 4, b + b"\0" * ((-len(b)) % 8), data.size))

    w3 = (req.windowRadix & 0xFFFFFFFF) | (struct.unpack("<I", struct.pack("<f", req.overlapRatio))[0] << 32)
    dwords = [req.memPTR & (2**64 - 1), req.posixFileDes & (2**64 - 1), req.windowsHandlePTR & (2**64 - 1), w3,
              req.dataLength, req.overlapdataLength]
    seg0 = [_struct_ptr(0, DATA_WORDS, POINTERS)] + dwords + [0] * POINTERS
    segs = [seg0]
    blobs = [b""]
    if layout == "single":
        tail = b""
        nxt = 1 + DATA_WORDS + POINTERS
        for slot, esize, payload, count in objs:
            at = 1 + DATA_WORDS + slot
            seg0[at] = _list_ptr(nxt - at - 1, esize, count)
            tail += payload
            nxt += len(payload) // 8
        blobs[0] = tail
    elif layout == "far":
        s1 = b""
        w = 0
        for slot, esize, payload, count in objs:
            at = 1 + DATA_WORDS + slot
            seg0[at] = _far_ptr(w, 1)
            s1 += struct.pack("<Q", _list_ptr(0, esize, count)) + payload  # pad right before the content
            w += 1 + len(payload) // 8
        segs.append([])
        blobs.append(s1)
    elif layout == "double-far":
        s1 = b""
        s2 = b""
        w1 = 0
        w2 = 0
        for slot, esize, payload, count in objs:
            at = 1 + DATA_WORDS + slot
            seg0[at] = _far_ptr(w2, 2, double=True)
            s2 += struct.pack("<QQ", _far_ptr(w1, 1), _list_ptr(0, esize, count))
            s1 += payload
            w1 += len(payload) // 8
            w2 += 2
        segs += [[], []]
        blobs += [s1, s2]
    else:
        raise ValueError(layout)
    seg_bytes = []
    for words, blob in zip(segs, blobs):
        seg_bytes.append(b"".join(struct.pack("<Q", x) for x in words) + blob)
    n = len(seg_bytes)
    table = struct.pack("<I", n - 1) + b"".join(struct.pack("<I", len(sb) // 8) for sb in seg_bytes)
    table += b"\0" * ((-len(table)) % 8)
    return table + b"".join(seg_bytes)


# ------------------------------------------------------------ decode
def _sext30(p: int) -> int:
    v = (p & 0xFFFFFFFF) >> 2
    return v - (1 << 30) if v & (1 << 29) else v


def decode(buf: bytes) -> Request:
    mv = memoryview(buf)
    if len(mv) < 8:
        raise WireError("short message")
    nseg = struct.unpack_from("<I", mv, 0)[0] + 1
    table = (4 * (1 + nseg) + 7) // 8 * 8
    sizes = struct.unpack_from("<%dI" % nseg, mv, 4)
    starts = []
    off = table
    for s in sizes:
        starts.append(off)
        off += s * 8
    if off > len(mv):
        raise WireError("segments run past the message")

    def word(seg, w):
        if w >= sizes[seg]:
            raise WireError("pointer outside its segment")
        return struct.unpack_from("<Q", mv, starts[seg] + 8 * w)[0]

    def resolve(seg, at):
        p = word(seg, at)
        if p == 0:
            return None
        kind = p & 3
        if kind in (0, 1):
            return seg, at + 1 + _sext30(p), p
        if kind != 2:
            raise WireError("capability pointer")
        pad = (p >> 3) & 0x1FFFFFFF
        ps = p >> 32
        if not (p >> 2) & 1:
            q = word(ps, pad)
            return ps, pad + 1 + _sext30(q), q
        f = word(ps, pad)
        tag = word(ps, pad + 1)
        return f >> 32, (f >> 3) & 0x1FFFFFFF, tag

    root = resolve(0, 0)
    if root is None or root[2] & 3:
        raise WireError("root is not a struct")
    rs, rw, rp = root
    dw, pc = (rp >> 32) & 0xFFFF, (rp >> 48) & 0xFFFF

    def dword(i):
        return word(rs, rw + i) if i < dw else 0

    def text(i):
        if i >= pc:
            return ""
        t = resolve(rs, rw + dw + i)
        if t is None:
            return ""
        s, w, tag = t
        n = tag >> 35
        if n == 0:
            return ""
        b = bytes(mv[starts[s] + 8 * w: starts[s] + 8 * w + n - 1])
        return b.decode()

    r = Request()
    r.memPTR, r.posixFileDes, r.windowsHandlePTR = dword(0), dword(1), dword(2)
    if r.posixFileDes >= 2**63:
        r.posixFileDes -= 2**64
    w3 = dword(3)
    r.windowRadix = w3 & 0xFFFFFFFF
    r.overlapRatio = struct.unpack("<f", struct.pack("<I", w3 >> 32))[0]
    r.dataLength, r.overlapdataLength = dword(4), dword(5)
    r.sharedMemory, r.mappedID, r.options = text(P_SHARED), text(P_ID), text(P_OPTIONS)
    if pc > P_DATA:
        t = resolve(rs, rw + dw + P_DATA)
        if t is not None:
            s, w, tag = t
            n = tag >> 35
            r.data = np.frombuffer(buf, dtype=np.float32, count=n, offset=starts[s] + 8 * w)
    return r
