"""occastft_gb300 — GB300-native batched STFT runner (Python host side).

The Python surface mirrors OCCAstft's runner contract
(StandAlone/cross_gpgpu/GLOBAL/RunnerInterface.hpp:108-131): a ``Runner``
whose ``ActivateSTFT(inData, windowSizeEXP, overlapRatio, options)`` returns
the output vector or ``None`` on error, and the per-stage ``runnerFunction``
hooks (RunnerInterface.hpp:36-104) on device buffers.  Everything calls the
C ABI in ``libocs_gb300.so`` (include/occastft_gb300.h); there is no CPU
fallback: without the native library every call raises.
"""
from __future__ import annotations

import ctypes
import os
from typing import Optional

import numpy as np

__all__ = [
    "Runner",
    "OcsError",
    "lib",
    "geometry",
    "activate",
    "activate_device",
    "runnerFunction",
    "DEFAULT_OPTIONS",
]

_PKG = os.path.dirname(os.path.abspath(__file__))
# OCS_LIBRARY selects another build of the runner (e.g. a tuning variant)
LIB_PATH = os.environ.get("OCS_LIBRARY") or os.path.join(_PKG, "libocs_gb300.so")

# STFTProxy's default option string (StandAlone/include/STFTProxy.hpp:62)
DEFAULT_OPTIONS = "--hanning_window --remove_dc --half_complex_return"

OCS_OK = 0
OCS_EINVAL = 1
OCS_EPIPELINE = 2
OCS_ENOMEM = 3
OCS_ECUDA = 4
OCS_ESPACE = 5
OCS_ETIMEDOUT = 6


class OcsError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"[{code}] {msg}")
        self.code = code
        self.msg = msg


class Geometry(ctypes.Structure):
    _fields_ = [
        ("qt", ctypes.c_uint32),
        ("hop", ctypes.c_uint32),
        ("ofull", ctypes.c_uint32),
        ("ohalf", ctypes.c_uint32),
        ("n_window", ctypes.c_uint32),
        ("reserved", ctypes.c_uint32),
        ("out_floats", ctypes.c_uint64),
        ("frames", ctypes.c_uint64),
    ]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_ if k != "reserved"}


_lib = None

_FP = ctypes.POINTER(ctypes.c_float)
_VP = ctypes.c_void_p

# symbol -> (restype, argtypes); the full C ABI of include/occastft_gb300.h
SIGNATURES = {
    "ocs_init": (ctypes.c_int, [ctypes.c_int]),
    "ocs_shutdown": (None, []),
    "ocs_last_error": (ctypes.c_char_p, []),
    "ocs_version": (ctypes.c_char_p, []),
    "ocs_geometry_get": (ctypes.c_int, [ctypes.c_uint64, ctypes.c_int, ctypes.c_float, ctypes.c_char_p,
                                        ctypes.POINTER(Geometry)]),
    "ocs_activate": (ctypes.c_int, [_VP, ctypes.c_uint64, ctypes.c_int, ctypes.c_float, ctypes.c_char_p, _VP,
                                    ctypes.c_uint64, ctypes.POINTER(ctypes.c_uint64)]),
    "ocs_activate_device": (ctypes.c_int, [_VP, ctypes.c_uint64, ctypes.c_int, ctypes.c_float, ctypes.c_char_p,
                                           _VP, ctypes.c_uint64, _VP]),
    "ocs_window_table": (ctypes.c_int, [ctypes.c_int, ctypes.c_uint32, ctypes.c_float, _VP]),
    "ocs_plan_tune": (ctypes.c_int, [ctypes.c_uint64, ctypes.c_int, ctypes.c_float, ctypes.c_char_p, _VP]),
    "ocs_host_alloc": (ctypes.c_int, [ctypes.POINTER(ctypes.c_void_p), ctypes.c_size_t]),
    "ocs_host_free": (ctypes.c_int, [_VP]),
    "ocs_host_register": (ctypes.c_int, [_VP, ctypes.c_size_t]),
    "ocs_host_unregister": (ctypes.c_int, [_VP]),
    "ocs_batch_prepare": (ctypes.c_int, [_VP, ctypes.c_int]),
    "ocs_batch_device": (ctypes.c_int, [_VP, ctypes.c_int, _VP]),
    "ocs_batch_device_noalloc": (ctypes.c_int, [_VP, ctypes.c_int, _VP]),
    "ocs_server_start": (ctypes.c_int, [_VP]),
    "ocs_server_submit": (ctypes.c_int, [_VP, ctypes.c_uint64, ctypes.c_int, ctypes.c_float, ctypes.c_char_p, _VP,
                                         ctypes.c_uint64, ctypes.POINTER(ctypes.c_uint64)]),
    "ocs_server_wait": (ctypes.c_int, [ctypes.c_uint64, ctypes.c_int, ctypes.POINTER(ctypes.c_int)]),
    "ocs_server_cancel": (ctypes.c_int, [ctypes.c_uint64]),
    "ocs_server_get_stats": (ctypes.c_int, [_VP]),
    "ocs_server_reset_stats": (ctypes.c_int, []),
    "ocs_server_stop": (ctypes.c_int, []),
    "ocs_stage_overlap": (ctypes.c_int, [_VP, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32,
                                         _VP, _VP]),
    "ocs_stage_window": (ctypes.c_int, [ctypes.c_int, _VP, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_float, _VP]),
    "ocs_stage_remove_dc": (ctypes.c_int, [_VP, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32, _VP]),
    "ocs_stage_fft": (ctypes.c_int, [_VP, _VP, ctypes.c_uint32, ctypes.c_uint32, _VP]),
    "ocs_stage_half_complex": (ctypes.c_int, [_VP, _VP, _VP, ctypes.c_uint32, ctypes.c_uint32, _VP]),
    "ocs_stage_to_power": (ctypes.c_int, [_VP, _VP, _VP, ctypes.c_uint32, _VP]),
}


def lib() -> ctypes.CDLL:
    """Load the native runner; raises if it was not built (no fallback)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise OcsError(OCS_ECUDA, f"native library missing: {LIB_PATH} (run occastft_gb300.build.build())")
        L = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name, None)
            if fn is None:
                continue
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def _check(rc: int):
    if rc != OCS_OK:
        raise OcsError(rc, lib().ocs_last_error().decode(errors="replace"))


def last_error() -> str:
    return lib().ocs_last_error().decode(errors="replace")


def geometry(n: int, window_size_exp: int, overlap_ratio: float, options: str = "") -> Geometry:
    g = Geometry()
    _check(lib().ocs_geometry_get(n, window_size_exp, overlap_ratio, options.encode(), ctypes.byref(g)))
    return g


def _stream_handle(stream) -> Optional[int]:
    if stream is None:
        try:
            import torch

            return torch.cuda.current_stream().cuda_stream
        except Exception:  # noqa: BLE001
            return None
    if isinstance(stream, int):
        return stream
    return getattr(stream, "cuda_stream", stream)


def _device_ptr(buf, count: int, what: str) -> int:
    """Device address of a pointer argument.  A torch tensor must be a CUDA,
    contiguous float32 tensor of at least `count` elements (a host tensor or a
    short one would turn into an illegal address on the GPU); a plain integer
    address is the caller's responsibility and passes unchecked."""
    if not hasattr(buf, "data_ptr"):
        return int(buf)
    if not getattr(buf, "is_cuda", False):
        raise OcsError(OCS_EINVAL, f"{what}: the tensor is not on a CUDA device")
    if str(buf.dtype) != "torch.float32":
        raise OcsError(OCS_EINVAL, f"{what}: tensor of {buf.dtype}, float32 expected")
    if not buf.is_contiguous():
        raise OcsError(OCS_EINVAL, f"{what}: the tensor is not contiguous")
    if buf.numel() < count:
        raise OcsError(OCS_EINVAL, f"{what}: the tensor holds {buf.numel()} floats, {count} needed")
    return buf.data_ptr()


def activate(signal: np.ndarray, window_size_exp: int, overlap_ratio: float, options: str = DEFAULT_OPTIONS,
             out: Optional[np.ndarray] = None) -> np.ndarray:
    """Host buffers in and out (ActivateSTFT semantics); raises OcsError on failure."""
    x = np.ascontiguousarray(signal, dtype=np.float32)
    g = geometry(x.size, window_size_exp, overlap_ratio, options)
    if out is None:
        out = np.empty(g.out_floats, dtype=np.float32)
    elif not (isinstance(out, np.ndarray) and out.dtype == np.float32 and out.flags.c_contiguous
              and out.flags.writeable):
        # the native call writes out.size float32 values at out's address
        raise OcsError(OCS_EINVAL, "out must be a writable C-contiguous float32 numpy array")
    n_out = ctypes.c_uint64(0)
    _check(lib().ocs_activate(x.ctypes.data, x.size, window_size_exp, overlap_ratio, options.encode(),
                              out.ctypes.data, out.size, ctypes.byref(n_out)))
    return out[: n_out.value]


def activate_device(d_in, n: int, window_size_exp: int, overlap_ratio: float, options: str, d_out,
                    out_cap: int, stream=None) -> None:
    """Device-resident pipeline (pointers as ints or torch tensors), asynchronous on `stream`."""
    pin = _device_ptr(d_in, n, "input")
    pout = _device_ptr(d_out, out_cap, "output")
    _check(lib().ocs_activate_device(pin, n, window_size_exp, overlap_ratio, options.encode(), pout, out_cap,
                                     _stream_handle(stream)))


def plan_tune(n: int, window_size_exp: int, overlap_ratio: float, options: str) -> int:
    """Tune the kernel choice for requests of this shape ahead of the first one;
    returns the chosen variant (-1 where the shape has a single form)."""
    v = ctypes.c_int(-1)
    _check(lib().ocs_plan_tune(n, window_size_exp, overlap_ratio, options.encode(), ctypes.byref(v)))
    return v.value


def window_table(kind: int, window_size: int, sigma: float = -1.0) -> np.ndarray:
    """Window coefficients the runner applies (host computation)."""
    out = np.empty(window_size, dtype=np.float32)
    _check(lib().ocs_window_table(kind, window_size, sigma, out.ctypes.data))
    return out


class Request(ctypes.Structure):
    """ocs_request: one request of a batch (device pointers)."""

    _fields_ = [
        ("in_", ctypes.c_void_p),
        ("n", ctypes.c_uint64),
        ("window_size_exp", ctypes.c_int),
        ("overlap_ratio", ctypes.c_float),
        ("options", ctypes.c_char_p),
        ("out", ctypes.c_void_p),
        ("out_cap", ctypes.c_uint64),
        ("status", ctypes.c_int),
        ("reserved", ctypes.c_int),
    ]


def make_requests(items):
    """items: iterable of (d_in, n, exp, overlap, options, d_out, out_cap); pointers as ints or tensors."""
    items = list(items)
    arr = (Request * len(items))()
    keep = []
    for i, (din, n, exp, ov, opts, dout, cap) in enumerate(items):
        ob = opts.encode()
        keep.append(ob)
        arr[i].in_ = _device_ptr(din, n, f"request {i} input")
        arr[i].n = n
        arr[i].window_size_exp = exp
        arr[i].overlap_ratio = ov
        arr[i].options = ob
        arr[i].out = _device_ptr(dout, cap, f"request {i} output")
        arr[i].out_cap = cap
        arr[i].status = -1
    arr._keep = keep  # the option strings must outlive the array
    return arr


def batch_prepare(reqs) -> None:
    _check(lib().ocs_batch_prepare(ctypes.cast(reqs, ctypes.c_void_p), len(reqs)))


def batch_device(reqs, stream=None) -> list:
    """One persistent launch over all requests; returns the per-request status codes."""
    _check(lib().ocs_batch_device(ctypes.cast(reqs, ctypes.c_void_p), len(reqs), _stream_handle(stream)))
    return [r.status for r in reqs]


class ServerConfig(ctypes.Structure):
    _fields_ = [("pool_bytes", ctypes.c_uint64), ("max_batch", ctypes.c_int), ("slots", ctypes.c_int)]


class ServerStats(ctypes.Structure):
    _fields_ = [(k, ctypes.c_uint64) for k in ("completed", "failed", "rejected", "pending", "batches", "samples")] + \
               [(k, ctypes.c_double) for k in ("elapsed_ms", "p50_ms", "p99_ms", "p999_ms", "max_ms")] + \
               [("pool_bytes", ctypes.c_uint64), ("pool_used", ctypes.c_uint64)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class Server:
    """Continuous-batching request server (host buffers in and out)."""

    def __init__(self, pool_bytes: int = 0, max_batch: int = 0, slots: int = 0):
        cfg = ServerConfig(pool_bytes, max_batch, slots)
        _check(lib().ocs_server_start(ctypes.byref(cfg)))
        self._keep = {}

    def submit(self, x: np.ndarray, window_size_exp: int, overlap_ratio: float, options: str,
               out: np.ndarray) -> int:
        t = ctypes.c_uint64()
        ob = options.encode()
        _check(lib().ocs_server_submit(x.ctypes.data, x.size, window_size_exp, overlap_ratio, ob,
                                       out.ctypes.data, out.size, ctypes.byref(t)))
        self._keep[t.value] = (x, out, ob)
        return t.value

    def submit_ptr(self, in_ptr: int, n: int, window_size_exp: int, overlap_ratio: float, options: bytes,
                   out_ptr: int, out_cap: int) -> int:
        t = ctypes.c_uint64()
        _check(lib().ocs_server_submit(in_ptr, n, window_size_exp, overlap_ratio, options, out_ptr, out_cap,
                                       ctypes.byref(t)))
        return t.value

    def wait(self, ticket: int, timeout_ms: int = -1) -> int:
        st = ctypes.c_int(-1)
        _check(lib().ocs_server_wait(ticket, timeout_ms, ctypes.byref(st)))
        self._keep.pop(ticket, None)
        return st.value

    def cancel(self, ticket: int) -> None:
        _check(lib().ocs_server_cancel(ticket))
        self._keep.pop(ticket, None)

    def stats(self) -> dict:
        s = ServerStats()
        _check(lib().ocs_server_get_stats(ctypes.byref(s)))
        return s.as_dict()

    def reset_stats(self) -> None:
        _check(lib().ocs_server_reset_stats())

    def stop(self) -> None:
        _check(lib().ocs_server_stop())


class Runner:
    """The reference's Runner (RunnerInterface.hpp:108-131) minus its server loop.

    InitEnv/BuildKernel happen in the constructor (CudaImpl.cpp:285-407);
    ActivateSTFT returns the output vector or None when the pipeline fails,
    exactly like the CUDA runner (CudaImpl.cpp:497-509).
    """

    def __init__(self, device: int = 0):
        self.device = device
        _check(lib().ocs_init(device))
        self.last_status = "OK"

    def ActivateSTFT(self, inData, windowSizeEXP: int, overlapRatio: float,
                     options: str = DEFAULT_OPTIONS) -> Optional[np.ndarray]:  # noqa: N802 (reference name)
        try:
            out = activate(np.asarray(inData, dtype=np.float32), windowSizeEXP, overlapRatio, options)
        except OcsError as e:
            self.last_status = e.msg
            return None
        self.last_status = "OK"
        return out

    def UnInit(self) -> None:  # noqa: N802
        lib().ocs_shutdown()


class runnerFunction:  # noqa: N801 (reference namespace name)
    """Per-stage hooks on device buffers (pointers or torch tensors)."""

    WINDOW_KINDS = {"Hanning": 1, "Hamming": 2, "Blackman": 3, "Nuttall": 4, "Blackman_Nuttall": 5,
                    "Blackman_Harris": 6, "FlatTop": 7, "Gaussian": 8}

    @staticmethod
    def _p(t):
        # tensors: CUDA, float32, contiguous (sizes are the stage's own arguments)
        return _device_ptr(t, 0, "stage buffer")

    @classmethod
    def Overlap(cls, origin, OFullSize, FullSize, windowSizeEXP, OMove, Realout, stream=None):  # noqa: N802,N803
        _check(lib().ocs_stage_overlap(cls._p(origin), OFullSize, FullSize, windowSizeEXP, OMove, cls._p(Realout),
                                       _stream_handle(stream)))
        return True

    @classmethod
    def Window(cls, kind: str, data, OFullSize, windowSize, sigma: float = -1.0, stream=None):  # noqa: N802,N803
        _check(lib().ocs_stage_window(cls.WINDOW_KINDS[kind], cls._p(data), OFullSize, windowSize, sigma,
                                      _stream_handle(stream)))
        return True

    @classmethod
    def RemoveDC(cls, data, qtConst, OFullSize, windowSize, stream=None):  # noqa: N802,N803
        _check(lib().ocs_stage_remove_dc(cls._p(data), qtConst, OFullSize, windowSize, _stream_handle(stream)))
        return True

    @classmethod
    def EXP(cls, Real, Imag, OHalfSize, windowSizeEXP, stream=None):  # noqa: N802,N803
        """EXP6..EXP11 and EXPC: full N-bin spectra written into Real/Imag."""
        _check(lib().ocs_stage_fft(cls._p(Real), cls._p(Imag), OHalfSize, windowSizeEXP, _stream_handle(stream)))
        return True

    @classmethod
    def HalfComplex(cls, out, realResult, imagResult, OHalfSize, windowSizeEXP, stream=None):  # noqa: N802,N803
        _check(lib().ocs_stage_half_complex(cls._p(out), cls._p(realResult), cls._p(imagResult), OHalfSize,
                                            windowSizeEXP, _stream_handle(stream)))
        return True

    @classmethod
    def ToPower(cls, out, realResult, imagResult, OFullSize, stream=None):  # noqa: N802,N803
        _check(lib().ocs_stage_to_power(cls._p(out), cls._p(realResult), cls._p(imagResult), OFullSize,
                                        _stream_handle(stream)))
        return True
