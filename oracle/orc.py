"""TEST INFRASTRUCTURE ONLY: ctypes access to the CPU oracle (liborc.so) and,
where it was built, to the reference's own CPU code (oracle/_ref/).

Imported by tests/, __graft_entry__.smoke() and bench.py's CPU legs — the
checker and the timed CPU baseline.  The product package never imports it.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from typing import Optional

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liborc.so")
REF_DIR = os.path.join(HERE, "_ref")

WINDOWS = {
    "none": 0,
    "hanning": 1,
    "hamming": 2,
    "blackman": 3,
    "nuttall": 4,
    "blackman_nuttall": 5,
    "blackman_harris": 6,
    "flattop": 7,
    "gaussian": 8,
}


class Geometry(ctypes.Structure):
    _fields_ = [
        ("qt", ctypes.c_uint32),
        ("hop", ctypes.c_uint32),
        ("ofull", ctypes.c_uint32),
        ("ohalf", ctypes.c_uint32),
        ("n_window", ctypes.c_uint32),
    ]


class Options(ctypes.Structure):
    _fields_ = [
        ("window", ctypes.c_int),
        ("sigma", ctypes.c_float),
        ("remove_dc", ctypes.c_int),
        ("half_complex", ctypes.c_int),
        ("dense", ctypes.c_int),
        ("serial_power", ctypes.c_int),
    ]


_lib = None


def build() -> None:
    """Compile liborc.so in place (gcc)."""
    subprocess.check_call(["make", "-s", "-C", HERE, "liborc.so"])


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < os.path.getmtime(
            os.path.join(HERE, "stft_oracle.c")
        ):
            build()
        L = ctypes.CDLL(LIB_PATH)
        fp = ctypes.POINTER(ctypes.c_float)
        dp = ctypes.POINTER(ctypes.c_double)
        L.orc_geometry_get.argtypes = [ctypes.c_uint32, ctypes.c_int, ctypes.c_float, ctypes.POINTER(Geometry)]
        L.orc_parse_options.argtypes = [ctypes.c_char_p, ctypes.POINTER(Options), ctypes.c_char_p, ctypes.c_size_t]
        L.orc_window_value.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_float]
        L.orc_window_value.restype = ctypes.c_float
        L.orc_serial_pipeline.argtypes = [fp, ctypes.c_uint32, ctypes.c_int, ctypes.c_float, ctypes.c_char_p,
                                          fp, ctypes.c_int, ctypes.c_int]
        L.orc_output_floats.argtypes = [ctypes.POINTER(Geometry), ctypes.POINTER(Options)]
        L.orc_output_floats.restype = ctypes.c_uint64
        L.orc_fp64_stft.argtypes = [fp, ctypes.c_uint32, ctypes.c_int, ctypes.c_float, ctypes.c_char_p,
                                    dp, ctypes.c_uint64, ctypes.c_int]
        L.orc_overlap.argtypes = [fp, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32, fp]
        L.orc_apply_window.argtypes = [ctypes.c_int, fp, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_float,
                                       ctypes.c_int]
        L.orc_remove_dc.argtypes = [fp, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_int]
        L.orc_set_reference_cost.argtypes = [ctypes.c_int]
        _lib = L
    return _lib


def _fptr(a: np.ndarray):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_float))


def geometry(n: int, exp: int, overlap: float) -> Optional[Geometry]:
    g = Geometry()
    if lib().orc_geometry_get(n, exp, overlap, ctypes.byref(g)) != 0:
        return None
    return g


def parse_options(options: str):
    o = Options()
    err = ctypes.create_string_buffer(64)
    rc = lib().orc_parse_options(options.encode(), ctypes.byref(o), err, 64)
    return rc, o, err.value.decode()


def output_floats(n: int, exp: int, overlap: float, options: str) -> int:
    g = geometry(n, exp, overlap)
    rc, o, _ = parse_options(options)
    return int(lib().orc_output_floats(ctypes.byref(g), ctypes.byref(o)))


def window(kind: str, nwin: int, sigma: float = -1.0) -> np.ndarray:
    k = WINDOWS[kind]
    return np.array([lib().orc_window_value(k, i, nwin, sigma) for i in range(nwin)], dtype=np.float32)


def serial_pipeline(x: np.ndarray, exp: int, overlap: float, options: str, fix_p4: bool = False,
                    nthreads: int = 1) -> np.ndarray:
    """float32 restatement of the reference Serial/OpenMP runner output (OFullSize floats)."""
    x = np.ascontiguousarray(x, dtype=np.float32)
    g = geometry(x.size, exp, overlap)
    if g is None:
        raise ValueError("unsupported geometry")
    out = np.zeros(g.ofull, dtype=np.float32)
    rc = lib().orc_serial_pipeline(_fptr(x), x.size, exp, overlap, options.encode(), _fptr(out),
                                   1 if fix_p4 else 0, nthreads)
    if rc != 0:
        raise ValueError(f"oracle pipeline failed rc={rc}")
    return out


def set_reference_cost(on: bool) -> None:
    """Time the port at the reference's cost: window coefficients evaluated per
    sample and twiddles per butterfly (the outputs do not change)."""
    lib().orc_set_reference_cost(1 if on else 0)


def fp64_stft(x: np.ndarray, exp: int, overlap: float, options: str, nthreads: int = 0) -> np.ndarray:
    """Double-precision STFT with the reference framing/windows, in the layout the options select."""
    x = np.ascontiguousarray(x, dtype=np.float32)
    if nthreads <= 0:
        nthreads = os.cpu_count() or 1
    nout = output_floats(x.size, exp, overlap, options)
    out = np.zeros(nout, dtype=np.float64)
    rc = lib().orc_fp64_stft(_fptr(x), x.size, exp, overlap, options.encode(),
                             out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), nout, nthreads)
    if rc != 0:
        raise ValueError(f"fp64 oracle failed rc={rc}")
    return out


def overlap_window(x: np.ndarray, exp: int, overlap: float, kind: str, sigma: float = -1.0,
                   remove_dc: bool = False) -> np.ndarray:
    x = np.ascontiguousarray(x, dtype=np.float32)
    g = geometry(x.size, exp, overlap)
    out = np.zeros(g.ofull, dtype=np.float32)
    L = lib()
    L.orc_overlap(_fptr(x), g.ofull, x.size, exp, g.hop, _fptr(out))
    L.orc_apply_window(WINDOWS[kind], _fptr(out), g.ofull, g.n_window, sigma, 1)
    if remove_dc:
        L.orc_remove_dc(_fptr(out), g.ofull, g.n_window, 1)
    return out


# ---------------------------------------------------------------- reference
class RefLib:
    """The reference's own Serial/OpenMP code, compiled by oracle/build_ref.sh."""

    def __init__(self, name: str = "libref_serial.so"):
        path = os.path.join(REF_DIR, name)
        self.L = ctypes.CDLL(path)
        fp = ctypes.POINTER(ctypes.c_float)
        u = ctypes.POINTER(ctypes.c_uint)
        self.L.ref_geometry.argtypes = [ctypes.c_uint, ctypes.c_int, ctypes.c_float, u, u, u, u]
        self.L.ref_activate.argtypes = [fp, ctypes.c_uint, ctypes.c_int, ctypes.c_float, ctypes.c_char_p, fp,
                                        ctypes.c_char_p, ctypes.c_int]
        self.L.ref_activate.restype = ctypes.c_longlong
        self.L.ref_overlap_window.argtypes = [fp, ctypes.c_uint, ctypes.c_int, ctypes.c_float, ctypes.c_int,
                                              ctypes.c_float, ctypes.c_int, fp]

    @staticmethod
    def available(name: str = "libref_serial.so") -> bool:
        return os.path.exists(os.path.join(REF_DIR, name))

    def geometry(self, n, exp, ov):
        v = [ctypes.c_uint() for _ in range(4)]
        self.L.ref_geometry(n, exp, ov, *[ctypes.byref(a) for a in v])
        return tuple(a.value for a in v)  # qt, hop, ofull, ohalf

    def activate(self, x: np.ndarray, exp: int, ov: float, options: str):
        x = np.ascontiguousarray(x, dtype=np.float32)
        qt, hop, ofull, ohalf = self.geometry(x.size, exp, ov)
        out = np.zeros(ofull, dtype=np.float32)
        st = ctypes.create_string_buffer(128)
        r = self.L.ref_activate(_fptr(x), x.size, exp, ov, options.encode(), _fptr(out), st, 128)
        return (out if r >= 0 else None), st.value.decode()

    def overlap_window(self, x, exp, ov, kind: str, sigma=-1.0, remove_dc=False):
        x = np.ascontiguousarray(x, dtype=np.float32)
        qt, hop, ofull, ohalf = self.geometry(x.size, exp, ov)
        out = np.zeros(ofull, dtype=np.float32)
        self.L.ref_overlap_window(_fptr(x), x.size, exp, ov, WINDOWS[kind], sigma, int(remove_dc), _fptr(out))
        return out


def rel_l2(a: np.ndarray, b: np.ndarray) -> float:
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    den = np.linalg.norm(b)
    if den == 0:
        return float(np.linalg.norm(a))
    return float(np.linalg.norm(a - b) / den)


def max_db_error(a: np.ndarray, b: np.ndarray, floor_rel: float = 1e-6) -> float:
    """Max per-bin |20 log10 |a| - 20 log10 |b||, magnitudes floored at floor_rel * max|b|."""
    a = np.abs(np.asarray(a, dtype=np.float64))
    b = np.abs(np.asarray(b, dtype=np.float64))
    fl = max(float(b.max()) * floor_rel, 1e-300)
    return float(np.max(np.abs(20 * np.log10(np.maximum(a, fl)) - 20 * np.log10(np.maximum(b, fl)))))
