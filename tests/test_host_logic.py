"""Host-side logic of the native runner, on CPU: the C-ABI library loads and
exports every function include/*.h declares; geometry, option parsing and
window tables agree with the oracle / the reference's golden vectors.  No
compute call is made (no GPU here)."""
import ctypes
import os
import re

import numpy as np
import pytest

from tests.conftest import ROOT, signal


def _declared(header):
    txt = open(os.path.join(ROOT, "include", header)).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(ocs_[a-z0-9_]+)\s*\(", txt)))


def test_library_exports_every_declared_symbol(ocs_lib):
    names = _declared("occastft_gb300.h")
    assert len(names) >= 15
    L = ctypes.CDLL(ocs_lib.LIB_PATH)
    for n in names:
        assert hasattr(L, n), n
        assert n in ocs_lib.SIGNATURES, n


def test_version(ocs_lib):
    assert b"sm_103a" in ocs_lib.lib().ocs_version()


@pytest.mark.parametrize("n,exp,ov", [(1 << 20, 10, 0.5), (100000000, 6, 0.5), (100000000, 15, 0.5),
                                      (100000000, 12, 0.75), (12345, 7, 0.0), (3001, 8, 0.5 + 1 / 256),
                                      (2000, 7, -0.5), (1, 6, 0.5), (16777217, 9, 0.3)])
def test_geometry_matches_oracle(ocs_lib, orc, n, exp, ov):
    g = ocs_lib.geometry(n, exp, ov, "--hanning_window")
    o = orc.geometry(n, exp, ov)
    assert (g.qt, g.hop, g.ofull, g.ohalf, g.n_window) == (o.qt, o.hop, o.ofull, o.ohalf, o.n_window)
    assert g.out_floats == o.ofull and g.frames == o.qt


def test_geometry_layouts(ocs_lib):
    g = ocs_lib.geometry(1 << 20, 10, 0.5, "--half_complex_return")
    assert g.out_floats == g.ofull and g.frames == (g.ohalf + 1023) // 1024
    g = ocs_lib.geometry(1 << 20, 10, 0.5, "--layout=dense")
    assert g.out_floats == g.qt * 513
    g = ocs_lib.geometry(1 << 20, 10, 0.5, "--layout=dense --half_complex_return")
    assert g.out_floats == g.qt * 513 * 2


def test_c0_frame_count(ocs_lib):
    # 2^20 samples, N=1024, overlap 0.5: toQuot gives 2049 zero-padded frames
    g = ocs_lib.geometry(1 << 20, 10, 0.5)
    assert (g.qt, g.hop, g.ofull) == (2049, 512, 2049 * 1024)


@pytest.mark.parametrize("opts,status", [
    ("--gaussian_window=4<<sigma", "--gaussian_window"),
    ("--gaussian_window=4abc<<sigma", "--gaussian_window"),
    ("--gaussian_window=41e-50<<sigma", "--gaussian_window"),
])
def test_option_errors(ocs_lib, orc, opts, status):
    with pytest.raises(ocs_lib.OcsError) as ei:
        ocs_lib.geometry(5000, 8, 0.5, opts)
    assert ei.value.msg == status
    rc, _, err = orc.parse_options(opts)
    assert rc != 0 and err == status


def test_exp_below_six_not_supported(ocs_lib):
    with pytest.raises(ocs_lib.OcsError) as ei:
        ocs_lib.geometry(5000, 5, 0.5)
    assert ei.value.msg == "Operation not supported"
    assert ocs_lib.Runner.__init__ is not None


def test_bad_overlap_rejected(ocs_lib):
    for ov in (1.0, 1.5, float("nan")):
        with pytest.raises(ocs_lib.OcsError):
            ocs_lib.geometry(5000, 8, ov)


@pytest.mark.parametrize("kind", list(range(1, 9)))
@pytest.mark.parametrize("exp", [6, 9, 10, 12, 15])
def test_window_table_matches_oracle(ocs_lib, orc, kind, exp):
    N = 1 << exp
    sigma = 0.312345 if kind == 8 else -1.0
    mine = ocs_lib.window_table(kind, N, sigma)
    names = {v: k for k, v in orc.WINDOWS.items()}
    ref = orc.window(names[kind], N, sigma)
    assert np.array_equal(mine.view(np.uint32), ref.view(np.uint32))


def test_window_table_matches_reference_golden(ocs_lib, golden):
    """Frame 0 of the reference's overlap+window stage equals x[0:N] * w."""
    manifest, arrays = golden
    kinds = {"hanning": 1, "hamming": 2, "blackman": 3, "nuttall": 4, "blackman_nuttall": 5,
             "blackman_harris": 6, "flattop": 7, "gaussian": 8}
    for w in manifest["windows"]:
        N = 1 << w["exp"]
        x = signal(w["seed"], w["n"])[:N]
        tab = ocs_lib.window_table(kinds[w["kind"]], N, w["sigma"])
        got = (x * tab).astype(np.float32)
        assert np.array_equal(got.view(np.uint32), arrays[w["key"]].view(np.uint32)), w["key"]


def test_gaussian_sigma_quirk(ocs_lib, orc):
    # "--gaussian_window=4.312345<<sigma": the first sigma character is skipped
    rc, o, _ = orc.parse_options("--gaussian_window=4.312345<<sigma")
    assert rc == 0 and abs(o.sigma - 0.312345) < 1e-7


def test_window_exponent_limits(ocs_lib):
    """Every window the reference's EXPC takes is accepted: exponents up to
    30, as long as OFullSize = qt * N stays below 2^32 (RunnerCommon.cpp:290-306);
    2^31 overflows the reference's int window size and is refused."""
    g = ocs_lib.geometry(50_000_000, 22, 0.5, "--hanning_window")
    assert g.n_window == 1 << 22 and g.out_floats == g.qt * (1 << 22)
    g = ocs_lib.geometry(50_000_000, 23, 0.5, "")
    assert g.n_window == 1 << 23 and g.qt == 50_000_000 // (1 << 22) + 1
    g = ocs_lib.geometry(1 << 31, 30, 0.0, "--blackman_window")
    assert g.qt == 3 and g.ofull == 3 << 30
    with pytest.raises(ocs_lib.OcsError, match="OFullSize"):
        ocs_lib.geometry(1 << 31, 30, 0.5, "")
    with pytest.raises(ocs_lib.OcsError, match="above 2\\^30"):
        ocs_lib.geometry(50_000_000, 31, 0.5, "")


def test_python_pointer_arguments_are_checked(ocs_lib):
    """Tensors handed to the device-pointer calls are checked on the host
    before any native call: a host tensor, another dtype, a strided view or a
    buffer shorter than the stated size would otherwise become an illegal
    address (or a wrong reading) on the GPU.  Raw integer addresses pass."""
    import torch

    cases = [(torch.zeros(64), "not on a CUDA device")]
    for t, why in cases:
        with pytest.raises(ocs_lib.OcsError, match=why):
            ocs_lib.activate_device(t, 64, 6, 0.5, "", 0, 64)
        with pytest.raises(ocs_lib.OcsError, match=why):
            ocs_lib.make_requests([(t, 64, 6, 0.5, "", 0, 64)])
        with pytest.raises(ocs_lib.OcsError, match=why):
            ocs_lib.runnerFunction.ToPower(t, 0, 0, 64)

    class Fake:  # stands in for a CUDA tensor on a machine without one
        def __init__(self, dtype="torch.float32", contiguous=True, numel=64):
            self.is_cuda, self.dtype, self._c, self._n = True, dtype, contiguous, numel

        def data_ptr(self):
            return 0x10000

        def is_contiguous(self):
            return self._c

        def numel(self):
            return self._n

    assert ocs_lib._device_ptr(Fake(), 64, "x") == 0x10000
    assert ocs_lib._device_ptr(0x2000, 1 << 40, "x") == 0x2000
    for fake, why in [(Fake(dtype="torch.float64"), "float32 expected"), (Fake(contiguous=False), "not contiguous"),
                      (Fake(numel=63), "63 floats, 64 needed")]:
        with pytest.raises(ocs_lib.OcsError, match=why):
            ocs_lib._device_ptr(fake, 64, "x")
        with pytest.raises(ocs_lib.OcsError, match=why):
            ocs_lib.make_requests([(fake, 64, 6, 0.5, "", 0x3000, 64)])


def test_activate_out_argument_is_checked(ocs_lib):
    """ocs_activate writes out.size float32 values at out's address: an out
    array of another dtype, read-only or strided is refused first."""
    x = signal(3, 1000)
    for out in (np.zeros(10000, np.int8), np.zeros(10000, np.float64), np.zeros(20000, np.float32)[::2]):
        with pytest.raises(ocs_lib.OcsError, match="float32 numpy array"):
            ocs_lib.activate(x, 6, 0.5, "", out=out)
    ro = np.zeros(10000, np.float32)
    ro.flags.writeable = False
    with pytest.raises(ocs_lib.OcsError, match="float32 numpy array"):
        ocs_lib.activate(x, 6, 0.5, "", out=ro)


def test_validation_before_any_device_call(ocs_lib):
    """Arguments the C ABI refuses before it touches a device, with the
    reference's status strings where it has one: these run on a machine
    without a GPU.  Addresses are plain integers that are never dereferenced."""
    L = ocs_lib.lib()
    P = 0x10000

    def err(rc, code, text):
        assert rc == code, (rc, ocs_lib.last_error())
        assert text in ocs_lib.last_error(), ocs_lib.last_error()

    # per-stage hooks (runnerFunction::*)
    err(L.ocs_stage_fft(P, P, 1024, 5, None), ocs_lib.OCS_EINVAL, "Operation not supported")
    err(L.ocs_stage_fft(P, P, 1024, 31, None), ocs_lib.OCS_EINVAL, "above 2^30")
    err(L.ocs_stage_fft(None, P, 1024, 10, None), ocs_lib.OCS_EINVAL, "null buffer")
    err(L.ocs_stage_window(0, P, 1024, 1024, -1.0, None), ocs_lib.OCS_EINVAL, "window")
    err(L.ocs_stage_window(1, P, 1024, 1000, -1.0, None), ocs_lib.OCS_EINVAL, "window")
    err(L.ocs_stage_window(1, P, 1 << 31, 1 << 31, -1.0, None), ocs_lib.OCS_EINVAL, "above 2^30")
    err(L.ocs_stage_remove_dc(None, 1, 1024, 1024, None), ocs_lib.OCS_EINVAL, "RemoveDC")
    err(L.ocs_stage_overlap(P, 1024, 1000, 5, 512, P, None), ocs_lib.OCS_EINVAL, "Overlap")
    err(L.ocs_stage_half_complex(None, P, P, 512, 10, None), ocs_lib.OCS_EINVAL, "HalfComplex")
    err(L.ocs_stage_to_power(P, None, P, 1024, None), ocs_lib.OCS_EINVAL, "ToPower")
    # whole-pipeline entry points
    g = ocs_lib.geometry(100000, 10, 0.5, "")
    n_out = ctypes.c_uint64()
    err(L.ocs_activate(P, 100000, 10, 0.5, b"", P, g.out_floats - 1, ctypes.byref(n_out)), ocs_lib.OCS_ESPACE,
        "too small")
    err(L.ocs_activate(None, 100000, 10, 0.5, b"", P, g.out_floats, ctypes.byref(n_out)), ocs_lib.OCS_EINVAL, "null")
    err(L.ocs_activate_device(P, 100000, 10, 0.5, b"", None, g.out_floats, None), ocs_lib.OCS_EINVAL, "null")
    err(L.ocs_activate(P, 100000, 7, 0.5, b"--precision=tc-fp16", P, 1 << 30, ctypes.byref(n_out)),
        ocs_lib.OCS_EINVAL, "2^8 .. 2^12")
    # a negative overlap ratio (accepted, as in the reference) advances frames by more than N
    assert ocs_lib.geometry(100000, 8, -0.5, "").hop == 384
    err(L.ocs_activate(P, 100000, 8, -0.5, b"--precision=tc-bf16x2", P, 1 << 30, ctypes.byref(n_out)),
        ocs_lib.OCS_EINVAL, "frame advance")
    err(L.ocs_activate(P, 0, 10, 0.5, b"", P, 1 << 30, ctypes.byref(n_out)), ocs_lib.OCS_EINVAL, "empty")
    err(L.ocs_activate(P, 100000, 10, 0.5, b"--gaussian_window=4<<sigma", P, 1 << 30, ctypes.byref(n_out)),
        ocs_lib.OCS_EPIPELINE, "--gaussian_window")
    # batches and the server
    err(L.ocs_batch_device(None, 3, None), ocs_lib.OCS_EINVAL, "bad request list")
    err(L.ocs_batch_prepare(None, -1), ocs_lib.OCS_EINVAL, "bad request list")
    err(L.ocs_batch_device_noalloc(None, 300, None), ocs_lib.OCS_EINVAL, "bad request list")
    t = ctypes.c_uint64()
    err(L.ocs_server_submit(P, 1000, 10, 0.5, b"", P, 1 << 20, ctypes.byref(t)), ocs_lib.OCS_EINVAL, "not running")
    err(L.ocs_server_wait(1, 0, None), ocs_lib.OCS_EINVAL, "not running")
    err(L.ocs_server_stop(), ocs_lib.OCS_EINVAL, "not running")
