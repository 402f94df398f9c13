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
    """Windows up to 2^22 are accepted (the reference's EXPC has no upper
    bound short of OFullSize < 2^32); 2^23 is refused with a status."""
    g = ocs_lib.geometry(50_000_000, 22, 0.5, "--hanning_window")
    assert g.n_window == 1 << 22 and g.out_floats == g.qt * (1 << 22)
    with pytest.raises(ocs_lib.OcsError, match="above 2\\^22"):
        ocs_lib.geometry(50_000_000, 23, 0.5, "")
