"""The oracle is pinned against golden vectors produced by the reference's
own Serial runner (tests/golden/make_golden.py): bit-exact outputs, geometry
and status strings."""
import hashlib

import numpy as np
import pytest

from tests.conftest import signal


def _cases(golden):
    return golden[0]["cases"]


def test_golden_cases_bit_exact(orc, golden):
    manifest, arrays = golden
    checked = 0
    for c in manifest["cases"]:
        if c["status"] != "OK":
            continue
        x = signal(c["seed"], c["n"])
        out = orc.serial_pipeline(x, c["exp"], c["overlap"], c["options"])
        ref = arrays[c["name"]]
        assert out.size == ref.size == c["ofull"], c["name"]
        assert hashlib.sha256(out.tobytes()).hexdigest() == c["sha256"], c["name"]
        assert np.array_equal(out.view(np.uint32), ref.view(np.uint32)), c["name"]
        checked += 1
    assert checked >= 30


def test_golden_geometry(orc, golden):
    for c in golden[0]["cases"]:
        if "qt" not in c:
            continue
        g = orc.geometry(c["n"], c["exp"], c["overlap"])
        assert (g.qt, g.hop, g.ofull, g.ohalf) == (c["qt"], c["hop"], c["ofull"], c["ohalf"]), c["name"]


def test_golden_statuses(orc, golden):
    for c in golden[0]["cases"]:
        rc, o, err = orc.parse_options(c["options"])
        if c["status"] == "OK":
            assert rc == 0, c["name"]
        elif c["status"].startswith("--"):
            assert rc != 0 and err == c["status"], c["name"]
        else:  # "Operation not supported": exponent below 6
            assert c["exp"] < 6
            assert orc.geometry(c["n"], c["exp"], c["overlap"]) is None


def test_c0_full_size(orc, golden):
    """C0: 2^20 uniform samples, N=1024 Hann, overlap 0.5, DC removal, power."""
    manifest, arrays = golden
    c = manifest["c0"]
    x = signal(c["seed"], c["n"])
    out = orc.serial_pipeline(x, c["exp"], c["overlap"], c["options"], nthreads=4)
    assert c["qt"] == 2049 and out.size == c["ofull"]
    assert hashlib.sha256(out.tobytes()).hexdigest() == c["sha256"]
    N = 1 << c["exp"]
    for i, f in enumerate(c["frames"]):
        assert np.array_equal(out[f * N:(f + 1) * N], arrays["c0_frames"][i])


def test_golden_windows(orc, golden):
    """Window formulas: overlap+window stage output of the reference, bit for bit."""
    manifest, arrays = golden
    for w in manifest["windows"]:
        N = 1 << w["exp"]
        x = signal(w["seed"], w["n"])
        mine = orc.overlap_window(x, w["exp"], 0.5, w["kind"], sigma=w["sigma"])[:N]
        assert np.array_equal(mine.view(np.uint32), arrays[w["key"]].view(np.uint32)), w["key"]


def test_p4_quirk_reproduced_and_fixed(orc, golden):
    """Odd exponents >= 13: the reference returns stage exp-2's buffer (a known
    defect).  The oracle reproduces it with fix_p4=False; the fixed variant
    agrees with the FP64 transform instead."""
    manifest, arrays = golden
    odd = [c for c in manifest["cases"] if c["exp"] in (13, 15) and c["status"] == "OK"]
    assert odd
    for c in odd:
        x = signal(c["seed"], c["n"])
        fixed = orc.serial_pipeline(x, c["exp"], c["overlap"], c["options"], fix_p4=True)
        f64 = orc.fp64_stft(x, c["exp"], c["overlap"], c["options"] + " --serial_power")
        assert orc.rel_l2(fixed, f64) < 1e-5
        assert orc.rel_l2(arrays[c["name"]], f64) > 0.1


def test_reference_cost_model_changes_no_output(orc):
    """The port's two cost models (per-call tables; per-element trig as the
    reference computes it) give the same bits."""
    x = signal(8, 40000)
    for exp, op in ((6, "--hanning_window --remove_dc"), (10, "--hamming_window"),
                    (13, "--nuttall_window --half_complex_return"), (9, "--gaussian_window=x0.4<<sigma")):
        a = orc.serial_pipeline(x, exp, 0.5, op, nthreads=2)
        orc.set_reference_cost(True)
        try:
            b = orc.serial_pipeline(x, exp, 0.5, op, nthreads=2)
        finally:
            orc.set_reference_cost(False)
        assert np.array_equal(a.view(np.uint32), b.view(np.uint32)), (exp, op)
