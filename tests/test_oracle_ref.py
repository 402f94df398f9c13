"""Live pin: the oracle restatement against the reference's own Serial and
OpenMP code compiled from source (oracle/build_ref.sh).  Skipped where the
reference checkout was not available to build oracle/_ref/."""
import numpy as np
import pytest

from tests.conftest import signal

ref_missing = pytest.mark.skipif(
    not __import__("oracle.orc", fromlist=["RefLib"]).RefLib.available(), reason="oracle/_ref not built")


@ref_missing
@pytest.mark.parametrize("exp", list(range(6, 16)))
def test_oracle_matches_reference_serial(orc, exp):
    R = orc.RefLib("libref_serial.so")
    rng = np.random.default_rng(exp)
    opts = ["--hanning_window --remove_dc", "--blackman_window --half_complex_return", "--hamming_window",
            "--flattop_window --remove_dc --half_complex_return", "--gaussian_window=x3.5<<sigma", ""]
    for ov in (0.0, 0.5, 0.75, 0.3):
        for op in opts:
            n = int(rng.integers(1 << exp, (1 << exp) * 6))
            x = signal(int(rng.integers(1 << 30)), n)
            ref, st = R.activate(x, exp, ov, op)
            assert st == "OK"
            mine = orc.serial_pipeline(x, exp, ov, op)
            assert np.array_equal(ref.view(np.uint32), mine.view(np.uint32)), (exp, ov, op)


@ref_missing
def test_openmp_equals_serial(orc):
    S = orc.RefLib("libref_serial.so")
    O = orc.RefLib("libref_openmp.so")
    x = signal(3, 50000)
    for exp in (6, 10, 12, 13):
        a, _ = S.activate(x, exp, 0.5, "--hanning_window --remove_dc")
        b, _ = O.activate(x, exp, 0.5, "--hanning_window --remove_dc")
        assert np.array_equal(a.view(np.uint32), b.view(np.uint32))


@ref_missing
def test_port_at_reference_cost_matches_reference(orc):
    """The cost model the CPU baseline is timed with (window per sample,
    twiddle per butterfly) gives the reference's output bit for bit."""
    O = orc.RefLib("libref_openmp.so")
    x = signal(4, 70000)
    orc.set_reference_cost(True)
    try:
        for exp, op in ((10, "--hamming_window"), (12, "--blackman_window --remove_dc"),
                        (7, "--hanning_window --half_complex_return")):
            ref, _ = O.activate(x, exp, 0.5, op)
            mine = orc.serial_pipeline(x, exp, 0.5, op, nthreads=4)
            assert np.array_equal(ref.view(np.uint32), mine.view(np.uint32)), (exp, op)
    finally:
        orc.set_reference_cost(False)


@ref_missing
def test_reference_serial_twiddle_overflow_from_2pow17(orc):
    """The reference's own Serial runner is not the DFT from window 2^17 on:
    its twiddle index (lsave % segmentSize) * HwindowSize (OKL/kernel.okl:141-144)
    overflows a 32-bit int once segmentSize * N/2 reaches 2^31.  The oracle's
    restatement reproduces the same bits; the FP64 oracle is the accuracy
    reference at those sizes."""
    R = orc.RefLib("libref_serial.so")
    for exp, bad in ((16, False), (18, True)):
        N = 1 << exp
        x = signal(5, 3 * N + 7)
        opts = "--hamming_window --half_complex_return"
        ref, st = R.activate(x, exp, 0.5, opts)
        assert st == "OK"
        mine = orc.serial_pipeline(x, exp, 0.5, opts, nthreads=4)
        assert np.array_equal(ref.view(np.uint32), mine.view(np.uint32))
        err = orc.rel_l2(ref, orc.fp64_stft(x, exp, 0.5, opts))
        assert (err > 0.1) if bad else (err < 1e-6), (exp, err)
