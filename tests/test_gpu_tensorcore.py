"""Tensor-core split-precision form (tcgen05, --precision=tc-fp16): windows
2^8 and 2^10, every output layout, against the FP64 oracle at the suite's
relative-L2 bar (the form trades exact fp32 arithmetic for fp16 hi/lo
products with fp32 accumulation)."""
import numpy as np
import pytest

from tests.conftest import signal

REL_L2 = 1e-5
pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("exp", [8, 10])
@pytest.mark.parametrize("opts", [
    "--hanning_window",
    "--hanning_window --remove_dc --half_complex_return",
    "--blackman_window --layout=dense",
    "--hamming_window --half_complex_return --layout=dense",
    "--flattop_window --serial_power",
])
def test_tc_matches_fp64(ocs_lib, orc, exp, opts):
    N = 1 << exp
    x = signal(77 + exp, 37 * N + 19)
    for ov in (0.75, 0.5):
        o = opts + " --precision=tc-fp16"
        got = ocs_lib.activate(x, exp, ov, o)
        ref = orc.fp64_stft(x, exp, ov, opts)
        assert got.size == ref.size
        err = orc.rel_l2(got, ref)
        assert err <= REL_L2, (exp, ov, opts, err)


def test_tc_scaling_extremes(ocs_lib, orc):
    """Per-frame power-of-two scaling keeps fp16 in range for tiny and huge signals."""
    for amp in (1e-6, 1.0, 3e4):
        x = (signal(5, 50000) * amp).astype(np.float32)
        got = ocs_lib.activate(x, 10, 0.75, "--hanning_window --precision=tc-fp16")
        ref = orc.fp64_stft(x, 10, 0.75, "--hanning_window")
        assert orc.rel_l2(got, ref) <= REL_L2, amp


def test_tc_rejects_unsupported_window(ocs_lib):
    with pytest.raises(ocs_lib.OcsError):
        ocs_lib.activate(signal(1, 10000), 9, 0.5, "--precision=tc-fp16")
