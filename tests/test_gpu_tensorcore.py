"""Tensor-core split-precision form (tcgen05): windows 2^8 .. 2^12 (the
pipelined kernel at 2^8 and 2^10, the generic N = P x Q kernel at 2^9, 2^11
and 2^12), every output layout, against the FP64 oracle.  fp16 hi/lo
(--precision=tc-fp16) and bf16 hi/mid/lo (tc-bf16x3) meet the suite's
relative-L2 bar of 1e-5; bf16 hi/lo (tc-bf16x2, about 16 significant bits per
operand) is reported for reference and held to 1e-4.  bf16 hi/mid/lo at 2^12
runs pass 2 in two halves of K (its whole A2 operand does not fit beside the
DFT matrices)."""
import numpy as np
import pytest

from tests.conftest import signal

REL_L2 = 1e-5
pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("exp", [8, 9, 10, 11, 12])
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


@pytest.mark.parametrize("exp", [10, 11, 12])
def test_tc_scaling_extremes(ocs_lib, orc, exp):
    """Per-frame power-of-two scaling keeps fp16 in range for tiny and huge signals."""
    for amp in (1e-6, 1.0, 3e4):
        x = (signal(5, 50000) * amp).astype(np.float32)
        got = ocs_lib.activate(x, exp, 0.75, "--hanning_window --precision=tc-fp16")
        ref = orc.fp64_stft(x, exp, 0.75, "--hanning_window")
        assert orc.rel_l2(got, ref) <= REL_L2, (exp, amp)


@pytest.mark.parametrize("prec,bar", [("tc-bf16x3", 1e-5), ("tc-bf16x2", 1e-4)])
@pytest.mark.parametrize("exp", [8, 9, 10, 11, 12])
@pytest.mark.parametrize("opts", [
    "--hanning_window --remove_dc",
    "--blackman_window --half_complex_return --layout=dense",
    "--hamming_window --half_complex_return",
])
def test_tc_bf16_modes(ocs_lib, orc, prec, bar, exp, opts):
    """Every size in both bf16 modes; at 2^12 bf16 hi/mid/lo runs pass 2 in
    two halves of K through one A2 buffer (the whole one does not fit)."""
    N = 1 << exp
    x = signal(300 + exp, 900 * N + 77)  # many tiles per CTA
    for ov in (0.75, 0.3):
        got = ocs_lib.activate(x, exp, ov, opts + " --precision=" + prec)
        ref = orc.fp64_stft(x, exp, ov, opts)
        err = orc.rel_l2(got, ref)
        assert err <= bar, (prec, exp, ov, opts, err)


def test_tc_bf16_needs_short_advance(ocs_lib):
    with pytest.raises(ocs_lib.OcsError, match="frame advance"):
        ocs_lib.activate(signal(1, 50000), 10, -0.5, "--precision=tc-bf16x3")


def test_tc_rejects_unsupported_window(ocs_lib):
    for exp in (7, 13):
        with pytest.raises(ocs_lib.OcsError):
            ocs_lib.activate(signal(1, 10000), exp, 0.5, "--precision=tc-fp16")


@pytest.mark.parametrize("exp", [9, 11, 12])
def test_tc_generic_any_advance(ocs_lib, orc, exp):
    """The generic kernel takes frame advances above the window in every mode."""
    x = signal(40 + exp, 200_003)
    for prec, bar in (("tc-fp16", REL_L2), ("tc-bf16x2", 1e-4), ("tc-bf16x3", REL_L2)):
        got = ocs_lib.activate(x, exp, -0.5, "--hanning_window --precision=" + prec)
        ref = orc.fp64_stft(x, exp, -0.5, "--hanning_window")
        assert orc.rel_l2(got, ref) <= bar, (exp, prec)


@pytest.mark.parametrize("exp", [8, 9, 10, 11, 12])
def test_tc_many_tiles_per_cta(ocs_lib, orc, exp):
    """Long signals: every CTA runs many tiles, so each double buffer is
    reused many times (phase parity of every pipeline barrier wraps)."""
    x = signal(900 + exp, 3_000_017)
    for opts in ("--hanning_window --remove_dc", "--blackman_window --half_complex_return --layout=dense"):
        got = ocs_lib.activate(x, exp, 0.75, opts + " --precision=tc-fp16")
        ref = orc.fp64_stft(x, exp, 0.75, opts)
        assert orc.rel_l2(got, ref) <= REL_L2, (exp, opts)


@pytest.mark.parametrize("exp", [10, 11])
@pytest.mark.parametrize("shift", [1, 2, 3, 5])
def test_tc_unaligned_device_input(ocs_lib, orc, exp, shift):
    """Signal pointers that are not 16-byte aligned (offset by whole floats)."""
    import torch
    ov, opts = 0.75, "--hamming_window --remove_dc --layout=dense"
    x = signal(31 + shift, 200_003)
    g = ocs_lib.geometry(x.size, exp, ov, opts)
    buf = torch.zeros(x.size + 8, dtype=torch.float32, device="cuda")
    buf[shift:shift + x.size] = torch.from_numpy(x).cuda()
    d_out = torch.empty(g.out_floats, dtype=torch.float32, device="cuda")
    ocs_lib.activate_device(buf[shift:].data_ptr(), x.size, exp, ov, opts + " --precision=tc-fp16", d_out,
                            g.out_floats)
    torch.cuda.synchronize()
    ref = orc.fp64_stft(x, exp, ov, opts)
    assert orc.rel_l2(d_out.cpu().numpy(), ref) <= REL_L2


def test_tc_hop_longer_than_window(ocs_lib, orc):
    """Negative overlap (frame advance above the window) takes the
    non-pipelined tensor-core kernel."""
    x = signal(8, 100_000)
    for exp in (8, 9, 10, 11, 12):
        got = ocs_lib.activate(x, exp, -0.5, "--hanning_window --precision=tc-fp16")
        ref = orc.fp64_stft(x, exp, -0.5, "--hanning_window")
        assert orc.rel_l2(got, ref) <= REL_L2, exp


STALL_CHILD = r'''
import sys
import numpy as np
sys.path.insert(0, {root!r})
import occastft_gb300 as ocs
from oracle import orc
x = np.random.default_rng(3).uniform(-1, 1, 400_000).astype(np.float32)
try:
    ocs.activate(x, 10, 0.75, "--hanning_window --precision=tc-fp16")
    print("NO-ERROR")
except ocs.OcsError as e:
    print("CODE", e.code)
got = ocs.activate(x, 10, 0.75, "--hanning_window")
print("AFTER", orc.rel_l2(got, orc.fp64_stft(x, 10, 0.75, "--hanning_window")))
'''


def test_tc_wait_timeout_reports_error():
    """Every pipeline wait of the tensor-core kernel is bounded: with the test
    hook the first input phase never completes, the waits give up after about
    a second, the call returns OCS_ETIMEDOUT and the context stays usable."""
    import os
    import subprocess
    import sys
    from tests.conftest import ROOT
    e = dict(os.environ)
    e["OCS_TC_TEST_STALL"] = "1"
    out = subprocess.run([sys.executable, "-c", STALL_CHILD.format(root=ROOT)], env=e, capture_output=True,
                         text=True, timeout=300)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = out.stdout.strip().splitlines()
    assert "CODE 6" in lines, lines
    after = float([ln for ln in lines if ln.startswith("AFTER")][0].split()[1])
    assert after <= REL_L2


@pytest.mark.parametrize("exp,ov", [(8, 0.3), (10, 0.33), (10, 0.1), (8, 0.0), (9, 0.3), (11, 0.1), (12, 0.33)])
def test_tc_odd_hop(ocs_lib, orc, exp, ov):
    """Frame advances that are not a multiple of four samples: frames start
    at every offset inside a 16-byte word of the staged input."""
    x = signal(400 + exp, 123_457)
    for opts in ("--hanning_window --remove_dc", "--blackman_window --half_complex_return"):
        got = ocs_lib.activate(x, exp, ov, opts + " --precision=tc-fp16")
        ref = orc.fp64_stft(x, exp, ov, opts)
        assert orc.rel_l2(got, ref) <= REL_L2, (exp, ov, opts)
