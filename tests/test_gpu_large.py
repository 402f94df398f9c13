"""Windows 2^16 .. 2^22 (the reference's EXPC range above the fused
kernels): the two-launch four-step FFT against the FP64 oracle, every output
layout, through the host entry (chunked copies, several frame ranges) and
the device entry; plus the reference Serial pipeline itself at an even
exponent, where its result is the full transform."""
import numpy as np
import pytest

from tests.conftest import signal

pytestmark = pytest.mark.gpu
REL_L2 = 1e-5

OPTS = ["--hamming_window", "--blackman_window --half_complex_return", "--hanning_window --layout=dense --remove_dc",
        "--nuttall_window --half_complex_return --layout=dense", "--flattop_window --serial_power",
        "--gaussian_window=x0.4<<sigma --remove_dc"]


@pytest.mark.parametrize("exp", [16, 17, 18, 19, 20, 21, 22])
def test_large_windows_match_fp64(ocs_lib, orc, exp):
    N = 1 << exp
    x = signal(700 + exp, 5 * N + 12345)
    for i, opts in enumerate(OPTS):
        ov = (0.5, 0.75, 0.3)[i % 3]
        got = ocs_lib.activate(x, exp, ov, opts)
        ref = orc.fp64_stft(x, exp, ov, opts)
        assert got.size == ref.size, (exp, opts)
        err = orc.rel_l2(got, ref)
        assert err <= REL_L2, (exp, ov, opts, err)


@pytest.mark.parametrize("exp", [16, 20])
def test_large_device_entry(ocs_lib, orc, exp):
    import torch

    N = 1 << exp
    x = signal(800 + exp, 9 * N + 7)
    opts = "--hanning_window --remove_dc"
    g = ocs_lib.geometry(x.size, exp, 0.5, opts)
    d_out = torch.empty(g.out_floats, device="cuda")
    ocs_lib.activate_device(torch.from_numpy(x).cuda(), x.size, exp, 0.5, opts, d_out, g.out_floats)
    torch.cuda.synchronize()
    got = d_out.cpu().numpy()
    assert orc.rel_l2(got, orc.fp64_stft(x, exp, 0.5, opts)) <= REL_L2
    # same bytes as the host entry (different frame chunking, same kernels)
    assert np.array_equal(got, ocs_lib.activate(x, exp, 0.5, opts))


def test_large_matches_reference_serial(ocs_lib, orc):
    """The reference Serial pipeline (restated in the oracle, pinned to the
    reference build) at window 2^16, power with the Serial runner's value."""
    x = signal(901, 4 * 65536 + 99)
    got = ocs_lib.activate(x, 16, 0.5, "--hanning_window --serial_power")
    ref = orc.serial_pipeline(x, 16, 0.5, "--hanning_window")
    assert orc.rel_l2(got, ref) <= REL_L2


@pytest.mark.parametrize("exp", [16, 18])
def test_large_small_scratch(ocs_lib, orc, monkeypatch, exp):
    """A 1 MB scratch limit: each launch pair holds a few frames, so the
    column pass's groups of four frames end part-way through a launch."""
    monkeypatch.setenv("OCS_LARGE_SCRATCH_MB", "1")
    N = 1 << exp
    x = signal(950 + exp, 7 * N + 333)
    for opts, ov in (("--hamming_window", 0.5), ("--blackman_window --half_complex_return", 0.75),
                     ("--hanning_window --remove_dc", 0.3)):
        got = ocs_lib.activate(x, exp, ov, opts)
        assert orc.rel_l2(got, orc.fp64_stft(x, exp, ov, opts)) <= REL_L2, (exp, opts, ov)

