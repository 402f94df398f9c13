"""Windows 2^16 .. 2^30 (the reference's EXPC range above the fused
kernels): the four-step FFT (two launches up to 2^22, three above) against
the FP64 oracle, every output layout, through the host entry (chunked
copies, several frame ranges) and the device entry; the stage hooks
(runnerFunction::Window / EXPC / HalfComplex / ToPower) at those sizes; plus
the reference Serial pipeline itself, whose result is the full transform at
even exponents and, with the odd-exponent buffer choice fixed, at odd ones."""
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



@pytest.mark.parametrize("exp", [23, 24])
def test_three_pass_windows_match_fp64(ocs_lib, orc, exp):
    """Windows above 2^22: the column pass, a middle pass and the row pass."""
    N = 1 << exp
    x = signal(720 + exp, 3 * N + 12345)
    for i, opts in enumerate(("--hamming_window", "--blackman_window --half_complex_return --remove_dc",
                              "--hanning_window --layout=dense --serial_power")):
        ov = (0.5, 0.75, 0.3)[i]
        got = ocs_lib.activate(x, exp, ov, opts)
        ref = orc.fp64_stft(x, exp, ov, opts)
        assert got.size == ref.size == ocs_lib.geometry(x.size, exp, ov, opts).out_floats, (exp, opts)
        err = orc.rel_l2(got, ref)
        assert err <= REL_L2, (exp, ov, opts, err)


@pytest.mark.parametrize("exp", [16, 20, 23])
def test_expc_stage_hook_large(ocs_lib, orc, exp):
    """runnerFunction::EXPC above 2^15 (Serial/src/functionImpl.cpp:208-262):
    Overlap, Window, RemoveDC, EXPC and HalfComplex / ToPower hook by hook,
    against the FP64 oracle, and against the Serial pipeline restated in the
    oracle where that pipeline is right: up to 2^16.  From 2^17 the
    reference's twiddle index (lsave % segmentSize) * HwindowSize
    (OKL/kernel.okl:141-144) overflows a 32-bit int in the last stages, so
    its result is not the transform; the restatement reproduces that, and the
    GPU result stays with FP64."""
    import torch

    N = 1 << exp
    x = signal(760 + exp, 3 * N + 999)
    ov = 0.5
    g = orc.geometry(x.size, exp, ov)
    rf = ocs_lib.runnerFunction
    real = torch.empty(g.ofull, device="cuda")
    imag = torch.full((g.ofull,), 3.0, device="cuda")  # ignored on input, as the reference's first stage does
    rf.Overlap(torch.from_numpy(x).cuda(), g.ofull, x.size, exp, g.hop, real)
    rf.Window("Hamming", real, g.ofull, N)
    rf.RemoveDC(real, g.qt, g.ofull, N)
    rf.EXP(real, imag, g.ohalf, exp)
    out = torch.empty(g.ofull, device="cuda")
    rf.HalfComplex(out, real, imag, g.ohalf, exp)
    torch.cuda.synchronize()
    opts = "--hamming_window --remove_dc --half_complex_return"
    hc = out.cpu().numpy()
    f64 = orc.fp64_stft(x, exp, ov, opts)
    assert orc.rel_l2(hc, f64) <= REL_L2
    ser = orc.serial_pipeline(x, exp, ov, opts, fix_p4=True, nthreads=16)
    if exp <= 16:
        assert orc.rel_l2(hc, ser) <= REL_L2
    else:
        assert orc.rel_l2(ser, f64) > 0.1  # the reference's own result is off at this size
    rf.ToPower(out, real, imag, g.ofull)
    torch.cuda.synchronize()
    assert orc.rel_l2(out.cpu().numpy(), orc.fp64_stft(x, exp, ov, "--hamming_window --remove_dc")) <= REL_L2


def test_expc_stage_hook_matches_full_transform_planes(ocs_lib):
    """EXPC at 2^17 leaves the full N-bin spectrum of every frame in the two
    planes, checked against a float64 FFT of the same frames."""
    import torch

    exp = 17
    N = 1 << exp
    frames = signal(790, 3 * N).reshape(3, N)
    re = torch.from_numpy(frames.reshape(-1).copy()).cuda()
    im = torch.zeros_like(re)
    ocs_lib.runnerFunction.EXP(re, im, 3 * N // 2, exp)
    torch.cuda.synchronize()
    X = np.fft.fft(frames.astype(np.float64), axis=1).reshape(-1)
    got = re.cpu().numpy().astype(np.float64) + 1j * im.cpu().numpy().astype(np.float64)
    assert np.linalg.norm(got - X) / np.linalg.norm(X) <= REL_L2
