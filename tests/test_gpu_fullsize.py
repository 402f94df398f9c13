"""Parity at full size, through the C ABI, against the FP64 oracle.

1. The window sweep's own workload: a 1e8-sample multi-sinusoid signal at
   windows 2^6, 2^10 and 2^15, Hamming and Blackman, power and half-complex
   (reference layout, plus the dense layout whose rows reach the zero-padded
   tail).  Frames from the start, the middle and the end of the output are
   compared with the oracle run on the matching slice of the signal; the frame
   count and the output length are checked bit for bit against toQuot
   (GLOBAL/RunnerInterface.hpp:26-35) restated in float32.
2. A request whose output crosses float index 2^31 (OFullSize between 2^31
   and 2^32, the reference's 32-bit limit): 1.1e9 samples at window 2^10,
   overlap 0.5, through the device entry, the host entry and the stage hooks
   (Overlap, Window, RemoveDC, EXP, ToPower / HalfComplex), with the frames on
   either side of index 2^31 compared with the oracle.

Bars: rel-L2 <= 1e-5 per group of frames against the FP64 oracle; lengths
exact."""
import numpy as np
import pytest

from tests.conftest import sweep_signal, to_quot_f32

pytestmark = pytest.mark.gpu
REL_L2 = 1e-5
K = 8  # frames per checked group

SWEEP_N = 100_000_000


def _row_floats(N: int, opts: str) -> int:
    half = "--half_complex_return" in opts
    if "--layout=dense" in opts:
        return (N // 2 + 1) * (2 if half else 1)
    return 2 * N if half else N


def _out_frames(g, opts: str) -> int:
    """Frames present in the output (compat half-complex holds ceil(qt/2))."""
    if "--half_complex_return" in opts and "--layout=dense" not in opts:
        return int(g.frames)
    return int(g.qt)


def _oracle_frames(orc, x_slice: np.ndarray, exp: int, ov: float, opts: str, hop: int, nfloats: int):
    """Oracle output of the first frames of a signal slice that starts at a
    frame boundary.  The slice is padded with zeros (what frames see past the
    signal end) to a length that holds 2K + 1 frames, so that every checked
    frame is complete in the oracle's own output, whatever the layout."""
    N = 1 << exp
    L = (2 * K + 1) * hop + N
    xs = np.zeros(L, dtype=np.float32)
    m = min(L, x_slice.size)
    xs[:m] = x_slice[:m]
    ref = orc.fp64_stft(xs, exp, ov, opts)
    assert ref.size >= nfloats
    return ref[:nfloats]


def _check_groups(orc, get_out, get_x, g, exp, ov, opts, firsts):
    """Compares groups of K output frames starting at each frame in `firsts`."""
    N = 1 << exp
    row = _row_floats(N, opts)
    for f0 in firsts:
        a = f0 * row
        b = min((f0 + K) * row, int(g.out_floats))
        got = get_out(a, b)
        s0 = f0 * g.hop
        L = (2 * K + 1) * g.hop + N
        ref = _oracle_frames(orc, get_x(s0, s0 + L), exp, ov, opts, g.hop, b - a)
        err = orc.rel_l2(got, ref)
        assert err <= REL_L2, (exp, ov, opts, f0, err)


@pytest.fixture(scope="module")
def sweep():
    import torch

    x = sweep_signal(SWEEP_N)
    return x, torch.from_numpy(x).cuda()


SWEEP_CASES = [(e, w, o) for e in (6, 10, 15) for w in ("--hamming_window", "--blackman_window")
               for o in ("", " --half_complex_return", " --half_complex_return --layout=dense")]


@pytest.mark.parametrize("exp,win,out", SWEEP_CASES)
def test_sweep_full_size_vs_fp64(ocs_lib, orc, sweep, exp, win, out):
    import torch

    x, d_x = sweep
    opts = win + out
    ov = 0.5
    N = 1 << exp
    g = ocs_lib.geometry(x.size, exp, ov, opts)
    # geometry bit for bit: toQuot in float32, OFullSize, the layout's length
    qt = to_quot_f32(x.size, N, ov)
    assert g.qt == qt and g.hop == N // 2 and g.ofull == qt * N
    og = orc.geometry(x.size, exp, ov)
    assert (og.qt, og.hop, og.ofull) == (g.qt, g.hop, g.ofull)
    if "--layout=dense" in opts:
        assert g.out_floats == qt * (N // 2 + 1) * 2
    else:
        assert g.out_floats == qt * N
    d_out = torch.full((g.out_floats + 64,), float("nan"), device="cuda")
    ocs_lib.activate_device(d_x, x.size, exp, ov, opts, d_out, g.out_floats)
    torch.cuda.synchronize()
    # the layout is filled exactly: nothing before out_floats left unwritten, nothing after it written
    assert not bool(torch.isnan(d_out[: g.out_floats]).any())
    assert bool(torch.isnan(d_out[g.out_floats:]).all())
    F = _out_frames(g, opts)
    firsts = [0, F // 2 - K // 2, F - K]
    _check_groups(orc, lambda a, b: d_out[a:b].cpu().numpy(), lambda a, b: x[a:b], g, exp, ov, opts, firsts)
    del d_out


def test_sweep_full_size_host_entry(ocs_lib, orc, sweep):
    """The headline configuration through ocs_activate (host buffers, chunked
    copies and launches), frames on either side of the chunk boundaries."""
    x, _ = sweep
    exp, ov, opts = 10, 0.5, "--hamming_window --remove_dc"
    g = ocs_lib.geometry(x.size, exp, ov, opts)
    got = ocs_lib.activate(x, exp, ov, opts)
    assert got.size == g.out_floats == g.qt * 1024
    F = int(g.qt)
    firsts = [0, F // 16 - K // 2, F // 3, F // 2 - K // 2, F - K]
    _check_groups(orc, lambda a, b: got[a:b], lambda a, b: x[a:b], g, exp, ov, opts, firsts)


# ------------------------------------------------------------ across 2^31
BIG_N = 1_100_000_000
BIG_EXP = 10
BIG_OV = 0.5


def _mem_available_gb() -> float:
    try:
        with open("/proc/meminfo") as f:
            for line in f:
                if line.startswith("MemAvailable:"):
                    return int(line.split()[1]) / 2**20
    except OSError:
        pass
    return 0.0


@pytest.fixture(scope="module")
def big():
    import torch

    gen = torch.Generator(device="cuda")
    gen.manual_seed(31)
    d_x = torch.rand(BIG_N, device="cuda", generator=gen).mul_(2.0).sub_(1.0)
    yield d_x
    del d_x
    torch.cuda.empty_cache()


def _big_geometry(ocs_lib, opts):
    g = ocs_lib.geometry(BIG_N, BIG_EXP, BIG_OV, opts)
    assert 2**31 < g.ofull < 2**32
    assert g.qt == to_quot_f32(BIG_N, 1 << BIG_EXP, BIG_OV)
    return g


def _firsts_across(index: int, row: int, F: int):
    """Groups at the start, straddling output float `index`, and at the end."""
    f = index // row
    return [0, f - K // 2, F - K]


@pytest.mark.parametrize("opts", ["--hamming_window", "--blackman_window --half_complex_return"])
def test_output_across_2pow31_device_entry(ocs_lib, orc, big, opts):
    import torch

    d_x = big
    g = _big_geometry(ocs_lib, opts)
    N = 1 << BIG_EXP
    d_out = torch.empty(g.out_floats, device="cuda")
    ocs_lib.activate_device(d_x, BIG_N, BIG_EXP, BIG_OV, opts, d_out, g.out_floats)
    torch.cuda.synchronize()
    F = _out_frames(g, opts)
    firsts = _firsts_across(2**31, _row_floats(N, opts), F)
    _check_groups(orc, lambda a, b: d_out[a:b].cpu().numpy(), lambda a, b: d_x[a:min(b, BIG_N)].cpu().numpy(),
                  g, BIG_EXP, BIG_OV, opts, firsts)
    del d_out
    torch.cuda.empty_cache()


def test_output_across_2pow31_host_entry(ocs_lib, orc, big):
    if _mem_available_gb() < 40:
        pytest.skip("needs about 14 GB of host memory for the signal and the result")
    d_x = big
    opts = "--hanning_window --remove_dc"
    g = _big_geometry(ocs_lib, opts)
    x = d_x.cpu().numpy()
    got = ocs_lib.activate(x, BIG_EXP, BIG_OV, opts)
    assert got.size == g.out_floats
    firsts = _firsts_across(2**31, 1 << BIG_EXP, int(g.qt))
    _check_groups(orc, lambda a, b: got[a:b], lambda a, b: x[a:b], g, BIG_EXP, BIG_OV, opts, firsts)
    del got, x


def test_output_across_2pow31_stage_hooks(ocs_lib, orc, big):
    """Default_Pipeline driven hook by hook (RunnerCommon.cpp:184-316) on
    [qt][N] planes of more than 2^31 floats each."""
    import torch

    d_x = big
    g = _big_geometry(ocs_lib, "--hamming_window --remove_dc")
    N = 1 << BIG_EXP
    rf = ocs_lib.runnerFunction
    real = torch.empty(g.ofull, device="cuda")
    imag = torch.empty(g.ofull, device="cuda")
    rf.Overlap(d_x, g.ofull, BIG_N, BIG_EXP, g.hop, real)
    rf.Window("Hamming", real, g.ofull, N)
    rf.RemoveDC(real, g.qt, g.ofull, N)
    rf.EXP(real, imag, g.ohalf, BIG_EXP)
    out = torch.empty(g.ofull, device="cuda")
    rf.ToPower(out, real, imag, g.ofull)
    torch.cuda.synchronize()
    get_x = lambda a, b: d_x[a:min(b, BIG_N)].cpu().numpy()  # noqa: E731
    opts = "--hamming_window --remove_dc"
    _check_groups(orc, lambda a, b: out[a:b].cpu().numpy(), get_x, g, BIG_EXP, BIG_OV, opts,
                  _firsts_across(2**31, N, int(g.qt)))
    rf.HalfComplex(out, real, imag, g.ohalf, BIG_EXP)
    torch.cuda.synchronize()
    opts_h = opts + " --half_complex_return"
    gh = _big_geometry(ocs_lib, opts_h)
    _check_groups(orc, lambda a, b: out[a:b].cpu().numpy(), get_x, gh, BIG_EXP, BIG_OV, opts_h,
                  _firsts_across(2**31, 2 * N, int(gh.frames)))
    del real, imag, out
    torch.cuda.empty_cache()
