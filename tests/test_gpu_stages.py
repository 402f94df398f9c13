"""The runnerFunction hooks (per-stage, reference [qt][N] planes) through the
C ABI, against the reference's stage outputs and the oracle."""
import numpy as np
import pytest

from tests.conftest import signal

REL_L2 = 1e-5
pytestmark = pytest.mark.gpu


def _t(a):
    import torch

    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


@pytest.mark.parametrize("exp,ov", [(6, 0.5), (10, 0.75), (12, 0.3), (9, -0.25)])
def test_overlap_bit_exact(ocs_lib, orc, exp, ov):
    import torch

    x = signal(21, 30000) - 0.25
    g = orc.geometry(x.size, exp, ov)
    real = torch.empty(g.ofull, device="cuda")
    ocs_lib.runnerFunction.Overlap(_t(x), g.ofull, x.size, exp, g.hop, real)
    torch.cuda.synchronize()
    ref = np.zeros(g.ofull, np.float32)
    orc.lib().orc_overlap(x.ctypes.data_as(orc.ctypes.POINTER(orc.ctypes.c_float)), g.ofull, x.size, exp, g.hop,
                          ref.ctypes.data_as(orc.ctypes.POINTER(orc.ctypes.c_float)))
    assert np.array_equal(real.cpu().numpy().view(np.uint32), ref.view(np.uint32))


def test_window_stage_bit_exact_vs_reference(ocs_lib, golden):
    import torch

    manifest, arrays = golden
    names = {"hanning": "Hanning", "hamming": "Hamming", "blackman": "Blackman", "nuttall": "Nuttall",
             "blackman_nuttall": "Blackman_Nuttall", "blackman_harris": "Blackman_Harris", "flattop": "FlatTop",
             "gaussian": "Gaussian"}
    for w in manifest["windows"]:
        N = 1 << w["exp"]
        x = signal(w["seed"], w["n"])[:N].copy()
        d = _t(x)
        ocs_lib.runnerFunction.Window(names[w["kind"]], d, N, N, w["sigma"])
        torch.cuda.synchronize()
        assert np.array_equal(d.cpu().numpy().view(np.uint32), arrays[w["key"]].view(np.uint32)), w["key"]


def test_remove_dc_stage(ocs_lib, orc):
    import torch

    x = signal(22, 40000) + 0.3
    for exp in (6, 11, 14):
        g = orc.geometry(x.size, exp, 0.5)
        framed = orc.overlap_window(x, exp, 0.5, "hanning")
        ref = orc.overlap_window(x, exp, 0.5, "hanning", remove_dc=True)
        d = _t(framed)
        ocs_lib.runnerFunction.RemoveDC(d, g.qt, g.ofull, 1 << exp)
        torch.cuda.synchronize()
        got = d.cpu().numpy()
        assert np.max(np.abs(got - ref)) <= 1e-6 * max(1.0, np.abs(framed).max())


@pytest.mark.parametrize("exp", list(range(6, 16)))
def test_fft_stage_planes(ocs_lib, orc, exp):
    import torch

    N = 1 << exp
    x = signal(23 + exp, 5 * N)
    framed = orc.overlap_window(x, exp, 0.5, "hamming")
    g = orc.geometry(x.size, exp, 0.5)
    re = _t(framed)
    im = torch.full_like(re, 7.0)  # ignored on input, as the reference's first stage does
    ocs_lib.runnerFunction.EXP(re, im, g.ohalf, exp)
    torch.cuda.synchronize()
    X = np.fft.fft(framed.reshape(g.qt, N).astype(np.float64), axis=1).reshape(-1)
    got = re.cpu().numpy().astype(np.float64) + 1j * im.cpu().numpy().astype(np.float64)
    assert np.linalg.norm(got - X) / np.linalg.norm(X) <= REL_L2


def test_post_stages(ocs_lib):
    import torch

    re = signal(24, 4096)
    im = signal(25, 4096)
    out = torch.empty(4096, device="cuda")
    ocs_lib.runnerFunction.ToPower(out, _t(re), _t(im), 4096)
    hc = torch.empty(4096, device="cuda")
    ocs_lib.runnerFunction.HalfComplex(hc, _t(re), _t(im), 2048, 6)
    torch.cuda.synchronize()
    exp_p = np.sqrt((re * re + im * im).astype(np.float32))
    assert np.array_equal(out.cpu().numpy(), exp_p)
    h = hc.cpu().numpy()
    assert np.array_equal(h[0::2], re[:2048]) and np.array_equal(h[1::2], im[:2048])


def test_stage_pipeline_equals_fused(ocs_lib, orc):
    """Default_Pipeline driven hook by hook equals the fused path."""
    import torch

    exp, ov = 10, 0.5
    x = signal(26, 100000)
    g = orc.geometry(x.size, exp, ov)
    real = torch.empty(g.ofull, device="cuda")
    imag = torch.zeros(g.ofull, device="cuda")
    out = torch.empty(g.ofull, device="cuda")
    rf = ocs_lib.runnerFunction
    rf.Overlap(_t(x), g.ofull, x.size, exp, g.hop, real)
    rf.Window("Hanning", real, g.ofull, 1 << exp)
    rf.RemoveDC(real, g.qt, g.ofull, 1 << exp)
    rf.EXP(real, imag, g.ohalf, exp)
    rf.ToPower(out, real, imag, g.ofull)
    torch.cuda.synchronize()
    fused = ocs_lib.activate(x, exp, ov, "--hanning_window --remove_dc")
    assert orc.rel_l2(out.cpu().numpy(), fused) <= REL_L2
