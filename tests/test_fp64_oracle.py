"""The FP64 oracle against an independent numpy FFT of the same frames."""
import numpy as np
import pytest

from tests.conftest import signal


@pytest.mark.parametrize("exp,ov,opts", [
    (6, 0.5, "--hanning_window --remove_dc"),
    (9, 0.75, "--blackman_window"),
    (11, 0.25, "--hamming_window --remove_dc --layout=dense"),
    (12, 0.5, "--flattop_window --half_complex_return --layout=dense"),
    (10, 0.5, "--nuttall_window --half_complex_return"),
    (8, 0.3, "--gaussian_window=x2.5<<sigma --serial_power"),
])
def test_fp64_matches_numpy(orc, exp, ov, opts):
    N = 1 << exp
    x = signal(5, 7 * N + 33)
    g = orc.geometry(x.size, exp, ov)
    rc, o, _ = orc.parse_options(opts)
    w = orc.window({0: "none", 1: "hanning", 2: "hamming", 3: "blackman", 4: "nuttall", 5: "blackman_nuttall",
                    6: "blackman_harris", 7: "flattop", 8: "gaussian"}[o.window], N, o.sigma).astype(np.float64)
    frames = np.zeros((g.qt, N))
    for f in range(g.qt):
        s = f * g.hop
        seg = x[s:s + N].astype(np.float64)
        frames[f, :seg.size] = seg
    frames *= w
    if o.remove_dc:
        frames -= frames.mean(axis=1, keepdims=True)
    X = np.fft.fft(frames, axis=1)
    if o.half_complex:
        if o.dense:
            exp_out = np.stack([X[:, :N // 2 + 1].real, X[:, :N // 2 + 1].imag], -1).reshape(-1)
        else:
            flat = X.reshape(-1)[: g.ohalf]
            exp_out = np.stack([flat.real, flat.imag], -1).reshape(-1)
    else:
        mag = np.sqrt(2) * np.abs(X.real) if o.serial_power else np.abs(X)
        exp_out = (mag[:, :N // 2 + 1] if o.dense else mag).reshape(-1)
    got = orc.fp64_stft(x, exp, ov, opts)
    assert got.size == exp_out.size
    assert np.max(np.abs(got - exp_out)) <= 1e-9 * max(1.0, np.max(np.abs(exp_out)))
