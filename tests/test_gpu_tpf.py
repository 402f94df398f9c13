"""The thread-per-frame kernels (one lane per frame at window 2^6, power and
half-complex; two and four lanes per frame at 2^7 and 2^8, power), forced with OCS_KERNEL=tpf,
against the FP64 oracle: frame advances that are multiples of 4, 2 and 1
samples (16-, 8- and 4-byte copies), ragged signal ends, one frame, DC
removal, the dense layout and the Serial runner's power."""
import numpy as np
import pytest

from tests.conftest import signal

pytestmark = pytest.mark.gpu
REL_L2 = 1e-5


@pytest.fixture()
def tpf(monkeypatch):
    monkeypatch.setenv("OCS_KERNEL", "tpf")


@pytest.mark.parametrize("exp", [6, 7, 8])
@pytest.mark.parametrize("n", [1, 63, 64, 1000, 4097, 1_000_003])
@pytest.mark.parametrize("ov", [0.5, 0.75, 0.3, 0.33, 0.1])
def test_tpf_sizes_and_advances(tpf, ocs_lib, orc, exp, n, ov):
    x = signal(n % 1000 + 17, n)
    for opts in ("--hamming_window", "--hanning_window --remove_dc", "--blackman_window --layout=dense",
                 "--flattop_window --serial_power", "--nuttall_window --remove_dc --layout=dense",
                 "--hamming_window --half_complex_return",
                 "--blackman_window --remove_dc --half_complex_return --layout=dense",
                 "--gaussian_window=x0.4<<sigma --remove_dc"):
        got = ocs_lib.activate(x, exp, ov, opts)
        ref = orc.fp64_stft(x, exp, ov, opts)
        assert got.size == ref.size
        assert orc.rel_l2(got, ref) <= REL_L2, (exp, n, ov, opts)


@pytest.mark.parametrize("exp", [7, 8])
def test_tpf_large_dc_offset(tpf, ocs_lib, orc, exp):
    """A signal sitting on a DC offset 1000 times its swing: only the frame's
    first lane carries the mean, the others cancel it exactly."""
    x = (signal(21, 200_003) * 1e-3 + 1.0).astype(np.float32)
    got = ocs_lib.activate(x, exp, 0.5, "--hanning_window --remove_dc")
    ref = orc.fp64_stft(x, exp, 0.5, "--hanning_window --remove_dc")
    assert orc.rel_l2(got, ref) <= 1e-4


@pytest.mark.parametrize("exp", [6, 7, 8])
def test_tpf_matches_other_kernels(tpf, ocs_lib, monkeypatch, exp):
    """Same result as the cooperative kernels within the suite's cross-kernel
    tolerance."""
    x = signal(5, 3_000_017)
    got = ocs_lib.activate(x, exp, 0.5, "--hanning_window --remove_dc")
    monkeypatch.setenv("OCS_KERNEL", "single")
    ref = ocs_lib.activate(x, exp, 0.5, "--hanning_window --remove_dc")
    np.testing.assert_allclose(got, ref, rtol=1e-5, atol=1e-6 * float(np.abs(ref).max()))


REINIT_CHILD = r'''
import sys
import numpy as np
sys.path.insert(0, {root!r})
import occastft_gb300 as ocs
from oracle import orc
x = np.random.default_rng(11).uniform(-1, 1, 300_001).astype(np.float32)
first = [ocs.activate(x, e, 0.5, "--hamming_window") for e in (6, 7, 8)]
ocs.Runner(0).UnInit()  # frees the plans and window tables
again = [ocs.activate(x, e, 0.5, "--hamming_window") for e in (6, 7, 8)]
same = all(np.array_equal(a, b) for a, b in zip(first, again))
err = max(orc.rel_l2(g, orc.fp64_stft(x, e, 0.5, "--hamming_window")) for g, e in zip(again, (6, 7, 8)))
print("SAME", same, "ERR", err)
'''


def test_tpf_after_reinit():
    """The lanes-per-frame kernels take the window from a host copy kept beside
    the device table; after a shutdown and re-initialisation (new device
    tables) they still get the right coefficients."""
    import os
    import subprocess
    import sys
    from tests.conftest import ROOT
    e = dict(os.environ, OCS_KERNEL="tpf", OCS_AUTOTUNE="0")
    out = subprocess.run([sys.executable, "-c", REINIT_CHILD.format(root=ROOT)], env=e, capture_output=True,
                         text=True, timeout=300)
    assert out.returncode == 0, out.stderr[-2000:]
    line = out.stdout.strip().splitlines()[-1].split()
    assert line[1] == "True", line
    assert float(line[3]) <= REL_L2, line

