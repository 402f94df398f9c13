"""The thread-per-frame kernel (window 2^6, power outputs), forced with
OCS_KERNEL=tpf, against the FP64 oracle: frame advances that are multiples
of 4, 2 and 1 samples (16-, 8- and 4-byte copies), ragged signal ends, one
frame, DC removal, the dense layout and the Serial runner's power."""
import numpy as np
import pytest

from tests.conftest import signal

pytestmark = pytest.mark.gpu
REL_L2 = 1e-5


@pytest.fixture()
def tpf(monkeypatch):
    monkeypatch.setenv("OCS_KERNEL", "tpf")


@pytest.mark.parametrize("n", [1, 63, 64, 1000, 4097, 1_000_003])
@pytest.mark.parametrize("ov", [0.5, 0.75, 0.3, 0.33, 0.1])
def test_tpf_sizes_and_advances(tpf, ocs_lib, orc, n, ov):
    x = signal(n % 1000 + 17, n)
    for opts in ("--hamming_window", "--hanning_window --remove_dc", "--blackman_window --layout=dense",
                 "--flattop_window --serial_power", "--nuttall_window --remove_dc --layout=dense"):
        got = ocs_lib.activate(x, 6, ov, opts)
        ref = orc.fp64_stft(x, 6, ov, opts)
        assert got.size == ref.size
        assert orc.rel_l2(got, ref) <= REL_L2, (n, ov, opts)


def test_tpf_matches_other_kernels(tpf, ocs_lib, monkeypatch):
    """Same result as the cooperative kernels within the suite's cross-kernel
    tolerance."""
    x = signal(5, 3_000_017)
    got = ocs_lib.activate(x, 6, 0.5, "--hanning_window --remove_dc")
    monkeypatch.setenv("OCS_KERNEL", "single")
    ref = ocs_lib.activate(x, 6, 0.5, "--hanning_window --remove_dc")
    np.testing.assert_allclose(got, ref, rtol=1e-5, atol=1e-6 * float(np.abs(ref).max()))
