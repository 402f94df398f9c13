"""ocs_activate with the result written over the signal (the shared-memory
runner path): out == in, and partly overlapping buffers, against separate
buffers.  Sizes give several copy chunks, so later chunks' input would be
overwritten by earlier chunks' results without the ordering."""
import ctypes

import numpy as np
import pytest

from tests.conftest import signal

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("exp,ov,opts", [
    (10, 0.5, "--hamming_window"),
    (8, 0.75, "--hanning_window --half_complex_return"),
    (12, 0.5, "--blackman_window --layout=dense --remove_dc"),
    (10, 0.75, "--hanning_window --precision=tc-fp16"),
])
@pytest.mark.parametrize("shift", [0, 1, 4096, -4096])
def test_in_place(ocs_lib, exp, ov, opts, shift):
    x = signal(50 + exp, 6_000_001)
    ref = ocs_lib.activate(x, exp, ov, opts)
    g = ocs_lib.geometry(x.size, exp, ov, opts)
    # one host buffer: the signal at offset a, the result at offset a + shift
    a = max(0, -shift)
    buf = np.zeros(a + max(x.size, shift + g.out_floats) + 16, dtype=np.float32)
    buf[a:a + x.size] = x
    base = buf.ctypes.data
    n_out = ctypes.c_uint64(0)
    ocs_lib._check(ocs_lib.lib().ocs_activate(base + 4 * a, x.size, exp, ov, opts.encode(),
                                              base + 4 * (a + shift), g.out_floats, ctypes.byref(n_out)))
    got = buf[a + shift: a + shift + g.out_floats]
    assert n_out.value == g.out_floats
    np.testing.assert_allclose(got, ref, rtol=1e-6, atol=1e-6 * float(np.abs(ref).max()))
