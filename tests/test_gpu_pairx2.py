"""The packed-FP32x2 paired-frame kernel (window 2^10), forced with
OCS_KERNEL=x2 in a child process: every output layout, the overlap-0.5 load
path and the general one, DC removal, a ragged tail and an odd frame count,
against the FP64 oracle and the scalar paired-frame kernel."""
import json
import os
import subprocess
import sys

import pytest

from tests.conftest import ROOT

pytestmark = pytest.mark.gpu

CHILD = r'''
import json, os, sys
import numpy as np
sys.path.insert(0, {root!r})
import occastft_gb300 as ocs
from oracle import orc
res = []
cases = [(0.5, "--hamming_window"), (0.5, "--hanning_window --remove_dc"), (0.75, "--blackman_window"),
         (0.3, "--hamming_window --half_complex_return"), (0.5, "--blackman_window --half_complex_return"),
         (0.5, "--hanning_window --layout=dense"), (0.6, "--hanning_window --half_complex_return --layout=dense"),
         (0.5, "--flattop_window --serial_power"), (0.0, "--gaussian_window=x0.3<<sigma --remove_dc"),
         (-0.5, "")]
for i, (ov, opts) in enumerate(cases):
    for n in (1024 * 9 + 77, 1024 * 40 + 512, 1000):
        x = np.random.default_rng(100 * i + n).uniform(-1, 1, n).astype(np.float32)
        got = ocs.activate(x, 10, ov, opts)
        ref = orc.fp64_stft(x, 10, ov, opts)
        res.append([ov, opts, n, orc.rel_l2(got, ref), int(got.size == ref.size)])
print(json.dumps(res))
'''


@pytest.mark.parametrize("kernel", ["x2", "pair"])
def test_pair_kernels_window_1024(kernel):
    e = dict(os.environ, OCS_KERNEL=kernel, OCS_AUTOTUNE="0")
    out = subprocess.run([sys.executable, "-c", CHILD.format(root=ROOT)], env=e, capture_output=True, text=True,
                         timeout=600)
    assert out.returncode == 0, out.stderr[-2000:]
    for ov, opts, n, err, size_ok in json.loads(out.stdout.strip().splitlines()[-1]):
        assert size_ok, (ov, opts, n)
        assert err <= 1e-5, (kernel, ov, opts, n, err)
