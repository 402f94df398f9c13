"""Every kernel variant (one frame per FFT with direct or staged I/O, two
frames per FFT in scalar or packed FP32x2 arithmetic, lanes per frame)
against the FP64 oracle.  Variants are forced through the
runner's environment switches in a child process, so each one is exercised
regardless of which the autotuner would pick."""
import json
import os
import subprocess
import sys

import pytest

from tests.conftest import ROOT

pytestmark = pytest.mark.gpu

CHILD = r'''
import json, sys
import numpy as np
sys.path.insert(0, {root!r})
import occastft_gb300 as ocs
from oracle import orc
res = []
for exp in range(6, 16):
    for opts in ("--hamming_window --remove_dc", "--blackman_window --half_complex_return",
                 "--hanning_window --layout=dense", "--hanning_window --half_complex_return --layout=dense --remove_dc",
                 "--flattop_window --serial_power"):
        N = 1 << exp
        x = np.random.default_rng(exp).uniform(-1, 1, 7 * N + 91).astype(np.float32)
        got = ocs.activate(x, exp, 0.5, opts)
        ref = orc.fp64_stft(x, exp, 0.5, opts)
        res.append([exp, opts, orc.rel_l2(got, ref), int(got.size == ref.size)])
print(json.dumps(res))
'''


@pytest.mark.parametrize("env", [
    {"OCS_KERNEL": "tpf", "OCS_AUTOTUNE": "0"},
    {"OCS_KERNEL": "x2", "OCS_AUTOTUNE": "0"},
    {"OCS_KERNEL": "pair", "OCS_AUTOTUNE": "0"},
    {"OCS_KERNEL": "single", "OCS_IO_SCHEME": "direct", "OCS_AUTOTUNE": "0"},
    {"OCS_KERNEL": "single", "OCS_AUTOTUNE": "0"},
    {"OCS_AUTOTUNE": "0"},
    {"OCS_AUTOTUNE": "1"},
])
def test_variant_parity(env):
    e = dict(os.environ)
    e.update(env)
    out = subprocess.run([sys.executable, "-c", CHILD.format(root=ROOT)], env=e, capture_output=True, text=True,
                         timeout=600)
    assert out.returncode == 0, out.stderr[-2000:]
    res = json.loads(out.stdout.strip().splitlines()[-1])
    for exp, opts, err, size_ok in res:
        assert size_ok, (exp, opts)
        assert err <= 1e-5, (env, exp, opts, err)
