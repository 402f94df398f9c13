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


def test_plan_tune_ahead_of_first_request(ocs_lib, orc):
    """ocs_plan_tune times the variants for a request shape ahead of time and
    reports the one the request then runs; the request's result is unchanged."""
    import numpy as np

    from tests.conftest import signal

    x = signal(4242, 3_000_017)
    for exp, opts in ((10, "--hamming_window"), (8, "--blackman_window --remove_dc"),
                      (12, "--hanning_window --half_complex_return"), (9, "--nuttall_window --layout=dense")):
        v = ocs_lib.plan_tune(x.size, exp, 0.5, opts)
        assert 0 <= v <= 4, (exp, opts, v)
        assert ocs_lib.plan_tune(x.size, exp, 0.5, opts) == v  # a tuned key keeps its choice
        got = ocs_lib.activate(x, exp, 0.5, opts)
        assert orc.rel_l2(got, orc.fp64_stft(x, exp, 0.5, opts)) <= 1e-5, (exp, opts)
    assert ocs_lib.plan_tune(x.size, 16, 0.5, "--hamming_window") == -1
    assert ocs_lib.plan_tune(x.size, 10, 0.75, "--hanning_window --precision=tc-fp16") == -1
