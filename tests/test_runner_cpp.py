"""The C++ runner (reference vendor contract: Runner + runnerFunction hooks)
built over the C ABI: symbols on CPU, both pipelines on the GPU."""
import os
import subprocess
import tempfile

import numpy as np
import pytest

from tests.conftest import ROOT, signal

PKG = os.path.join(ROOT, "occastft_gb300")
RUNNER_LIB = os.path.join(PKG, "libocs_runner.so")
DEMO = os.path.join(PKG, "ocs_runner_demo")

CONTRACT = [
    "Runner::InitEnv()", "Runner::BuildKernel()", "Runner::UnInit()", "Runner::Runner(int const&)",
    "Runner::ActivateSTFT(", "runnerFunction::Overlap(", "runnerFunction::Hanning(", "runnerFunction::Hamming(",
    "runnerFunction::Blackman(", "runnerFunction::Nuttall(", "runnerFunction::Blackman_Nuttall(",
    "runnerFunction::Blackman_Harris(", "runnerFunction::FlatTop(", "runnerFunction::Gaussian(",
    "runnerFunction::RemoveDC(", "runnerFunction::EXP6(", "runnerFunction::EXP7(", "runnerFunction::EXP8(",
    "runnerFunction::EXP9(", "runnerFunction::EXP10(", "runnerFunction::EXP11(", "runnerFunction::EXPC(",
    "runnerFunction::HalfComplex(", "runnerFunction::ToPower(", "runnerFunction::Default_Pipeline(",
]


@pytest.fixture(scope="module")
def built(ocs_lib):
    if not (os.path.exists(RUNNER_LIB) and os.path.exists(DEMO)):
        from occastft_gb300 import build

        build.build()
    return True


def test_runner_exports_contract(built):
    out = subprocess.run(["nm", "-DC", RUNNER_LIB], capture_output=True, text=True, check=True).stdout
    for sym in CONTRACT:
        assert sym in out, sym


def test_runner_header_compiles():
    src = '#include "occastft_runner.hpp"\nint main(){ return toQuot(1048576.0f, 0.5f, 1024.0f) == 2049 ? 0 : 1; }\n'
    with tempfile.TemporaryDirectory() as d:
        p = os.path.join(d, "t.cpp")
        open(p, "w").write(src)
        exe = os.path.join(d, "t")
        subprocess.run(["g++", "-std=c++17", "-I", os.path.join(ROOT, "include"), p, "-o", exe], check=True)
        assert subprocess.run([exe]).returncode == 0


@pytest.mark.gpu
@pytest.mark.parametrize("exp,ov,opts", [
    (10, 0.5, "--hanning_window --remove_dc"),
    (13, 0.5, "--blackman_window --half_complex_return"),
    (7, 0.25, "--gaussian_window=x1.5<<sigma --remove_dc"),
])
def test_runner_fused_and_stage_paths(built, ocs_lib, orc, exp, ov, opts):
    x = signal(31 + exp, 60000)
    with tempfile.TemporaryDirectory() as d:
        fin = os.path.join(d, "in.f32")
        x.tofile(fin)
        outs = {}
        for mode in ("fused", "stages"):
            fout = os.path.join(d, mode + ".f32")
            args = [DEMO, fin, fout, str(exp), str(ov), opts] + (["stages"] if mode == "stages" else [])
            r = subprocess.run(args, capture_output=True, text=True, timeout=300)
            assert r.returncode == 0, r.stderr
            outs[mode] = np.fromfile(fout, dtype=np.float32)
    ref = orc.fp64_stft(x, exp, ov, opts)
    for mode, got in outs.items():
        assert got.size == ref.size, mode
        assert orc.rel_l2(got, ref) <= 1e-5, mode
    # the two processes may autotune to different kernel variants: equal within rounding
    assert orc.rel_l2(outs["fused"], ocs_lib.activate(x, exp, ov, opts)) <= 1e-6


@pytest.mark.gpu
def test_runner_error_status(built):
    with tempfile.TemporaryDirectory() as d:
        fin = os.path.join(d, "in.f32")
        signal(1, 1000).tofile(fin)
        r = subprocess.run([DEMO, fin, os.path.join(d, "o"), "5", "0.5", "--hanning_window"], capture_output=True,
                           text=True)
        assert r.returncode == 1 and "Operation not supported" in r.stderr
