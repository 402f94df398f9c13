"""Builds the native runner in place: occastft_gb300/libocs_gb300.so.

CUDA sources are compiled for sm_103a only; translation units build in
parallel.  Run `python -m occastft_gb300.build` or call build().
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
RUNNER = os.path.join(PKG, "runner")
OUT_DIR = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libocs_gb300.so")
RUNNER_LIB = os.path.join(PKG, "libocs_runner.so")
RUNNER_DEMO = os.path.join(PKG, "ocs_runner_demo")
STANDALONE = os.path.join(PKG, "standalone")
# the runner executable the reference's proxy launches (`<dir>/cudaRun <port>`)
CUDARUN = os.path.join(PKG, "cudaRun")
STANDALONE_SOURCES = ["request_codec.cpp", "ws_server.cpp", "shm_payload.cpp", "cudaRun.cpp"]

CU_SOURCES = ["stft_fused.cu", "stft_fused_lo.cu", "stft_fused_hi.cu", "stft_pair_lo.cu", "stft_pair_hi.cu", "stft_pairx2.cu",
              "stft_batch.cu", "stft_batch_noalloc.cu", "stft_tc.cu", "stft_stages.cu", "stft_large.cu", "stft_tpf.cu"]
CPP_SOURCES = ["ocs_api.cpp", "ocs_host.cpp", "ocs_server.cpp"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def cuda_home() -> str:
    for c in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if c and os.path.exists(os.path.join(c, "bin", "nvcc")):
            return c
    nvcc = shutil.which("nvcc")
    if nvcc:
        return os.path.dirname(os.path.dirname(nvcc))
    raise RuntimeError("nvcc not found")


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed: " + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r.stdout + r.stderr


def _stale(target: str, deps) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _headers():
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    hs.append(os.path.join(ROOT, "include", "occastft_gb300.h"))
    hs.append(os.path.join(ROOT, "include", "occastft_runner.hpp"))
    return [h for h in hs if os.path.exists(h)]


def build(verbose: bool = False, force: bool = False) -> str:
    cuda = cuda_home()
    nvcc = os.path.join(cuda, "bin", "nvcc")
    os.makedirs(OUT_DIR, exist_ok=True)
    inc = ["-I", CSRC, "-I", os.path.join(ROOT, "include"), "-I", os.path.join(cuda, "include")]
    headers = _headers()
    jobs = []
    objs = []
    for src in CU_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(OUT_DIR, src + ".o")
        objs.append(o)
        if force or _stale(o, [s] + headers):
            jobs.append([nvcc, "-std=c++17", *ARCH, "-lineinfo", "-O3", "--expt-relaxed-constexpr",
                         "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off", *inc, "-c", s, "-o", o])
    for src in CPP_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(OUT_DIR, src + ".o")
        objs.append(o)
        if force or _stale(o, [s] + headers):
            jobs.append(["g++", "-std=c++17", "-O2", "-fPIC", "-ffp-contract=off", "-Wall", *inc, "-c", s, "-o", o])
    runner_srcs = [os.path.join(RUNNER, f) for f in ("RunnerGB300.cpp", "functionImpl.cpp", "RunnerStandalone.cpp")]
    runner_objs = []
    for s in runner_srcs:
        if not os.path.exists(s):
            continue
        o = os.path.join(OUT_DIR, os.path.basename(s) + ".o")
        runner_objs.append(o)
        if force or _stale(o, [s] + headers):
            jobs.append(["g++", "-std=c++17", "-O2", "-fPIC", "-Wall", *inc, "-I", RUNNER, "-c", s, "-o", o])
    sa_objs = []
    sa_headers = [os.path.join(STANDALONE, f) for f in os.listdir(STANDALONE) if f.endswith(".hpp")] \
        if os.path.isdir(STANDALONE) else []
    for f in STANDALONE_SOURCES:
        s = os.path.join(STANDALONE, f)
        if not os.path.exists(s):
            continue
        o = os.path.join(OUT_DIR, "sa_" + f + ".o")
        sa_objs.append(o)
        if force or _stale(o, [s] + headers + sa_headers):
            jobs.append(["g++", "-std=c++17", "-O2", "-Wall", *inc, "-I", STANDALONE, "-c", s, "-o", o])
    log = []
    with ThreadPoolExecutor(max_workers=max(2, min(8, os.cpu_count() or 2))) as ex:
        for out in ex.map(_run, jobs):
            log.append(out)
    libdir = os.path.join(cuda, "lib64")
    if not os.path.isdir(libdir):
        libdir = os.path.join(cuda, "lib")
    if force or jobs or not os.path.exists(LIB):
        _run([nvcc, *ARCH, "-shared", "-o", LIB, *objs, "-Xlinker", "-soname=libocs_gb300.so",
              "-cudart", "static", "-lpthread"])
    if runner_objs and (force or jobs or not os.path.exists(RUNNER_LIB) or not os.path.exists(RUNNER_DEMO)):
        # the C++ Runner (reference contract) on top of the C ABI
        _run(["g++", "-shared", "-o", RUNNER_LIB, *runner_objs, "-L", PKG, "-locs_gb300",
              "-Wl,-rpath,$ORIGIN"])
        demo_src = os.path.join(RUNNER, "runner_demo.cpp")
        if os.path.exists(demo_src):
            _run(["g++", "-std=c++17", "-O2", *inc, "-I", RUNNER, demo_src, "-o", RUNNER_DEMO, "-L", PKG,
                  "-locs_runner", "-locs_gb300", "-L", libdir, "-lcudart", "-Wl,-rpath,$ORIGIN",
                  "-Wl,-rpath," + libdir])
    if sa_objs and (force or jobs or not os.path.exists(CUDARUN)):
        _run(["g++", "-o", CUDARUN, *sa_objs, "-L", PKG, "-locs_gb300", "-lpthread", "-lrt", "-Wl,-rpath,$ORIGIN"])
    if verbose:
        print("\n".join(l for l in log if l.strip()))
    return LIB


if __name__ == "__main__":
    build(verbose="-v" in sys.argv, force="-f" in sys.argv)
    print(LIB)
