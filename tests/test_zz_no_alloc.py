"""ocs_batch_device_noalloc: the batch entry point for callers that cannot
allocate GPU memory (an application whose own allocator owns the device, or a
process that must not block on or fail in cudaMalloc once it runs).  Its
scratch is a fixed device array inside the library.  This file is collected
last so a run that stops at the first failure has run every other test; it
passes on its own in a fresh process as well.

Checks, through the C ABI: two calls in a row each match the allocating
ocs_batch_device on the same requests within the suite's tolerance, and sizes
beyond the array's limits are refused with an error before any launch."""
import ctypes

import numpy as np
import pytest

from tests.conftest import signal

REL_L2 = 1e-5
pytestmark = pytest.mark.gpu


def _requests(ocs, seed):
    import torch

    rng = np.random.default_rng(seed)
    items, bufs = [], []
    opts_pool = ["--hanning_window --remove_dc", "--blackman_window --half_complex_return", "--hamming_window",
                 "--flattop_window --layout=dense", "--gaussian_window=x0.25<<sigma --serial_power", ""]
    for i in range(40):
        exp = int(rng.integers(6, 14))
        N = 1 << exp
        n = int(rng.integers(N // 2, 9 * N))
        ov = float(rng.choice([0.0, 0.25, 0.5, 0.75]))
        opts = opts_pool[i % len(opts_pool)]
        x = signal(500 + i, n)
        g = ocs.geometry(n, exp, ov, opts)
        d_in = torch.from_numpy(x).cuda()
        bufs.append((d_in, g))
        items.append((x, exp, ov, opts, g))
    return items, bufs


def _run(ocs, items, bufs, fn):
    import torch

    outs = [torch.full((g.out_floats,), float("nan"), device="cuda") for (_, g) in bufs]
    reqs = ocs.make_requests([(bufs[i][0], it[0].size, it[1], it[2], it[3], outs[i], it[4].out_floats)
                              for i, it in enumerate(items)])
    rc = fn(ctypes.cast(reqs, ctypes.c_void_p), len(reqs), torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    return rc, [r.status for r in reqs], [o.cpu().numpy() for o in outs]


def test_noalloc_batch_matches_allocating_batch_twice(ocs_lib, orc):
    L = ocs_lib.lib()
    items, bufs = _requests(ocs_lib, 7)
    rc, st, ref = _run(ocs_lib, items, bufs, L.ocs_batch_device)
    assert rc == 0 and all(s == 0 for s in st)
    for call in range(2):  # two calls in a row share (and reuse) the static array
        rc, st, got = _run(ocs_lib, items, bufs, L.ocs_batch_device_noalloc)
        assert rc == 0, ocs_lib.last_error()
        assert all(s == 0 for s in st), st
        for (x, exp, ov, opts, g), a, b in zip(items, got, ref):
            assert not np.isnan(a).any(), (call, exp, opts)
            assert orc.rel_l2(a, b) <= REL_L2, (call, exp, ov, opts)
    # and against the FP64 oracle for a few
    for (x, exp, ov, opts, g), a in list(zip(items, got))[:6]:
        assert orc.rel_l2(a, orc.fp64_stft(x, exp, ov, opts)) <= REL_L2


def test_noalloc_rejects_oversize(ocs_lib):
    import torch

    L = ocs_lib.lib()
    x = torch.zeros(4096, device="cuda")
    out = torch.zeros(1 << 16, device="cuda")
    # more requests than the array holds descriptors for
    reqs = ocs_lib.make_requests([(x, 4096, 8, 0.5, "--hanning_window", out, out.numel())] * 257)
    rc = L.ocs_batch_device_noalloc(ctypes.cast(reqs, ctypes.c_void_p), len(reqs), None)
    assert rc == ocs_lib.OCS_ENOMEM and "requests" in ocs_lib.last_error()
    # window above the supported range: per-request status
    big = torch.zeros(1 << 15, device="cuda")
    g = ocs_lib.geometry(1 << 15, 14, 0.5, "")
    bout = torch.zeros(g.out_floats, device="cuda")
    reqs = ocs_lib.make_requests([(big, 1 << 15, 14, 0.5, "", bout, g.out_floats)])
    rc = L.ocs_batch_device_noalloc(ctypes.cast(reqs, ctypes.c_void_p), 1, None)
    torch.cuda.synchronize()
    assert rc == 0 and reqs[0].status == ocs_lib.OCS_EINVAL
    # many distinct window tables at 2^13: more than the array's window
    # region holds, so nothing is launched and every accepted request says so
    n = 1 << 14
    xs = torch.zeros(n, device="cuda")
    g = ocs_lib.geometry(n, 13, 0.5, "--gaussian_window=x0.3<<sigma")
    outs = [torch.zeros(g.out_floats, device="cuda") for _ in range(40)]
    reqs = ocs_lib.make_requests([(xs, n, 13, 0.5, f"--gaussian_window=x0.{10 + i}<<sigma", outs[i], g.out_floats)
                                  for i in range(40)])
    rc = L.ocs_batch_device_noalloc(ctypes.cast(reqs, ctypes.c_void_p), len(reqs), None)
    torch.cuda.synchronize()
    assert rc == ocs_lib.OCS_ENOMEM and "window tables" in ocs_lib.last_error()
    assert all(r.status == ocs_lib.OCS_ENOMEM for r in reqs)


def test_noalloc_refuses_tensor_core_precision(ocs_lib):
    """The tensor-core forms need tables the array has no room for: such a
    request is refused with a status, never run in FP32 instead."""
    import torch

    L = ocs_lib.lib()
    n = 1 << 14
    x = torch.from_numpy(signal(71, n)).cuda()
    opts = "--hanning_window --precision=tc-fp16"
    g = ocs_lib.geometry(n, 10, 0.5, opts)
    out = torch.full((g.out_floats,), float("nan"), device="cuda")
    reqs = ocs_lib.make_requests([(x, n, 10, 0.5, opts, out, g.out_floats)])
    rc = L.ocs_batch_device_noalloc(ctypes.cast(reqs, ctypes.c_void_p), 1, None)
    torch.cuda.synchronize()
    assert rc == 0 and reqs[0].status == ocs_lib.OCS_EINVAL
    assert bool(torch.isnan(out).all())


def test_noalloc_refused_under_stream_capture(ocs_lib):
    """A call on a stream that is capturing a CUDA graph returns OCS_EINVAL
    and launches nothing: its descriptors go through a host staging buffer
    that every later call rewrites, so a replay could not reproduce it."""
    import torch

    L = ocs_lib.lib()
    n = 1 << 14
    x = torch.from_numpy(signal(72, n)).cuda()
    g = ocs_lib.geometry(n, 9, 0.5, "--hamming_window")
    out = torch.full((g.out_floats,), float("nan"), device="cuda")
    reqs = ocs_lib.make_requests([(x, n, 9, 0.5, "--hamming_window", out, g.out_floats)])
    # set-up (the first call on the device synchronizes its stream) before the capture
    assert L.ocs_batch_device_noalloc(ctypes.cast(reqs, ctypes.c_void_p), 0, None) == 0
    torch.cuda.synchronize()
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph):
        rc = L.ocs_batch_device_noalloc(ctypes.cast(reqs, ctypes.c_void_p), 1,
                                        torch.cuda.current_stream().cuda_stream)
    assert rc == ocs_lib.OCS_EINVAL and "graph" in ocs_lib.last_error()
    graph.replay()
    torch.cuda.synchronize()
    assert bool(torch.isnan(out).all())
    # the same call outside the capture still works
    rc = L.ocs_batch_device_noalloc(ctypes.cast(reqs, ctypes.c_void_p), 1, None)
    torch.cuda.synchronize()
    assert rc == 0 and reqs[0].status == 0 and not bool(torch.isnan(out).any())
