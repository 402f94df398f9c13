"""Uneven batches in one persistent launch (C ABI ocs_batch_device):
per-request parity with the single-request path and the FP64 oracle,
alone-vs-in-the-mix equality, per-request errors, CUDA-graph capture."""
import numpy as np
import pytest

from tests.conftest import signal

REL_L2 = 1e-5
pytestmark = pytest.mark.gpu

WINDOWS = ["--hanning_window", "--hamming_window", "--blackman_window", "--flattop_window",
           "--gaussian_window=x0.3<<sigma", ""]
OUTS = ["", " --half_complex_return", " --layout=dense", " --half_complex_return --layout=dense", " --serial_power"]


def _mix(count, seed=0, exps=range(6, 16)):
    import torch

    rng = np.random.default_rng(seed)
    exps = list(exps)
    items = []
    for i in range(count):
        exp = int(rng.choice(exps))
        N = 1 << exp
        n = int(rng.integers(N // 2, 12 * N))
        ov = float(rng.choice([0.0, 0.25, 0.5, 0.75, 0.3]))
        opts = str(rng.choice(WINDOWS)) + str(rng.choice(OUTS)) + (" --remove_dc" if rng.random() < 0.5 else "")
        x = signal(1000 + i, n)
        items.append((x, exp, ov, opts.strip()))
    return items


def _run_batch(ocs_lib, items, stream=None):
    import torch

    bufs = []
    reqs_in = []
    for (x, exp, ov, opts) in items:
        g = ocs_lib.geometry(x.size, exp, ov, opts)
        d_in = torch.from_numpy(x).cuda()
        d_out = torch.full((g.out_floats + 8,), float("nan"), device="cuda")
        bufs.append((d_in, d_out, g))
        reqs_in.append((d_in, x.size, exp, ov, opts, d_out, g.out_floats))
    reqs = ocs_lib.make_requests(reqs_in)
    st = ocs_lib.batch_device(reqs, stream)
    torch.cuda.synchronize()
    return st, [b[1].cpu().numpy() for b in bufs], bufs


def test_mixed_batch_matches_single_requests(ocs_lib, orc):
    items = _mix(48, seed=1)
    st, outs, bufs = _run_batch(ocs_lib, items)
    assert all(s == 0 for s in st), st
    for (x, exp, ov, opts), out, (_, _, g) in zip(items, outs, bufs):
        got = out[: g.out_floats]
        assert not np.isnan(got).any() and np.isnan(out[g.out_floats:]).all(), (exp, opts)
        single = ocs_lib.activate(x, exp, ov, opts)
        assert orc.rel_l2(got, single) <= REL_L2, (exp, ov, opts)
        ref = orc.fp64_stft(x, exp, ov, opts)
        assert orc.rel_l2(got, ref) <= REL_L2, (exp, ov, opts)


def test_alone_equals_in_the_mix(ocs_lib):
    items = _mix(30, seed=2, exps=range(6, 14))
    _, mixed, _ = _run_batch(ocs_lib, items)
    for k in (0, 7, 19, 29):
        _, alone, _ = _run_batch(ocs_lib, [items[k]])
        assert np.array_equal(alone[0], mixed[k], equal_nan=True), k


def test_batch_deterministic(ocs_lib):
    items = _mix(20, seed=3)
    _, a, _ = _run_batch(ocs_lib, items)
    _, b, _ = _run_batch(ocs_lib, items)
    for x, y in zip(a, b):
        assert np.array_equal(x, y, equal_nan=True)


def test_tile_length_changes_nothing(ocs_lib, orc, monkeypatch):
    """Every tile length the batch autotuner may pick (8 .. 64 frame groups per
    tile) writes the same bytes: tiles only split frames between CTAs."""
    items = _mix(40, seed=7, exps=range(6, 14))
    outs = {}
    for g in ("8", "16", "32", "64"):
        monkeypatch.setenv("OCS_BATCH_GROUPS", g)
        st, out, bufs = _run_batch(ocs_lib, items)
        assert all(s == 0 for s in st), (g, st)
        outs[g] = [o[: b[2].out_floats] for o, b in zip(out, bufs)]
    for g in ("16", "32", "64"):
        for a, b in zip(outs["8"], outs[g]):
            assert np.array_equal(a, b), g
    # and the tuned choice (first uncaptured call of this mix) too
    monkeypatch.delenv("OCS_BATCH_GROUPS")
    st, out, bufs = _run_batch(ocs_lib, items)
    for a, o, b in zip(outs["8"], out, bufs):
        assert np.array_equal(a, o[: b[2].out_floats])
    for (x, exp, ov, opts), a in zip(items, outs["8"]):
        assert orc.rel_l2(a, orc.fp64_stft(x, exp, ov, opts)) <= REL_L2, (exp, ov, opts)


def test_per_request_errors(ocs_lib, orc):
    import torch

    x = signal(5, 5000)
    d_in = torch.from_numpy(x).cuda()
    g = ocs_lib.geometry(x.size, 8, 0.5, "--hanning_window")
    outs = [torch.zeros(g.out_floats, device="cuda") for _ in range(3)]
    reqs = ocs_lib.make_requests([
        (d_in, x.size, 8, 0.5, "--hanning_window", outs[0], g.out_floats),
        (d_in, x.size, 5, 0.5, "--hanning_window", outs[1], g.out_floats),          # exponent below 6
        (d_in, x.size, 8, 0.5, "--gaussian_window=4<<sigma", outs[2], g.out_floats),  # sigma parse error
    ])
    st = ocs_lib.batch_device(reqs)
    torch.cuda.synchronize()
    assert st == [0, ocs_lib.OCS_EINVAL, ocs_lib.OCS_EPIPELINE]
    assert orc.rel_l2(outs[0].cpu().numpy(), orc.fp64_stft(x, 8, 0.5, "--hanning_window")) <= REL_L2


def test_tensor_core_precision_is_honoured_in_batches(ocs_lib, orc):
    """A request that asks for a tensor-core form gets that form in a batch
    (its own launch beside the persistent FP32 launch): the same bits as the
    single-request call with the same options, not the FP32 result."""
    items = [(signal(40, 70000), 10, 0.75, "--hanning_window --precision=tc-fp16"),
             (signal(41, 50000), 9, 0.5, "--hamming_window"),
             (signal(42, 90000), 12, 0.5, "--blackman_window --half_complex_return --precision=tc-bf16x2")]
    import torch

    st, outs, bufs = _run_batch(ocs_lib, items)
    assert st == [0, 0, 0]
    for (x, exp, ov, opts), out, (d_in, _, g) in zip(items, outs, bufs):
        got = out[: g.out_floats]
        d_single = torch.empty(g.out_floats, device="cuda")
        ocs_lib.activate_device(d_in, x.size, exp, ov, opts, d_single, g.out_floats)
        torch.cuda.synchronize()
        single = d_single.cpu().numpy()
        if "--precision" in opts:
            assert np.array_equal(got, single), opts
        else:  # the batch kernel and the single-request kernel may differ in rounding
            assert orc.rel_l2(got, single) <= REL_L2, opts
        tol = 1e-4 if "bf16x2" in opts else REL_L2
        assert orc.rel_l2(got, orc.fp64_stft(x, exp, ov, opts)) <= tol, opts
    # the tensor-core result differs from the FP32 one: the form really ran
    fp32 = ocs_lib.activate(items[0][0], 10, 0.75, "--hanning_window")
    assert not np.array_equal(outs[0][: bufs[0][2].out_floats], fp32)


def test_batch_cuda_graph_capture(ocs_lib):
    import torch

    items = _mix(24, seed=4, exps=range(8, 13))
    bufs = []
    reqs_in = []
    for (x, exp, ov, opts) in items:
        g = ocs_lib.geometry(x.size, exp, ov, opts)
        d_in = torch.from_numpy(x).cuda()
        d_out = torch.zeros(g.out_floats, device="cuda")
        bufs.append((d_in, d_out))
        reqs_in.append((d_in, x.size, exp, ov, opts, d_out, g.out_floats))
    reqs = ocs_lib.make_requests(reqs_in)
    ocs_lib.batch_prepare(reqs)
    eager = ocs_lib.batch_device(reqs)
    torch.cuda.synchronize()
    ref = [b[1].clone() for b in bufs]
    for b in bufs:
        b[1].zero_()
    s = torch.cuda.Stream()
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.stream(s):
        with torch.cuda.graph(graph, stream=s):
            st = ocs_lib.batch_device(reqs, s)
    assert st == eager
    for b in bufs:
        b[1].zero_()
    torch.cuda.synchronize()
    for _ in range(3):
        graph.replay()
    torch.cuda.synchronize()
    for b, r in zip(bufs, ref):
        assert torch.equal(b[1], r)


def _device_requests(ocs_lib, items):
    import torch

    bufs, reqs_in = [], []
    for (x, exp, ov, opts) in items:
        g = ocs_lib.geometry(x.size, exp, ov, opts)
        d_in = torch.from_numpy(x).cuda()
        d_out = torch.zeros(g.out_floats, device="cuda")
        bufs.append((d_in, d_out))
        reqs_in.append((d_in, x.size, exp, ov, opts, d_out, g.out_floats))
    return bufs, ocs_lib.make_requests(reqs_in)


def test_batch_graph_replays_its_own_requests(ocs_lib):
    """A captured batch keeps its own descriptors: replayed after an eager
    batch and a second capture have used the library's batch buffers, each
    graph still computes exactly its own requests."""
    import torch

    ba, ra = _device_requests(ocs_lib, _mix(16, seed=5, exps=range(6, 14)))
    bb, rb = _device_requests(ocs_lib, _mix(20, seed=6, exps=range(6, 14)))
    assert all(s == 0 for s in ocs_lib.batch_device(ra))
    assert all(s == 0 for s in ocs_lib.batch_device(rb))
    torch.cuda.synchronize()
    ref_a = [b[1].clone() for b in ba]
    ref_b = [b[1].clone() for b in bb]
    s = torch.cuda.Stream()
    graphs = []
    for reqs in (ra, rb):
        ocs_lib.batch_prepare(reqs)  # once before each capture
        g = torch.cuda.CUDAGraph()
        with torch.cuda.stream(s):
            with torch.cuda.graph(g, stream=s):
                ocs_lib.batch_device(reqs, s)
        graphs.append(g)
    for b in ba + bb:
        b[1].zero_()
    ocs_lib.batch_device(rb)  # an eager batch after both captures
    torch.cuda.synchronize()
    graphs[0].replay()
    torch.cuda.synchronize()
    assert all(torch.equal(b[1], r) for b, r in zip(ba, ref_a))
    assert all(torch.equal(b[1], r) for b, r in zip(bb, ref_b))
    for b in ba + bb:
        b[1].zero_()
    torch.cuda.synchronize()
    graphs[1].replay()
    graphs[0].replay()
    torch.cuda.synchronize()
    assert all(torch.equal(b[1], r) for b, r in zip(ba, ref_a))
    assert all(torch.equal(b[1], r) for b, r in zip(bb, ref_b))
