"""Frame-range sharding across ranks (the multi-GPU path) on CPU: two gloo
ranks each compute their shard from their input slice (with the oracle as the
per-rank compute) and the gathered rows equal the single-shard result."""
import os
import socket

import numpy as np
import pytest
import torch.distributed as dist
import torch.multiprocessing as mp

from tests.conftest import ROOT, signal


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank(rank, world, port, cfgs, q):
    import sys

    sys.path.insert(0, ROOT)
    import torch

    from occastft_gb300 import shard
    from oracle import orc

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        for (n, exp, ov, opts) in cfgs:
            x = signal(n + exp, n)
            g = orc.geometry(n, exp, ov)
            sh = shard.plan(n, g.qt, g.hop, g.n_window, opts, world)[rank]
            part = orc.fp64_stft(x[sh.s0:sh.s1], exp, ov, opts, nthreads=1) if sh.s1 > sh.s0 else np.zeros(0)
            rows = shard.slice_rows(part, sh) if sh.f1 > sh.f0 else np.zeros(0)
            rows = np.zeros((sh.f1 - sh.f0) * sh.row) if rows.size < (sh.f1 - sh.f0) * sh.row else rows
            gathered = [None] * world
            dist.all_gather_object(gathered, rows)
            if rank == 0:
                full = orc.fp64_stft(x, exp, ov, opts, nthreads=1)
                q.put(bool(np.array_equal(np.concatenate(gathered), full)))
    finally:
        dist.destroy_process_group()


def test_two_rank_frame_shards_equal_single_shard():
    cfgs = [(50000, 10, 0.5, "--hanning_window --remove_dc"), (33333, 8, 0.75, "--blackman_window --layout=dense"),
            (20001, 9, 0.3, "--hamming_window --half_complex_return --layout=dense"), (5000, 12, 0.5, "")]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    mp.start_processes(_rank, args=(2, port, cfgs, q), nprocs=2, join=True, start_method="spawn")
    res = [q.get(timeout=60) for _ in cfgs]
    assert all(res), res


def test_plan_covers_all_frames():
    from occastft_gb300 import shard

    for world in (1, 2, 3, 8):
        sh = shard.plan(1_000_000, 1953, 512, 1024, "", world)
        assert sh[0].f0 == 0 and sh[-1].f1 == 1953
        assert all(a.f1 == b.f0 for a, b in zip(sh, sh[1:]))
    with pytest.raises(ValueError):
        shard.row_floats(1024, "--half_complex_return")
