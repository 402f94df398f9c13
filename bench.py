"""Benchmark: plain fused FP32 STFT on one GB300 (the 1e8-sample window sweep).

Workload (one "step"): one STFT of a 1e8-sample float32 signal (sum of 8
seeded sinusoids in [20 Hz, 20 kHz] at fs = 48 kHz, amplitudes in
[0.05, 0.5], plus Gaussian noise of sigma 0.01), window 2^10, Hamming,
overlap 0.5, power output in the reference's layout (qt x N floats).  The
metric is input samples per second (Gsamples/s).

  value    device-resident: input already in HBM, one fused kernel per step,
           CUDA events on the launching stream; 1.2 GB per step > L2, so no
           L2 flush is needed between steps.
  e2e      the public C ABI call ocs_activate with pinned host buffers: the
           host->device copy of the signal and the device->host copy of the
           result are inside the timed region.
  roofline algorithmic bytes (4 n + 4 qt N) per launch / mean launch time,
           against the measured HBM copy bandwidth.
  sweep    the rest of the config: windows 2^6..2^15 x {Hamming, Blackman} x
           {power, half-complex}, device-resident.

`--impl reference` times the reference's own CPU implementation of the path
(its OpenMP runner built from source when available, else the pinned oracle
port of it) on all host cores, on a bounded sample of the same workload.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N_SAMPLES = 100_000_000
FS = 48000.0
HEAD_EXP = 10
HEAD_OV = 0.5
HEAD_OPTS = "--hamming_window"
METRIC = "Gsamples/s"


# --------------------------------------------------------------- workload
def signal_params(seed: int = 1):
    rng = np.random.default_rng(seed)
    f = rng.uniform(20.0, 20000.0, 8)
    a = rng.uniform(0.05, 0.5, 8)
    ph = rng.uniform(0.0, 2 * np.pi, 8)
    return rng, f, a, ph


def make_signal_np(n: int, seed: int = 1) -> np.ndarray:
    rng, f, a, ph = signal_params(seed)
    out = np.empty(n, dtype=np.float32)
    noise_rng = np.random.default_rng(seed + 1000)
    chunk = 1 << 22
    for s in range(0, n, chunk):
        e = min(n, s + chunk)
        t = np.arange(s, e, dtype=np.float64) / FS
        acc = np.zeros(e - s, dtype=np.float64)
        for k in range(8):
            acc += a[k] * np.sin(2 * np.pi * f[k] * t + ph[k])
        acc += 0.01 * noise_rng.standard_normal(e - s)
        out[s:e] = acc.astype(np.float32)
    return out


def make_signal_torch(n: int, seed: int = 1):
    """Same recipe, sinusoids evaluated in float64 on the GPU; noise from numpy."""
    import torch

    _, f, a, ph = signal_params(seed)
    noise = np.random.default_rng(seed + 1000).standard_normal(n).astype(np.float32)
    x = torch.from_numpy(noise).cuda().double().mul_(0.01)
    chunk = 1 << 25
    for s in range(0, n, chunk):
        e = min(n, s + chunk)
        t = torch.arange(s, e, dtype=torch.float64, device="cuda") / FS
        for k in range(8):
            x[s:e] += a[k] * torch.sin(2 * np.pi * f[k] * t + ph[k])
    return x.float().contiguous()


# --------------------------------------------------------------- clocks
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int = 0, period_ms: int = 50):
        self.samples = []
        self.proc = None
        self.index = index
        self.period_ms = period_ms

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", str(self.period_ms)], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:  # noqa: BLE001
            self.proc = None
            return
        threading.Thread(target=self._reader, daemon=True).start()

    def _reader(self):
        for line in self.proc.stdout:
            self.samples.append((time.time(), line.strip()))

    def stop(self):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:  # noqa: BLE001
                self.proc.kill()

    def summary(self, t0: float, t1: float):
        rows = [s for (ts, s) in self.samples if t0 <= ts <= t1]
        if not rows:
            rows = [s for (_, s) in self.samples]
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            p = [v.strip() for v in r.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                mx.append(float(p[2]))
            except ValueError:
                continue
            for nm, v in zip(names, p[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


# --------------------------------------------------------------- helpers
def algorithmic_bytes(n: int, geo, half_complex: bool, dense: bool) -> int:
    """Bytes the path must move: signal samples the computed frames cover + the output."""
    N = geo.n_window
    read = min(n, (geo.frames - 1) * geo.hop + N) * 4
    return int(read + geo.out_floats * 4)


FP32_LANES_PER_SM = 128       # FP32 FMA lanes per Blackwell SM
NOMINAL_SM_MAX_MHZ = 2070.0   # GB300 maximum SM clock, used when none was sampled


def fp32_pipe_bound(n_window: int, frames: int, seconds: float, sms: int, sm_mhz: float) -> dict:
    """FP32-pipe bound of the plain form, reported beside the HBM one: a
    real-input N-point FFT counted as 5*(N/2)*log2(N/2) flops per frame (the
    complex half-length FFT; the O(N) untangle, window and magnitude are left
    out), against the nominal FMA rate of `sms` SMs at `sm_mhz`."""
    half = n_window / 2
    flops = 5.0 * half * math.log2(half) * frames
    peak = sms * FP32_LANES_PER_SM * 2.0 * sm_mhz * 1e6
    achieved = flops / seconds
    return {"gflop_s": round(achieved / 1e9, 1), "peak_gflop_s": round(peak / 1e9, 1),
            "frac": round(achieved / peak, 4)}


def load_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:  # noqa: BLE001
        return 6800.0, "fallback"


def load_traffic(key: str):
    """DRAM bytes per launch from the committed ncu summary, if any."""
    p = os.path.join(ROOT, "profiles", "traffic_per_launch.txt")
    try:
        for line in open(p):
            if line.startswith(key + ":"):
                return int(float(line.split(":", 1)[1].split()[0]))
    except Exception:  # noqa: BLE001
        pass
    return None


def dist_setup():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


# --------------------------------------------------------------- CPU legs
# Samples per CPU step: the same bounded slice of the 1e8-sample signal in the
# reference arm and in cpu_baseline, so that the two numbers describe one thing.
CPU_SAMPLE = 1 << 22
# Port at the reference's cost against the reference's own OpenMP build (-O3),
# same 2^22-sample slice, measured on an 8-thread x86 host where both run:
# the port evaluates windows per sample and twiddles per butterfly, as the
# reference does, and runs 1.35x faster on 8 threads (0.91x on one).  The
# table-driven port, without that cost model, ran 2.2-2.6x faster.
PORT_VS_REFERENCE = "port at the reference's per-element cost: 1.35x the reference's own OpenMP build on 8 x86 " \
                    "threads (0.91x on one), so the port understates the reference's time"


def port_at_reference_cost(x: np.ndarray, nthreads: int) -> np.ndarray:
    """The oracle port timed with the reference's per-element work (window per
    sample, twiddle per butterfly); the oracle returns to its table form after."""
    from oracle import orc

    orc.set_reference_cost(True)
    try:
        return orc.serial_pipeline(x, HEAD_EXP, HEAD_OV, HEAD_OPTS, nthreads=nthreads)
    finally:
        orc.set_reference_cost(False)


def cpu_reference_impl():
    """The reference's OpenMP runner built from source if present, else the oracle port at the reference's cost."""
    from oracle import orc

    if orc.RefLib.available("libref_openmp_fast.so"):
        R = orc.RefLib("libref_openmp_fast.so")
        return "reference", (lambda x: R.activate(x, HEAD_EXP, HEAD_OV, HEAD_OPTS)[0]), \
            "reference OpenMP runner (StandAlone/cross_gpgpu/OpenMP) built -O3 from source"
    nt = os.cpu_count() or 1
    return "port", (lambda x: port_at_reference_cost(x, nt)), \
        "oracle port of the reference OpenMP runner (bit-exact to it), OpenMP over all host cores; " + PORT_VS_REFERENCE


def cpu_serial_baseline(sample_n: int = 1 << 21, budget_s: float = 3.0) -> dict:
    """The reference's Serial runner on one host core, on a bounded sample of
    the same workload: its own code built from source where present, else the
    oracle port of it (bit-exact) with one thread."""
    from oracle import orc

    if orc.RefLib.available("libref_serial.so"):
        R = orc.RefLib("libref_serial.so")
        kind, desc = "reference", "reference Serial runner (StandAlone/cross_gpgpu/Serial) built -O2 from source"
        fn = lambda x: R.activate(x, HEAD_EXP, HEAD_OV, HEAD_OPTS)[0]  # noqa: E731
    else:
        kind, desc = "port", "oracle port of the reference Serial runner (bit-exact to it); " + PORT_VS_REFERENCE
        fn = lambda x: port_at_reference_cost(x, 1)  # noqa: E731
    x = make_signal_np(sample_n)
    fn(x)  # warm
    times = []
    t_end = time.time() + budget_s
    while time.time() < t_end or len(times) < 3:
        t0 = time.perf_counter()
        fn(x)
        times.append(time.perf_counter() - t0)
    med = statistics.median(times)
    return {"value": sample_n / med / 1e9, "unit": METRIC, "cores": 1, "kind": kind,
            "sample": f"first {sample_n} samples of the 1e8 signal, same options; median of {len(times)} runs; "
                      f"{desc}, one thread"}


def cpu_baseline(sample_n: int = CPU_SAMPLE, budget_s: float = 12.0):
    kind, fn, desc = cpu_reference_impl()
    x = make_signal_np(sample_n)
    fn(x)  # warm
    times = []
    t_end = time.time() + budget_s
    while time.time() < t_end or len(times) < 3:
        t0 = time.perf_counter()
        fn(x)
        times.append(time.perf_counter() - t0)
    med = statistics.median(times)
    return {"value": sample_n / med / 1e9, "unit": METRIC, "cores": os.cpu_count(), "kind": kind,
            "sample": f"first {sample_n} samples of the 1e8 signal, N=1024 Hamming ov 0.5 power; "
                      f"median of {len(times)} runs; {desc}",
            "serial_1core": cpu_serial_baseline()}


def run_reference_arm(args):
    ws, rank, _ = dist_setup()
    if rank != 0:
        return
    kind, fn, desc = cpu_reference_impl()
    sample_n = CPU_SAMPLE
    x = make_signal_np(sample_n)
    for _ in range(args.warmup):
        fn(x)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        fn(x)
    dt = time.perf_counter() - t0
    v = sample_n * args.steps / dt / 1e9
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": METRIC, "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": dt / args.steps * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": "fused STFT, 1e8-sample multi-sinusoid signal, N=1024 Hamming, overlap 0.5, power "
                               "(reference layout); each step a bounded sample", "window": 1024, "overlap": 0.5,
                   "output": "power", "sample_samples": sample_n,
                   "sample_fraction": round(sample_n / 100_000_000, 4),
                   "same_config": False,
                   "note": f"each step runs the first {sample_n} samples ({sample_n / 1e6:.1f}%) of the 1e8-sample "
                           "signal; the throughput per sample is comparable, and the small slice favours the CPU "
                           "(its working set stays closer to the caches)"},
        "cpu_baseline": {"value": v, "unit": METRIC, "cores": os.cpu_count(), "kind": kind,
                         "sample": f"first {sample_n} samples per step; {desc}"},
        "e2e": {"value": v, "unit": METRIC, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


# --------------------------------------------------------------- GPU arm
def time_device(ocs, d_in, n, exp, ov, opts, d_out, cap, steps, warmup, stream):
    import torch

    for _ in range(warmup):
        ocs.activate_device(d_in, n, exp, ov, opts, d_out, cap, stream)
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(steps):
        ocs.activate_device(d_in, n, exp, ov, opts, d_out, cap, stream)
    e1.record(stream)
    e1.synchronize()
    return e0.elapsed_time(e1) / 1e3 / steps


def make_uneven_batch(count: int = 4096, seed: int = 2, lmin: int = 12, lmax: int = 22):
    """Uneven batch: lengths log-uniform in [2^lmin, 2^lmax], window {256..4096},
    overlap {0.25, 0.5, 0.75}, window {Hann, Hamming, Blackman}; signal = U(-1, 1)
    noise + a chirp from 100 Hz to 10 kHz at 48 kHz.  Built on the GPU."""
    import torch

    rng = np.random.default_rng(seed)
    lens = np.round(2.0 ** rng.uniform(lmin, lmax, count)).astype(np.int64)
    exps = rng.choice([8, 9, 10, 11, 12], count)
    ovs = rng.choice([0.25, 0.5, 0.75], count)
    wins = rng.choice(["--hanning_window", "--hamming_window", "--blackman_window"], count)
    offs = np.zeros(count + 1, dtype=np.int64)
    offs[1:] = np.cumsum((lens + 63) // 64 * 64)  # 256-byte aligned starts
    g = torch.Generator(device="cuda")
    g.manual_seed(seed)
    sig = torch.rand(int(offs[-1]), generator=g, device="cuda") * 2 - 1
    for i in range(count):
        L = int(lens[i])
        t = torch.arange(L, device="cuda", dtype=torch.float64) / FS
        T = max(L / FS, 1e-9)
        phase = 2 * np.pi * (100.0 * t + (10000.0 - 100.0) * t * t / (2 * T))
        sig[offs[i]:offs[i] + L] += torch.sin(phase).float()
    return sig, lens, offs, exps, ovs, wins


def run_batch_leg(ocs, steps: int, warmup: int, count: int = 4096):
    """One persistent, CUDA-graph-captured launch over the uneven batch vs the
    same requests launched one by one (device-resident in both cases)."""
    import torch

    sig, lens, offs, exps, ovs, wins = make_uneven_batch(count)
    geos = [ocs.geometry(int(lens[i]), int(exps[i]), float(ovs[i]), str(wins[i])) for i in range(count)]
    ooffs = np.zeros(count + 1, dtype=np.int64)
    ooffs[1:] = np.cumsum([(g.out_floats + 63) // 64 * 64 for g in geos])
    out = torch.empty(int(ooffs[-1]), device="cuda")
    items = [(sig.data_ptr() + 4 * int(offs[i]), int(lens[i]), int(exps[i]), float(ovs[i]), str(wins[i]),
              out.data_ptr() + 4 * int(ooffs[i]), geos[i].out_floats) for i in range(count)]
    reqs = ocs.make_requests(items)
    ocs.batch_prepare(reqs)
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        ocs.batch_device(reqs, s)
    torch.cuda.synchronize()
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.stream(s):
        with torch.cuda.graph(graph, stream=s):
            ocs.batch_device(reqs, s)
    for _ in range(warmup):
        graph.replay()
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(steps):
        graph.replay()
    e1.record()
    e1.synchronize()
    dt = e0.elapsed_time(e1) / 1e3 / steps
    total = int(lens.sum())
    alg = sum(4 * min(int(lens[i]), (geos[i].frames - 1) * geos[i].hop + geos[i].n_window) + 4 * geos[i].out_floats
              for i in range(count))
    # the same requests one launch each; one untimed pass first, so that the
    # autotuner has settled every (window, size class) key before timing
    for it in items:
        ocs.activate_device(it[0], it[1], it[2], it[3], it[4], it[5], it[6], s)
    torch.cuda.synchronize()
    e0.record(s)
    for it in items:
        ocs.activate_device(it[0], it[1], it[2], it[3], it[4], it[5], it[6], s)
    e1.record(s)
    e1.synchronize()
    dt_plain = e0.elapsed_time(e1) / 1e3
    peak, _ = load_peaks()
    res = {"requests": count, "samples": total, "ms_per_batch": round(dt * 1e3, 3),
           "gsamples_s": round(total / dt / 1e9, 2), "hbm_frac": round(alg / dt / 1e9 / peak, 3),
           "algorithmic_bytes": int(alg), "launches_per_batch": 1,
           "plain_per_request_gsamples_s": round(total / dt_plain / 1e9, 2),
           "speedup_vs_per_request": round(dt_plain / dt, 2),
           "workload": f"{count} signals, lengths log-uniform [2^12, 2^22], windows {{256..4096}}, overlap "
                       "{0.25,0.5,0.75}, Hann/Hamming/Blackman, noise + 100 Hz->10 kHz chirp; power, reference "
                       "layout; one CUDA-graph-captured persistent launch vs one fused launch per request"}
    del out, sig
    torch.cuda.empty_cache()
    return res


def pinned(ocs, nfloats: int):
    import ctypes

    p = ctypes.c_void_p()
    ocs._check(ocs.lib().ocs_host_alloc(ctypes.byref(p), nfloats * 4))
    return p.value, np.ctypeslib.as_array((ctypes.c_float * nfloats).from_address(p.value))


def link_bandwidth(ocs):
    """Host<->device copy bandwidth with pinned buffers (the bound of served traffic)."""
    import torch

    n = 1 << 27  # 512 MB
    hp, hx = pinned(ocs, n)
    hx[:] = 1.0
    d = torch.empty(n, device="cuda")
    h = torch.from_numpy(hx)
    for _ in range(2):
        d.copy_(h, non_blocking=True)
        h.copy_(d, non_blocking=True)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(4):
        d.copy_(h, non_blocking=True)
    torch.cuda.synchronize()
    h2d = 4 * n * 4 / (time.perf_counter() - t0) / 1e9
    t0 = time.perf_counter()
    for _ in range(4):
        h.copy_(d, non_blocking=True)
    torch.cuda.synchronize()
    d2h = 4 * n * 4 / (time.perf_counter() - t0) / 1e9
    del d, h
    ocs.lib().ocs_host_free(hp)
    return {"h2d_gbs": round(h2d, 1), "d2h_gbs": round(d2h, 1)}


def draw_served(rng, count):
    """Request draws: length log-uniform [2^14, 2^24], window/overlap/type as in the uneven batch,
    half power, half half-complex."""
    lens = np.round(2.0 ** rng.uniform(14, 24, count)).astype(np.int64)
    exps = rng.choice([8, 9, 10, 11, 12], count)
    ovs = rng.choice([0.25, 0.5, 0.75], count)
    wins = rng.choice(["--hanning_window", "--hamming_window", "--blackman_window"], count)
    half = rng.random(count) < 0.5
    opts = [(w + (" --half_complex_return" if h else "")).encode() for w, h in zip(wins, half)]
    return lens, exps, ovs, opts


def run_runner_leg(ocs, x_host, n, reps=5, warmup=2, env=None):
    """The drop-in runner executable end to end: occastft_gb300/cudaRun
    serving RequestCapnp messages over a WebSocket with the signal in POSIX
    shared memory (the reference proxy's local-runner path).  Timed per
    request from send to answer; the proxy's refill of the shared memory
    with the signal (the runner writes its result over it) is outside."""
    import socket
    import subprocess

    from occastft_gb300 import proxy, wire

    exe = os.path.join(ROOT, "occastft_gb300", "cudaRun")
    if not os.path.exists(exe):
        return {"unavailable": "cudaRun not built"}
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    penv = dict(os.environ)
    penv.update(env or {})
    p = subprocess.Popen([exe, str(port)], stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL, env=penv)
    shm = None
    ws = None
    try:
        for _ in range(600):
            try:
                ws = proxy.WsClient("127.0.0.1", port, timeout=0.2)
                break
            except OSError:
                time.sleep(0.1)
        if ws is None:
            return {"unavailable": "cudaRun did not accept a connection"}
        olen = proxy.to_overlap_length(n, HEAD_OV, 1 << HEAD_EXP)
        shm = proxy.SharedPayload("bench", olen)
        view = shm.floats()
        req = wire.Request(windowRadix=HEAD_EXP, overlapRatio=HEAD_OV, mappedID="bench", sharedMemory=shm.name,
                           dataLength=n, overlapdataLength=olen, options=HEAD_OPTS, posixFileDes=-1)
        msg = wire.encode(req)
        times = []
        for i in range(warmup + reps):
            view[:n] = x_host
            t0 = time.perf_counter()
            ws.send_binary(msg)
            op, payload = ws.recv(timeout=120)
            dt = time.perf_counter() - t0
            if op != 2 or wire.decode(payload).sharedMemory == "ERR":
                return {"unavailable": "cudaRun answered ERR"}
            if i >= warmup:
                times.append(dt)
        del view
        ms = float(np.median(times)) * 1e3
        return {"workload": f"{n} samples, window {1 << HEAD_EXP}, overlap {HEAD_OV}, '{HEAD_OPTS}', "
                            "signal and result in one POSIX shared memory region",
                "ms_per_request": round(ms, 3), "gsamples_s": round(n / ms / 1e6, 2), "requests": reps,
                "bytes_in": n * 4, "bytes_out": olen * 4,
                "note": "send-to-answer time of one request through the WebSocket protocol; the runner copies the "
                        "signal to the device in chunks and writes each part of the result back once the input "
                        "it overwrites has been copied"}
    finally:
        if ws is not None:
            try:
                ws.send_text("CLOSE_REQUEST")
                ws.recv(timeout=10)
            except Exception:  # noqa: BLE001
                pass
            ws.close()
        if shm is not None:
            shm.release()
        try:
            p.wait(timeout=20)
        except subprocess.TimeoutExpired:
            p.kill()
            p.wait()


def run_serving_leg(ocs, rates=(2000, 5000, 10000, 50000), durations=(1.0, 0.6, 0.5, 0.3), seed=3):
    """Poisson request stream against the continuous-batching server (host buffers in and out),
    and the same draws served one at a time through ocs_activate.  Each row states the bytes
    it moved each way per second against the measured host link (link_frac); the last row
    repeats the saturated stream with the power requests in the dense layout (N/2+1 bins)."""
    import ctypes

    import torch

    link = link_bandwidth(ocs)
    res = {"link": link}
    pool_n = 1 << 26
    ip, ix = pinned(ocs, pool_n)  # signal pool: noise + chirp, requests read slices of it
    g = np.random.default_rng(seed)
    ix[:] = g.uniform(-1, 1, pool_n).astype(np.float32)
    t = np.arange(pool_n, dtype=np.float64) / FS
    ix[:] += np.sin(2 * np.pi * (100.0 * t + 9900.0 * t * t / (2 * t[-1]))).astype(np.float32)
    out_n = 1 << 28
    op, _ = pinned(ocs, out_n)
    srv = ocs.Server(pool_bytes=48 << 30, max_batch=256, slots=4)
    rows = []

    def stream(rate, dur, dense_power=False):
        rng = np.random.default_rng(seed + rate)
        count = int(rate * dur)
        arrivals = np.cumsum(rng.exponential(1.0 / rate, count))
        lens, exps, ovs, opts = draw_served(rng, count)
        if dense_power:
            opts = [o if b"--half_complex_return" in o else o + b" --layout=dense" for o in opts]
        starts = rng.integers(0, pool_n - lens.max(), count)
        geos = [ocs.geometry(int(lens[i]), int(exps[i]), float(ovs[i]), opts[i].decode()) for i in range(count)]
        ooff = 0
        srv.reset_stats()
        tickets = []
        t0 = time.perf_counter()
        for i in range(count):
            while time.perf_counter() - t0 < arrivals[i]:
                pass
            of = geos[i].out_floats
            if ooff + of > out_n:
                ooff = 0
            tickets.append(srv.submit_ptr(ip + 4 * int(starts[i]), int(lens[i]), int(exps[i]), float(ovs[i]),
                                          opts[i], op + 4 * ooff, of))
            ooff += (of + 63) // 64 * 64
        for tk in tickets:
            srv.wait(tk, 600000)
        wall = time.perf_counter() - t0
        st = srv.stats()
        bin_ = 4 * int(lens.sum())
        bout = 4 * sum(int(gg.out_floats) for gg in geos)
        return {"offered_req_s": rate, "requests": count, "wall_s": round(wall, 3),
                "achieved_req_s": round(count / wall, 1),
                "gsamples_s": round(int(lens.sum()) / wall / 1e9, 2),
                "p50_ms": round(st["p50_ms"], 3), "p99_ms": round(st["p99_ms"], 3),
                "p999_ms": round(st["p999_ms"], 3), "batches": st["batches"],
                "mean_batch": round(count / max(1, st["batches"]), 1),
                "h2d_gbs": round(bin_ / wall / 1e9, 1), "d2h_gbs": round(bout / wall / 1e9, 1),
                "link_frac": {"h2d": round(bin_ / wall / 1e9 / link["h2d_gbs"], 3),
                              "d2h": round(bout / wall / 1e9 / link["d2h_gbs"], 3)},
                "layout": "dense for power requests" if dense_power else "reference"}

    try:
        for rate, dur in zip(rates, durations):
            rows.append(stream(rate, dur))
        rows.append(stream(10000, 0.5, dense_power=True))
        # plain: the same kind of draws, one synchronous ocs_activate per request
        rng = np.random.default_rng(seed + 1)
        lens, exps, ovs, opts = draw_served(rng, 400)
        starts = rng.integers(0, pool_n - lens.max(), 400)
        L = ocs.lib()
        nlen = ctypes.c_uint64()
        # untimed pass over the same draws (at most ~3 s): the autotuner settles its keys
        tw = time.perf_counter()
        for i in range(400):
            of = ocs.geometry(int(lens[i]), int(exps[i]), float(ovs[i]), opts[i].decode()).out_floats
            ocs._check(L.ocs_activate(ip + 4 * int(starts[i]), int(lens[i]), int(exps[i]), float(ovs[i]), opts[i],
                                      op, of, ctypes.byref(nlen)))
            if time.perf_counter() - tw > 3.0:
                break
        done = 0
        t0 = time.perf_counter()
        for i in range(400):
            of = ocs.geometry(int(lens[i]), int(exps[i]), float(ovs[i]), opts[i].decode()).out_floats
            ocs._check(L.ocs_activate(ip + 4 * int(starts[i]), int(lens[i]), int(exps[i]), float(ovs[i]), opts[i],
                                      op, of, ctypes.byref(nlen)))
            done += int(lens[i])
            if time.perf_counter() - t0 > 3.0:
                break
        plain = done / (time.perf_counter() - t0) / 1e9
    finally:
        srv.stop()
        ocs.lib().ocs_host_free(ip)
        ocs.lib().ocs_host_free(op)
    res["rates"] = rows
    res["plain_per_request_gsamples_s"] = round(plain, 2)
    best = max(r["gsamples_s"] for r in rows if r["layout"] == "reference")
    res["served_vs_plain"] = round(best / plain, 2)
    res["workload"] = ("Poisson arrivals; length log-uniform [2^14, 2^24], window {256..4096}, overlap "
                       "{0.25,0.5,0.75}, Hann/Hamming/Blackman, half power / half half-complex; pinned host "
                       "buffers; latency = submit to result in host memory; link_frac = bytes moved per second "
                       "each way over the measured pinned copy bandwidth")
    torch.cuda.empty_cache()
    return res


# ---------------------------------------------------------------- accuracy
# FP64 reference for the accuracy slices, written with numpy (the oracle is
# kept for the CPU baseline legs): the same framing, the window evaluated in
# float64 from its formula (OKL/kernel.okl:33-56; independent of the library's
# own table, which rounds like the reference's serial build), a float64 real
# FFT, |X| in the reference layout (N bins per frame, bins above N/2 mirrored).
def window_fp64(opts: str, N: int) -> np.ndarray:
    i = np.arange(N, dtype=np.float64)
    if "--hanning_window" in opts:
        return 0.5 * (1.0 - np.cos(2 * np.pi * i / (N - 1)))
    if "--hamming_window" in opts:
        return 0.54 - 0.46 * np.cos(2 * np.pi * i / (N - 1))
    if "--blackman_window" in opts:
        a = 2 * np.pi * i / N
        return 0.42 - 0.5 * np.cos(a) + 0.08 * np.cos(2 * a)
    return np.ones(N)


def geo_is_power_compat(opts: str) -> bool:
    """Options the float64 check covers: power in the reference layout with
    no window, Hann, Hamming or Blackman."""
    return not any(o in opts for o in ("--half_complex_return", "--layout=dense", "--serial_power",
                                      "--nuttall_window", "--blackman_nuttall_window", "--blackman_harris_window",
                                      "--flattop_window", "--gaussian_window"))


def fp64_power_reference(xs: np.ndarray, exp: int, hop: int, nf: int, opts: str) -> np.ndarray:
    N = 1 << exp
    w = window_fp64(opts, N)
    x = np.zeros((nf - 1) * hop + N)
    x[: xs.size] = xs[: x.size]
    frames = np.lib.stride_tricks.as_strided(x, shape=(nf, N), strides=(hop * 8, 8)) * w
    if "--remove_dc" in opts:
        frames = frames - frames.mean(axis=1, keepdims=True)
    half = np.abs(np.fft.rfft(frames, axis=1))
    full = np.concatenate([half, half[:, 1:N // 2][:, ::-1]], axis=1)
    return full.reshape(-1)


def rel_l2(a, b) -> float:
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def max_db_error(a, b, floor_rel: float = 1e-6) -> float:
    a = np.abs(np.asarray(a, np.float64))
    b = np.abs(np.asarray(b, np.float64))
    fl = max(float(b.max()) * floor_rel, 1e-300)
    return float(np.max(np.abs(20 * np.log10(np.maximum(a, fl)) - 20 * np.log10(np.maximum(b, fl)))))


def run_tc_leg(ocs, x, n, d_out, stream, steps=10, warmup=3):
    """Windows 256..4096, Hann, overlap 0.75 on the 1e8-sample signal: plain FP32
    against the tensor-core split-precision form, with accuracy vs FP64."""
    import torch

    peak, _ = load_peaks()
    rows = []
    # overlap 0.75 writes ~4 floats per input sample
    d_out = torch.empty(max(ocs.geometry(n, e, 0.75, "").out_floats for e in (8, 9, 10, 11, 12)), device="cuda")
    for exp in (8, 9, 10, 11, 12):
        for prec in ("fp32", "tc-fp16", "tc-bf16x3", "tc-bf16x2"):
            opts = "--hanning_window" + (" --precision=" + prec if prec != "fp32" else "")
            try:
                g = ocs.geometry(n, exp, 0.75, opts)
            except ocs.OcsError:
                continue
            if g.out_floats > d_out.numel():
                continue
            dt = time_device(ocs, x, n, exp, 0.75, opts, d_out, d_out.numel(), steps, warmup, stream)
            # accuracy on 300 frames from the middle of the signal
            nf = 300
            f0 = g.qt // 2
            s0 = f0 * g.hop
            xs = x[s0:s0 + (nf - 1) * g.hop + g.n_window].cpu().numpy()
            got = d_out[f0 * g.n_window:(f0 + nf) * g.n_window].cpu().numpy()
            ref = fp64_power_reference(xs, exp, g.hop, nf, "--hanning_window")
            b = algorithmic_bytes(n, g, False, False)
            rows.append({"N": 1 << exp, "precision": prec, "gsamples_s": round(n / dt / 1e9, 2),
                         "ms": round(dt * 1e3, 4), "hbm_frac": round(b / dt / 1e9 / peak, 3),
                         "rel_l2_vs_fp64": float("%.3g" % rel_l2(got, ref)),
                         "max_db_vs_fp64": round(max_db_error(got, ref), 4)})
    del d_out
    torch.cuda.empty_cache()
    return {"rows": rows, "workload": "1e8-sample multi-sinusoid signal, Hann, overlap 0.75, power (reference "
                                      "layout); tc-* = tcgen05 four-step FFT with split operands: fp16 hi/lo, bf16 "
                                      "hi/mid/lo (6 products), bf16 hi/lo (for reference); accuracy vs a float64 "
                                      "numpy FFT of 300 frames"}


def cpu_baseline_subprocess() -> dict:
    """cpu_baseline in a fresh process started before this one initialises
    CUDA: no GPU-side threads, pinned buffers or earlier legs share the host
    cores with it, as none do in the reference arm's process."""
    r = subprocess.run([sys.executable, os.path.abspath(__file__), "--cpu-leg", "--n", str(N_SAMPLES),
                        "--exp", str(HEAD_EXP), "--overlap", str(HEAD_OV), "--options=" + HEAD_OPTS],
                       capture_output=True, text=True, timeout=600)
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    if r.returncode != 0 or not lines:
        return {"unavailable": f"CPU leg failed (rc {r.returncode}): {r.stderr.strip()[-300:]}"}
    return json.loads(lines[-1])


def run_ours(args):
    ws, rank, local = dist_setup()
    # the CPU baseline runs first, on rank 0 at N=1 only, before CUDA starts
    cpu = cpu_baseline_subprocess() if (rank == 0 and ws == 1 and not args.no_cpu) else None

    import torch

    import occastft_gb300 as ocs

    torch.cuda.set_device(local)
    if ws > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    ocs.Runner(local)
    stream = torch.cuda.current_stream()
    n = N_SAMPLES
    x = make_signal_torch(n)
    geo = ocs.geometry(n, HEAD_EXP, HEAD_OV, HEAD_OPTS)
    # room for the largest output of the sweep (windows up to 2^22, overlap 0.5)
    cap = max([geo.out_floats] + [ocs.geometry(n, e, 0.5, "").out_floats for e in range(6, 23)])
    d_out = torch.empty(cap, device="cuda")
    peak, peak_kind = load_peaks()

    def barrier():
        torch.cuda.synchronize()
        if ws > 1:
            import torch.distributed as dist

            dist.barrier()
            torch.cuda.synchronize()

    # warm-up
    for _ in range(args.warmup):
        ocs.activate_device(x, n, HEAD_EXP, HEAD_OV, HEAD_OPTS, d_out, geo.out_floats, stream)
    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.3)
    barrier()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    t_start = time.time()
    e0.record(stream)
    for _ in range(args.steps):
        ocs.activate_device(x, n, HEAD_EXP, HEAD_OV, HEAD_OPTS, d_out, geo.out_floats, stream)
    e1.record(stream)
    e1.synchronize()
    t_stop = time.time()
    barrier()
    elapsed = e0.elapsed_time(e1) / 1e3
    if ws > 1:
        import torch.distributed as dist

        t = torch.tensor([elapsed], device="cuda", dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        elapsed = float(t.item())
    time.sleep(0.1)
    clocks.stop()
    clk = clocks.summary(t_start, t_stop)
    per_step = elapsed / args.steps
    value = n * ws / per_step / 1e9
    alg = algorithmic_bytes(n, geo, False, False)
    achieved = alg / per_step / 1e9

    # accuracy on a slice of frames: float64 FFT of the same samples
    acc = {}
    if rank == 0:
        f0 = geo.qt // 3
        nf = max(1, min(400, geo.qt - f0))
        s0 = f0 * geo.hop
        xs = x[s0:s0 + (nf - 1) * geo.hop + geo.n_window].cpu().numpy()
        got = d_out[f0 * geo.n_window:(f0 + nf) * geo.n_window].cpu().numpy()
        if not geo_is_power_compat(HEAD_OPTS):
            acc = {"skipped": "float64 check covers power in the reference layout"}
        else:
            ref = fp64_power_reference(xs, HEAD_EXP, geo.hop, nf, HEAD_OPTS)
            acc = {"rel_l2_vs_fp64": rel_l2(got, ref), "max_db_vs_fp64": max_db_error(got, ref),
                   "frames_checked": nf}

    # end to end through the public host API (pinned host buffers)
    e2e = None
    if not args.no_e2e:
        import ctypes

        L = ocs.lib()
        hin = ctypes.c_void_p()
        hout = ctypes.c_void_p()
        ocs._check(L.ocs_host_alloc(ctypes.byref(hin), n * 4))
        ocs._check(L.ocs_host_alloc(ctypes.byref(hout), geo.out_floats * 4))
        hx = np.ctypeslib.as_array((ctypes.c_float * n).from_address(hin.value))
        hx[:] = x.cpu().numpy()
        nlen = ctypes.c_uint64()
        e2e_steps = max(3, min(args.steps, 30))
        for _ in range(max(3, args.warmup)):
            ocs._check(L.ocs_activate(hin, n, HEAD_EXP, HEAD_OV, HEAD_OPTS.encode(), hout, geo.out_floats,
                                      ctypes.byref(nlen)))
        barrier()
        t0 = time.perf_counter()
        for _ in range(e2e_steps):
            ocs._check(L.ocs_activate(hin, n, HEAD_EXP, HEAD_OV, HEAD_OPTS.encode(), hout, geo.out_floats,
                                      ctypes.byref(nlen)))
        dt = (time.perf_counter() - t0) / e2e_steps
        e2e = {"value": n * ws / dt / 1e9, "unit": METRIC, "h2d_bytes_per_step": n * 4,
               "d2h_bytes_per_step": int(geo.out_floats * 4), "ms_per_step": dt * 1e3, "steps": e2e_steps,
               "api": "ocs_activate (C ABI, host buffers from ocs_host_alloc)"}
        L.ocs_host_free(hin)
        L.ocs_host_free(hout)

    # the rest of the config: window sweep, device-resident
    sweep = []
    if rank == 0 and not args.no_sweep:
        sms = torch.cuda.get_device_properties(local).multi_processor_count
        pipe_mhz = clk.get("sm_max_mhz") or NOMINAL_SM_MAX_MHZ
        for exp in range(6, 23):
            for wname in ("hamming", "blackman"):
                for out_kind in ("power", "half_complex"):
                    opts = f"--{wname}_window" + (" --half_complex_return" if out_kind == "half_complex" else "")
                    g = ocs.geometry(n, exp, 0.5, opts)
                    dt = time_device(ocs, x, n, exp, 0.5, opts, d_out, d_out.numel(), 10, 3, stream) \
                        if g.out_floats <= d_out.numel() else None
                    if dt is None:
                        continue
                    b = algorithmic_bytes(n, g, out_kind == "half_complex", False)
                    sweep.append({"N": 1 << exp, "window": wname, "output": out_kind,
                                  "gsamples_s": round(n / dt / 1e9, 2), "ms": round(dt * 1e3, 4),
                                  "hbm_frac": round(b / dt / 1e9 / peak, 3),
                                  "fp32_pipe": fp32_pipe_bound(g.n_window, g.frames, dt, sms, pipe_mhz)})

    # cuFFT reference point (same GPU): batched R2C over pre-framed data
    cufft = None
    if rank == 0 and not args.no_sweep:
        N = 1 << HEAD_EXP
        frames = x.unfold(0, N, geo.hop).contiguous()
        win = torch.from_numpy(ocs.window_table(2, N)).cuda()
        for _ in range(3):
            torch.fft.rfft(frames, dim=1)
        torch.cuda.synchronize()
        a0 = torch.cuda.Event(enable_timing=True)
        a1 = torch.cuda.Event(enable_timing=True)
        a0.record()
        for _ in range(10):
            torch.fft.rfft(frames, dim=1)
        a1.record()
        a1.synchronize()
        t_fft = a0.elapsed_time(a1) / 1e3 / 10
        a0.record()
        for _ in range(10):
            torch.fft.rfft(x.unfold(0, N, geo.hop) * win, dim=1).abs()
        a1.record()
        a1.synchronize()
        t_pipe = a0.elapsed_time(a1) / 1e3 / 10
        cufft = {"rfft_only_ms": round(t_fft * 1e3, 4), "rfft_only_gsamples_s": round(n / t_fft / 1e9, 2),
                 "torch_pipeline_ms": round(t_pipe * 1e3, 4),
                 "torch_pipeline_gsamples_s": round(n / t_pipe / 1e9, 2),
                 "note": "cuFFT via torch.fft.rfft over frames already materialised (rfft_only) and a torch "
                         "unfold*window->rfft->abs pipeline (N/2+1 bins), same GPU"}
        del frames

    tc = None
    if rank == 0 and not args.no_sweep:
        tc = run_tc_leg(ocs, x, n, d_out, stream)
    batch = None
    if rank == 0 and not args.no_batch:
        batch = run_batch_leg(ocs, steps=5, warmup=3, count=args.batch_count)
    serving = None
    if rank == 0 and not args.no_serve:
        serving = run_serving_leg(ocs)
    runner_exe = None
    if rank == 0 and not args.no_serve:
        runner_exe = run_runner_leg(ocs, x.cpu().numpy(), n)

    if rank != 0:
        if ws > 1:
            import torch.distributed as dist

            dist.barrier()
            dist.destroy_process_group()
        return

    headline = (n == 100_000_000 and HEAD_EXP == 10 and HEAD_OV == 0.5 and HEAD_OPTS == "--hamming_window")
    # the committed ncu traffic figure belongs to the headline workload only
    traffic = load_traffic(f"stft_pair_e{HEAD_EXP}_hamming_power_1e8") if headline else None
    if headline:
        workload = ("fused STFT of a 1e8-sample float32 signal (8 seeded sinusoids + N(0,0.01^2), fs 48 kHz), "
                    "window 1024 Hamming, overlap 0.5, power in the reference layout (qt x N floats)")
    else:
        workload = (f"fused STFT of a {n}-sample float32 signal (8 seeded sinusoids + N(0,0.01^2), fs 48 kHz), "
                    f"window {1 << HEAD_EXP}, overlap {HEAD_OV}, options '{HEAD_OPTS}'")
    line = {
        "metric": METRIC, "value": round(value, 3), "unit": METRIC, "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(per_step * 1e3, 5), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": workload, "samples": n, "window": 1 << HEAD_EXP, "overlap": HEAD_OV,
                   "options": HEAD_OPTS, "frames": geo.qt, "l2_flush": "not needed: 1.2 GB per step > 129 MB L2",
                   "parallelism": f"replica x{ws} (frames shard with no exchange)"},
        "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                     "frac": round(achieved / peak, 4), "traffic": traffic, "algorithmic_bytes": alg,
                     "peak_source": f"MEASURED_PEAKS.json hbm_gbs ({peak_kind})"},
        "e2e": e2e,
        "gpu_launches": args.steps,
        "clocks": clk,
        "accuracy": acc,
        "cpu_baseline": cpu,
        "sweep": sweep,
        "cufft_reference": cufft,
        "tensor_core": tc,
        "uneven_batch": batch,
        "serving": serving,
        "runner_executable": runner_exe,
    }
    print(json.dumps(line))
    if ws > 1:
        import torch.distributed as dist

        dist.barrier()
        dist.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-sweep", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-batch", action="store_true")
    ap.add_argument("--batch-count", type=int, default=4096, help="requests in the uneven batch (profiling runs use fewer)")
    ap.add_argument("--no-serve", action="store_true")
    ap.add_argument("--n", type=int, default=N_SAMPLES, help="signal samples (profiling runs use fewer)")
    ap.add_argument("--exp", type=int, default=HEAD_EXP)
    ap.add_argument("--options", default=HEAD_OPTS)
    ap.add_argument("--overlap", type=float, default=HEAD_OV)
    ap.add_argument("--cpu-leg", action="store_true", help=argparse.SUPPRESS)
    ap.add_argument("--cpu-sample", type=int, default=0, help=argparse.SUPPRESS)
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    globals().update(N_SAMPLES=args.n, HEAD_EXP=args.exp, HEAD_OPTS=args.options, HEAD_OV=args.overlap)
    if args.cpu_leg:
        if args.cpu_sample:
            print(json.dumps(cpu_baseline(sample_n=args.cpu_sample, budget_s=0.5)))
        else:
            print(json.dumps(cpu_baseline()))
    elif args.impl == "reference":
        run_reference_arm(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
