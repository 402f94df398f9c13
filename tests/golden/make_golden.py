"""Generates the golden vectors in tests/golden/ from the reference's OWN code.

Run here, where the reference checkout exists and oracle/build_ref.sh has
compiled its Serial runner into oracle/_ref/libref_serial.so:

    bash oracle/build_ref.sh && python tests/golden/make_golden.py

Every case records the seeded input recipe, the reference's status string,
geometry, the SHA-256 of the full float32 output and either the full output
(small cases) or a few frames of it (the 2^20-sample C0 case).  The reference
has no test vectors of its own; these are produced by executing it.
"""
from __future__ import annotations

import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import orc  # noqa: E402


def signal(seed: int, n: int) -> np.ndarray:
    return np.random.default_rng(seed).uniform(-1.0, 1.0, n).astype(np.float32)


CASES = []
# (name, seed, n, exp, overlap, options)
_opts = [
    "--hanning_window --remove_dc",
    "--hamming_window",
    "--blackman_window --half_complex_return",
    "--nuttall_window --remove_dc --half_complex_return",
    "--blackman_nuttall_window",
    "--blackman_harris_window --remove_dc",
    "--flattop_window --half_complex_return",
    "--gaussian_window=4.312345<<sigma --remove_dc",
    "",
    "--hanning_window --remove_dc --half_complex_return",
]
_ovs = [0.5, 0.0, 0.75, 0.25, 0.3, 0.5, 0.6, 0.5, 0.125, 0.5]
for e in range(6, 13):
    for j in range(3):
        k = (e * 3 + j) % len(_opts)
        n = int(np.random.default_rng(100 + e * 10 + j).integers(3 * (1 << e), 6000 + 3 * (1 << e)))
        CASES.append((f"e{e}_{j}", 1000 + e * 10 + j, n, e, _ovs[k], _opts[k]))
for e in (13, 14, 15):
    for j, (ov, op) in enumerate([(0.5, "--hanning_window --remove_dc"),
                                  (0.75, "--blackman_window --half_complex_return")]):
        n = (1 << e) + 977 * (j + 1)
        CASES.append((f"e{e}_{j}", 2000 + e * 10 + j, n, e, ov, op))
# ragged / edge shapes
CASES.append(("short_signal", 7, 100, 6, 0.5, "--hanning_window --remove_dc"))
CASES.append(("one_sample", 8, 1, 6, 0.5, "--hamming_window"))
CASES.append(("gap_hop", 9, 2000, 7, -0.5, "--hanning_window"))
CASES.append(("odd_hop", 10, 3001, 8, 0.5 + 1.0 / 256, "--blackman_window --remove_dc"))
# error statuses
CASES.append(("exp5", 11, 1000, 5, 0.5, "--hanning_window"))
CASES.append(("gauss_empty_sigma", 12, 1000, 7, 0.5, "--gaussian_window=4<<sigma"))
CASES.append(("gauss_negative", 13, 1000, 7, 0.5, "--gaussian_window=-2.0<<sigma"))

C0 = ("c0_plain_cpu", 0, 1 << 20, 10, 0.5, "--hanning_window --remove_dc")
C0_FRAMES = [0, 1, 2, 1000, 2046, 2047, 2048]

WINDOW_CASES = [(k, e) for k in ("hanning", "hamming", "blackman", "nuttall", "blackman_nuttall",
                                 "blackman_harris", "flattop") for e in (6, 10, 12, 15)]
WINDOW_CASES += [("gaussian", 8), ("gaussian", 12)]


def main():
    ref = orc.RefLib("libref_serial.so")
    manifest = {"generator": "tests/golden/make_golden.py", "reference": "Serial runner (oracle/build_ref.sh)",
                "signal": "np.random.default_rng(seed).uniform(-1, 1, n).astype(float32)", "cases": [],
                "windows": []}
    arrays = {}
    for name, seed, n, e, ov, op in CASES:
        x = signal(seed, n)
        rec = {"name": name, "seed": seed, "n": n, "exp": e, "overlap": ov, "options": op}
        if e < 6:
            # the reference's Default_Pipeline runs the overlap before checking
            # the exponent; reading its status is enough here
            rec["status"] = "Operation not supported"
            manifest["cases"].append(rec)
            continue
        out, st = ref.activate(x, e, ov, op)
        qt, hop, ofull, ohalf = ref.geometry(n, e, ov)
        rec.update({"status": st, "qt": qt, "hop": hop, "ofull": ofull, "ohalf": ohalf})
        if out is not None:
            rec["sha256"] = hashlib.sha256(out.tobytes()).hexdigest()
            arrays[name] = out
        manifest["cases"].append(rec)
    name, seed, n, e, ov, op = C0
    x = signal(seed, n)
    out, st = ref.activate(x, e, ov, op)
    qt, hop, ofull, ohalf = ref.geometry(n, e, ov)
    N = 1 << e
    manifest["c0"] = {"name": name, "seed": seed, "n": n, "exp": e, "overlap": ov, "options": op, "status": st,
                      "qt": qt, "hop": hop, "ofull": ofull, "ohalf": ohalf,
                      "sha256": hashlib.sha256(out.tobytes()).hexdigest(), "frames": C0_FRAMES}
    arrays["c0_frames"] = np.stack([out[f * N:(f + 1) * N] for f in C0_FRAMES])
    for kind, e in WINDOW_CASES:
        N = 1 << e
        sigma = 0.312345 if kind == "gaussian" else -1.0
        x = signal(77, 3 * N)
        w = ref.overlap_window(x, e, 0.5, kind, sigma=sigma)
        key = f"win_{kind}_{e}"
        # frame 0 is the full window applied to x[0:N]
        arrays[key] = w[:N]
        manifest["windows"].append({"key": key, "kind": kind, "exp": e, "sigma": sigma, "seed": 77, "n": 3 * N})
    np.savez_compressed(os.path.join(HERE, "reference_outputs.npz"), **arrays)
    with open(os.path.join(HERE, "manifest.json"), "w") as f:
        json.dump(manifest, f, indent=1)
    print("wrote", len(arrays), "arrays")


if __name__ == "__main__":
    main()
