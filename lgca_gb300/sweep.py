"""Roofline sweep of the plain and temporally blocked kernels.

Workload: fully periodic lattices, no obstacles; models HPP, FHP-I, FHP-II,
FHP-III; sizes 4096x4096, 16384x8192 and 32768x16384; Bernoulli occupation
p in {0.1, 0.5} on every channel, seed 3; steps per HBM pass k in {1, 2, 4,
8} -- k = 1 with the one-step kernel (variant 5) and, where the lattice fits
it, the resident kernel (variant 6: every step of the run on chip, no HBM
traffic between steps), k > 1 with the register wavefront (variant 2; FHP
up to k = 4) and with shared-memory tiles (variant 3).
Each case runs `steps` steps (default 2000) timed with CUDA events on the
lattice's stream after a warm-up.

Algorithmic HBM bytes per site-step: 2 * D / 8 / k (D = 4, 6, 7, 7 planes
read and written once per pass).  `gbs` is those bytes over the measured
time, `frac` the fraction of the measured copy bandwidth (MEASURED_PEAKS.json
at the repository root, else 6800 GB/s).  Results are bit-exact with the
reference: tests/test_gpu_step.py checks every model, variant and depth of
this sweep on a 1024x1024 lattice against the oracle.

    python -m lgca_gb300.sweep [--steps 2000] [--sizes 4096x4096 ...] [--json out.json]
"""
from __future__ import annotations

import argparse
import json
import os

import lgca_gb300 as gpu

SIZES = [(4096, 4096), (16384, 8192), (32768, 16384)]
DEPTHS = [1, 2, 4, 8]
PROBS = [0.1, 0.5]
NUM_DIR = {0: 4, 1: 6, 2: 7, 3: 7}


def hbm_peak() -> tuple[float, str]:
    path = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))),
                        "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def time_case(L, torch, steps: int, depth: int) -> float:
    """Seconds per lattice step over `steps` steps (a multiple of depth)."""
    s = torch.cuda.ExternalStream(L.stream_ptr())
    L.collide_and_propagate(2 * depth)  # warm-up (kernel load, caches)
    L.sync()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(s)
    L.collide_and_propagate(steps)
    e1.record(s)
    e1.synchronize()
    return e0.elapsed_time(e1) / 1e3 / steps


def sweep(sizes=SIZES, models=(0, 1, 2, 3), probs=PROBS, depths=DEPTHS, steps: int = 2000):
    import torch

    peak, kind = hbm_peak()
    rows = []
    for W, H in sizes:
        for model in models:
            L = gpu.GpuLattice(model, W, H, seed=3)
            for p in probs:
                L.init_random(p, p)
                for depth in depths:
                    for variant in ((5, 6) if depth == 1 else (2, 3)):
                        if variant == 2 and depth == 8 and model != 0:
                            continue  # the FHP wavefront holds at most 4 time levels
                        L.set_kernel_variant(variant)
                        L.set_temporal_depth(depth)
                        if variant == 6 and L.step_plan(steps)[0] != 6:
                            continue  # the lattice does not fit the resident kernel
                        n = max(depth, steps // depth * depth)
                        t = time_case(L, torch, n, depth)
                        bytes_site = 2 * NUM_DIR[model] / 8 / depth
                        gbs = W * H * bytes_site / t / 1e9
                        rows.append({"W": W, "H": H, "model": model, "p": p, "depth": depth,
                                     "kernel": {5: "one-step", 6: "resident", 2: "wavefront",
                                                3: "tiles"}[variant],
                                     "ms_per_step": t * 1e3, "gsite_updates_s": W * H / t / 1e9,
                                     "gbs": gbs, "frac": gbs / peak, "peak_gbs": peak,
                                     "peak_kind": kind})
                        print(json.dumps(rows[-1]), flush=True)
            L.close()
    return rows


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--sizes", nargs="+", default=[f"{w}x{h}" for w, h in SIZES])
    ap.add_argument("--models", type=int, nargs="+", default=[0, 1, 2, 3])
    ap.add_argument("--json", default=None, help="also write all rows to this file")
    a = ap.parse_args(argv)
    gpu.build()
    sizes = [tuple(int(v) for v in s.split("x")) for s in a.sizes]
    rows = sweep(sizes, a.models, steps=a.steps)
    if a.json:
        with open(a.json, "w") as f:
            json.dump(rows, f, indent=1)


if __name__ == "__main__":
    main()
