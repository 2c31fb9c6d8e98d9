"""Batched form: many independent lattices in one work-list per step, against
the same jobs run one at a time through the plain single-lattice kernel.

Workload (512 jobs by default): width and height log-uniform in [256, 4096]
rounded to multiples of 64; model uniform over HPP, FHP-I, FHP-II, FHP-III;
geometry uniform over periodic, pipe (walls plus a forcing column at x = 8,
flip probability 0.01) and a no-slip disc (radius H/16 at x = W/8, no walls);
occupation Bernoulli p ~ U(0.1, 0.4) per channel; seed 1000 + job index;
1000 steps each.  Every job must end in the same state both ways.

    python -m lgca_gb300.batched [--jobs 512] [--steps 1000] [--no-tune]
"""
from __future__ import annotations

import argparse
import hashlib
import json
import math
import time

import numpy as np

import lgca_gb300 as gpu
from lgca_gb300.autotune import Autotuner

GEOMETRIES = ("periodic", "pipe", "disc")


def round64(v: float) -> int:
    return max(64, int(round(v / 64.0)) * 64)


def make_jobs(n: int = 512, lo: int = 256, hi: int = 4096, rng_seed: int = 4):
    rng = np.random.default_rng(rng_seed)
    jobs = []
    for i in range(n):
        W = round64(math.exp(rng.uniform(math.log(lo), math.log(hi))))
        H = round64(math.exp(rng.uniform(math.log(lo), math.log(hi))))
        jobs.append(dict(index=i, model=int(rng.integers(4)), W=W, H=H,
                         geometry=GEOMETRIES[int(rng.integers(3))],
                         p=float(rng.uniform(0.1, 0.4)), seed=1000 + i))
    return jobs


def build(job) -> "gpu.GpuLattice":
    W, H = job["W"], job["H"]
    L = gpu.GpuLattice(job["model"], W, H, seed=job["seed"])
    if job["geometry"] == "pipe":
        L.apply_bc_pipe()
        L.set_forcing_column(8, 0.01)
    elif job["geometry"] == "disc":
        L.paint_cells(gpu.SHAPE_DISC, gpu.SOLID_NO_SLIP, W // 8, H // 2, max(1, H // 16))
    L.init_random(job["p"], job["p"])
    return L


def digest(L: "gpu.GpuLattice") -> str:
    return hashlib.sha256(L.download().tobytes()).hexdigest()


def run_batched(jobs, steps: int, tune: bool = True, tuner: Autotuner | None = None):
    lattices = [build(j) for j in jobs]
    tuned = {}
    if tune:
        tuner = tuner or Autotuner()
        tuned = tuner.tune_batch_members(lattices)
    B = gpu.GpuBatch()
    for L in lattices:
        B.add(L)
    for L in lattices:
        L.sync()
    t0 = time.perf_counter()
    B.step(steps)
    B.sync()
    dt = time.perf_counter() - t0
    hashes = [digest(L) for L in lattices]
    B.close()
    for L in lattices:
        L.close()
    return dt, hashes, tuned


def run_one_by_one(jobs, steps: int):
    total, hashes = 0.0, []
    for j in jobs:
        L = build(j)
        L.set_kernel_variant(0)  # the plain kernel: one step per pass, its fastest form
        L.sync()
        t0 = time.perf_counter()
        L.collide_and_propagate(steps)
        L.sync()
        total += time.perf_counter() - t0
        hashes.append(digest(L))
        L.close()
    return total, hashes


def compare(n_jobs: int = 512, steps: int = 1000, tune: bool = True) -> dict:
    jobs = make_jobs(n_jobs)
    sites = sum(j["W"] * j["H"] for j in jobs)
    tb, hb, tuned = run_batched(jobs, steps, tune)
    ts, hs = run_one_by_one(jobs, steps)
    return {"jobs": n_jobs, "steps": steps, "sites": sites,
            "batched_s": tb, "one_by_one_s": ts,
            "batched_gsite_updates_s": sites * steps / tb / 1e9,
            "one_by_one_gsite_updates_s": sites * steps / ts / 1e9,
            "speedup": ts / tb, "bit_exact": hb == hs,
            "tuned": {k: list(v) for k, v in tuned.items()}, "final_sha": hb}


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--jobs", type=int, default=512)
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--no-tune", action="store_true")
    a = ap.parse_args(argv)
    gpu.build()
    r = compare(a.jobs, a.steps, not a.no_tune)
    r.pop("final_sha")
    print(json.dumps(r))


if __name__ == "__main__":
    main()
