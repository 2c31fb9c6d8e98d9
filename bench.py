"""Benchmark of the lattice-gas hot path on GB300.

Workload (one "step" of this benchmark): the FHP-III Karman vortex street on
an 8192 x 2048 lattice -- pipe walls on the first and last row, a no-slip disc
of radius 128 centred at (1024, 1024), a forcing column at x = 16 with flip
probability 0.02, Bernoulli(0.3) occupation of all seven channels from seed 2
-- advanced by 100 lattice steps followed by the 32 x 32 integer block sums of
the coarse-graining.  `--steps 100` is the whole 10000-step run.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Prints one JSON line (rank 0).  `value` is site updates per second of the
whole job with the lattice resident in HBM; `e2e` is the same metric through
the C ABI with the state uploaded from / downloaded to pinned host memory
every step; `roofline` is the step kernel against its bound (the resident
kernel that holds the lattice on chip: instruction issue; `roofline_gate` is
the one-step kernel on a lattice 16x larger against the measured HBM copy
bandwidth); `cpu_baseline` is the CPU oracle (the reference algorithm in C,
OpenMP) on this host's cores.  Multi-GPU (torchrun) runs one independent
lattice per rank (weak scaling; no collective on the data path).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

W_K, H_K = 8192, 2048
STEPS_PER_CHUNK = 100
BLOCK = 32
MODEL = 3  # FHP-III
METRIC = "GSite-updates/s & %HBM roofline; batched/served vs plain jobs/s, p50/p99 lat"
UNIT = "GSite-updates/s"
WORKLOAD = ("FHP-III Karman vortex street 8192x2048: walls on rows 0 and 2047, no-slip disc r=128 "
            "at (1024,1024), forcing column x=16 p=0.02, Bernoulli p=0.3 (moving and rest) seed 2; "
            "bench step = 100 lattice steps + 32x32 integer block sums")
SMI_FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def profiled_value(name, key="traffic_bytes_per_launch"):
    """A per-launch figure from a committed ncu summary (a line `key: N`, e.g.
    DRAM bytes or warp instructions per launch), or None."""
    path = os.path.join(ROOT, "profiles", name)
    try:
        for line in open(path):
            if line.strip().startswith(key + ":"):
                return float(line.split(":", 1)[1])
    except OSError:
        pass
    return None


def profiled_traffic(name):
    return profiled_value(name, "traffic_bytes_per_launch")


class ClockSampler:
    """nvidia-smi clock / throttle samples during the timed region."""

    def __init__(self, index):
        self.index = index
        self.proc = None
        # raw samples go to $LGCA_CLOCKS_CSV when set, else to a temporary file
        self.path = os.environ.get("LGCA_CLOCKS_CSV") or os.path.join(
            tempfile.gettempdir(), f"lgca_clocks_{index}.csv")

    def __enter__(self):
        try:
            os.makedirs(os.path.dirname(self.path), exist_ok=True)
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={SMI_FIELDS}", "--format=csv",
                 "-lms", "200"], stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.f.close()

    def summary(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm, smax, reasons = [], None, set()
        names = ["active", "hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown",
                 "sw_power_cap"]
        try:
            for line in open(self.path):
                parts = [p.strip() for p in line.split(",")]
                if len(parts) < 9 or not parts[1].split()[0].isdigit():
                    continue
                sm.append(int(parts[1].split()[0]))
                smax = int(parts[2].split()[0])
                for n, v in zip(names[1:], parts[5:9]):
                    if v.lower().startswith("active"):
                        reasons.add(n)
        except OSError:
            pass
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": smax, "reasons": sorted(reasons), "samples": 0}
        loaded = [s for s in sm if s > 0.5 * (smax or max(sm))] or sm
        return {"sm_mhz": statistics.median(loaded), "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


def karman_types():
    from lgca_gb300 import geometry as G
    return G.disc(W_K, H_K, 1024, 1024, 128)


def cpu_baseline(budget_s=12.0):
    """The oracle (reference algorithm in C, OpenMP on all host threads) on a
    bounded sample of the same workload: lattice steps of the 8192x2048
    Karman lattice until ~budget_s seconds have been spent."""
    from oracle import oracle as O
    O.build(ref=False)
    types = karman_types()
    st = O.init_bernoulli(MODEL, W_K, H_K, types, seed=2, p_move=0.3, p_rest=0.3)
    O.run(MODEL, st, 1, types=types, seed=2, force_x=16, force_p=0.02)  # warm-up
    steps, t0 = 0, time.perf_counter()
    cur = st
    while time.perf_counter() - t0 < budget_s and steps < 400:
        cur = O.run(MODEL, cur, 2, types=types, seed=2, t0=steps, force_x=16, force_p=0.02)
        steps += 2
    dt = time.perf_counter() - t0
    return {"value": W_K * H_K * steps / dt / 1e9, "unit": UNIT, "cores": O.lib().oracle_threads(),
            "kind": "port",
            "sample": f"{steps} lattice steps of the 8192x2048 FHP-III Karman lattice (incl. forcing)"}


def run_reference(args):
    ws, rank, _ = dist_env()
    if rank != 0:
        return
    from oracle import oracle as O
    O.build(ref=False)
    types = karman_types()
    st = O.init_bernoulli(MODEL, W_K, H_K, types, seed=2, p_move=0.3, p_rest=0.3)
    per_step = 2  # lattice steps per benchmark step: a bounded sample of the 100-step chunk
    t = 0
    for _ in range(args.warmup):
        st = O.run(MODEL, st, per_step, types=types, seed=2, t0=t, force_x=16, force_p=0.02)
        t += per_step
    t0 = time.perf_counter()
    for _ in range(args.steps):
        st = O.run(MODEL, st, per_step, types=types, seed=2, t0=t, force_x=16, force_p=0.02)
        t += per_step
    dt = time.perf_counter() - t0
    value = W_K * H_K * per_step * args.steps / dt / 1e9
    cores = O.lib().oracle_threads()
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt / args.steps * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u8",
        "data": "synthetic",
        "config": {"workload": WORKLOAD, "reference_step": f"{per_step} lattice steps (bounded sample)",
                   "parallelism": f"cpu x{cores} threads"},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": f"{per_step * args.steps} lattice steps of the 8192x2048 FHP-III "
                                   "Karman lattice"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def gate_measurement(gpu, torch, hbm_peak):
    """Plain single-lattice kernel on the 32768x16384 FHP-III periodic lattice
    (the roofline gate): HBM bytes per step = 2 * 7/8 B per site."""
    W, H = 32768, 16384
    with gpu.GpuLattice(MODEL, W, H, seed=3) as L:
        L.init_random(0.5, 0.5)
        L.set_kernel_variant(5)  # one step per pass (the automatic choice blocks 2 steps here)
        s = torch.cuda.ExternalStream(L.stream_ptr())
        L.collide_and_propagate(3)
        n = 30
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        L.sync()
        e0.record(s)
        L.collide_and_propagate(n)
        e1.record(s)
        e1.synchronize()
        ms = e0.elapsed_time(e1) / n
    bytes_step = W * H * 2 * 7 / 8
    gbs = bytes_step / (ms * 1e-3) / 1e9
    return {"workload": "FHP-III periodic 32768x16384, plain kernel, 1 step per pass",
            "ms_per_launch": ms, "gsite_updates_s": W * H / (ms * 1e-3) / 1e9,
            "achieved": gbs, "peak": hbm_peak, "unit": "GB/s", "frac": gbs / hbm_peak,
            "bytes_per_launch": bytes_step, "traffic": profiled_traffic("step_fhp3_32768x16384.md")}


def oracle_check(final_sha):
    """Compare the batched run's final states with the committed hashes of
    the same 512 jobs stepped one by one by the CPU oracle."""
    path = os.path.join(ROOT, "tests", "golden", "batched_512.json")
    try:
        with open(path) as f:
            want = json.load(f)["final_sha"]
    except OSError:
        return {"oracle_checked": 0}
    same = sum(a == b for a, b in zip(final_sha, want))
    return {"oracle_checked": min(len(final_sha), len(want)), "oracle_bit_exact": same,
            "oracle_all_equal": same == len(want) == len(final_sha)}


def batched_bytes_per_step():
    """Algorithmic bytes of one step of the 512-job batched workload."""
    from lgca_gb300 import batched as BT
    total = 0.0
    for j in BT.make_jobs(512):
        D = {0: 4, 1: 6, 2: 7, 3: 7}[j["model"]]
        total += j["W"] * j["H"] * (2 * D / 8 + (1 / 8 if j["geometry"] != "periodic" else 0))
    return total


def served_leg(rate, duration):
    """The served workload, bounded: Poisson arrivals at `rate` jobs/s for
    `duration` s (sizes 256x256..8192x4096, 100..20000 steps, 16x16 fields
    every 500 steps, 150 GB budget), a 10 s drain; FCFS single-lattice
    execution of the same jobs from measured per-step times, and of the first
    200 jobs run back to back on the GPU; 8 sampled jobs rerun alone with
    every streamed field compared."""
    from lgca_gb300 import serve as SV
    r = SV.serve(rate, duration, budget=150e9, drain_limit=10.0, verify=8, fcfs=True,
                 fcfs_sample=1000)
    fm = r.get("fcfs_measured", {})
    return {"rate_jobs_s": rate, "duration_s": duration, "jobs": r["jobs"],
            "completed": r["completed"], "backlog": r["backlog"], "elapsed_s": r["elapsed_s"],
            "p50_s": r["p50_latency_s"], "p99_s": r["p99_latency_s"],
            "sustained_gsite_updates_s": r["sustained_gsite_updates_s"],
            "fcfs_p50_s": r["fcfs"]["p50_latency_s"], "fcfs_p99_s": r["fcfs"]["p99_latency_s"],
            "fcfs_gsite_updates_s": r["fcfs"]["sustained_gsite_updates_s"],
            "x_fcfs": r["throughput_speedup_vs_fcfs"],
            "x_fcfs_best_repeat": r["throughput_speedup_vs_fcfs_best"],
            "fcfs_measured_gsite_updates_s": fm.get("gsite_updates_s"),
            "fcfs_measured_jobs": fm.get("jobs"),
            "fcfs_table_gsite_updates_s_same_jobs": fm.get("table_gsite_updates_s"),
            "x_fcfs_measured": r.get("throughput_speedup_vs_fcfs_measured"),
            "sample_verified": r.get("sample_verified"),
            "sample_bit_exact": r.get("sample_bit_exact"),
            "evictions": r["evictions"], "batch_calls": r["batch_calls"],
            "limited_by": "the batch step kernel (k_batch_persist), at 0.90 of the measured HBM "
                          "bandwidth on a 1 G-site mix (profiles/batch_512_mixed.md); FCFS runs "
                          "each job alone with the fastest single-lattice path (the automatic "
                          "choice, which takes the resident kernel for large jobs)"}


def run_ours(args):
    import torch
    import lgca_gb300 as gpu

    ws, rank, local = dist_env()
    if ws > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    else:
        torch.cuda.set_device(0)
    dev = torch.cuda.current_device()
    gpu.build()
    hbm_peak, peak_kind = peaks()
    seed = 2 + 1000 * rank
    types = karman_types()
    L = gpu.GpuLattice(MODEL, W_K, H_K, seed=seed)
    L.set_cell_types(types)
    L.init_random(0.3, 0.3)
    L.set_forcing_column(16, 0.02)
    stream = torch.cuda.ExternalStream(L.stream_ptr())
    Hb, Wb = H_K // BLOCK, W_K // BLOCK
    sums = torch.empty((3, Hb, Wb), dtype=torch.int32, device="cuda")
    flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device="cuda")  # > 129 MB L2

    def chunk():
        # 100 steps and the 32x32 block sums of their result (the sums inside
        # the step launch where the resident kernel runs)
        L.collide_and_propagate_sums(STEPS_PER_CHUNK, BLOCK, sums[0].data_ptr(), sums[1].data_ptr(),
                                     sums[2].data_ptr())

    for _ in range(args.warmup):
        chunk()
    L.sync()
    ev = [[torch.cuda.Event(enable_timing=True) for _ in range(2)] for _ in range(args.steps)]

    def barrier():
        torch.cuda.synchronize()
        if ws > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    barrier()
    with ClockSampler(dev) as clk:
        t_wall = time.perf_counter()
        for i in range(args.steps):
            with torch.cuda.stream(stream):
                flush.fill_(i & 0xff)  # L2 flush between timed steps (outside the events)
            ev[i][0].record(stream)
            chunk()
            ev[i][1].record(stream)
        barrier()
        t_wall = time.perf_counter() - t_wall
    step_ms = [e[0].elapsed_time(e[1]) for e in ev]
    # the step launch and its fused block sums are one launch: the launch time
    # is the bench step's time
    kern_ms = step_ms
    t_dev = sum(step_ms) / 1e3
    if ws > 1:
        tt = torch.tensor([t_dev], device="cuda", dtype=torch.float64)
        torch.distributed.all_reduce(tt, op=torch.distributed.ReduceOp.MAX)
        t_dev = float(tt.item())
    sites = W_K * H_K * STEPS_PER_CHUNK * args.steps
    value = sites * ws / t_dev / 1e9

    # roofline of the step kernel.  A call of 100 steps is one launch of the
    # resident kernel (the plan below says which kernels a call runs); the
    # lattice stays on chip across its steps, so its bound is instruction
    # issue, not memory: warp instructions per launch (ncu, committed
    # summary) over the launch time, against one warp instruction per clock
    # per SM sub-partition at the sampled clock.
    family, launches_per_call = L.step_plan(STEPS_PER_CHUNK)
    launch_s = sum(kern_ms) / 1e3 / (launches_per_call * args.steps)
    sms = torch.cuda.get_device_properties(dev).multi_processor_count
    clk_hz = (clk.summary().get("sm_mhz") or 2070) * 1e6
    issue_peak = sms * 4 * clk_hz
    # algorithmic bytes of the same steps: 7 planes read + written, the solid plane read
    bytes_step = W_K * H_K * (2 * 7 / 8 + 1 / 8)
    step_s = sum(kern_ms) / 1e3 / (STEPS_PER_CHUNK * args.steps)
    if family == 6:
        prof = "resident_fhp3_karman_8192x2048.md"
        inst = profiled_value(prof, "inst_per_launch")
        roofline = {"bound": "alu-issue", "achieved": inst / launch_s if inst else None,
                    "peak": issue_peak, "unit": "warp-instructions/s",
                    "frac": inst / launch_s / issue_peak if inst else None,
                    "traffic": profiled_traffic(prof), "inst_per_launch": inst,
                    "steps_per_launch": STEPS_PER_CHUNK, "launch_ms": launch_s * 1e3,
                    "alu_pipe_active": profiled_value(prof, "alu_pipe_active"),
                    "kernel": "k_resident<FHP_II/III, GEOM_NOSLIP, row barriers>: 100 steps "
                              "per launch, the lattice on chip between steps",
                    "hbm_equivalent": {"bytes_per_step": bytes_step,
                                       "achieved": bytes_step / step_s / 1e9, "peak": hbm_peak,
                                       "unit": "GB/s", "peak_kind": peak_kind},
                    "note": "DRAM traffic per launch is the state read once (ncu); the ALU pipe "
                            "is 78 % busy while SMs are active and runs logic at half the "
                            "issue rate, so frac (issue) near 0.6 is close to the ALU bound; "
                            "hbm_equivalent is the algorithmic bytes of the same steps over "
                            "time, which never reach HBM; the HBM gate is roofline_gate"}
    else:
        prof = "step_fhp3_karman_8192x2048.md"
        inst = profiled_value(prof, "inst_per_launch")
        achieved = bytes_step / launch_s / 1e9
        roofline = {"bound": "hbm", "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
                    "frac": achieved / hbm_peak, "traffic": profiled_traffic(prof),
                    "peak_kind": peak_kind, "bytes_per_launch": bytes_step,
                    "kernel": "k_step2<FHP_II/III, GEOM_NOSLIP> (two words per lane)",
                    "alu_issue": {"achieved": inst / launch_s if inst else None,
                                  "peak": issue_peak, "unit": "warp-instructions/s",
                                  "frac": inst / launch_s / issue_peak if inst else None}}

    # end to end through the C ABI with host buffers: every bench step is one
    # job -- the input state from pinned memory, 100 lattice steps, the final
    # state and its 32x32 block sums back to pinned memory -- one
    # lgca_run_job_async call: the resident kernel converts the byte-per-cell
    # layout and adds up the block sums inside its launch.  Two lattices take the jobs in
    # turn so that one job's copies overlap the other's steps; each job's step
    # launch occupies all but a few SMs, so the two lattices' steps run one
    # after the other and this rate cannot exceed the one-lattice rate.  Every
    # job starts from the same state at step 0, so all jobs must give
    # identical outputs (checked).
    L2 = gpu.GpuLattice(MODEL, W_K, H_K, seed=seed)
    L2.set_cell_types(types)
    L2.set_forcing_column(16, 0.02)
    lats = [L, L2]
    aos_in = torch.empty((H_K, W_K), dtype=torch.uint8, pin_memory=True).numpy()
    L.download(aos_in)
    aos_out = [torch.empty((H_K, W_K), dtype=torch.uint8, pin_memory=True).numpy() for _ in lats]
    hs = [torch.empty((3, Hb, Wb), dtype=torch.int32, pin_memory=True).numpy() for _ in lats]
    e2e_steps = max(2, min(args.steps, 50))
    # warm-up jobs (first-call allocations, pinned flags) outside the timed
    # region; their outputs are what every timed job must reproduce
    for X, out, h in zip(lats, aos_out, hs):
        X.set_step(0)
        X.run_job_async(aos_in, STEPS_PER_CHUNK, out, BLOCK, h)
    for X in lats:
        X.sync()
    expect = (aos_out[0].copy(), hs[0].copy())
    e2e_same = np.array_equal(aos_out[1], expect[0]) and np.array_equal(hs[1], expect[1])
    barrier()
    t_e2e = time.perf_counter()
    for i in range(e2e_steps):
        k = i & 1
        X = lats[k]
        X.set_step(0)
        X.run_job_async(aos_in, STEPS_PER_CHUNK, aos_out[k], BLOCK, hs[k])
        if i >= 1:  # the other lattice's job is complete before that lattice takes the next
            lats[k ^ 1].sync()
    lats[(e2e_steps - 1) & 1].sync()
    barrier()
    t_e2e = time.perf_counter() - t_e2e
    # the last job of each lattice reproduced the warm-up output
    e2e_same = e2e_same and all(np.array_equal(aos_out[k], expect[0]) and
                                np.array_equal(hs[k], expect[1]) for k in range(2))
    L2.close()
    if ws > 1:
        tt = torch.tensor([t_e2e], device="cuda", dtype=torch.float64)
        torch.distributed.all_reduce(tt, op=torch.distributed.ReduceOp.MAX)
        t_e2e = float(tt.item())
    e2e = {"value": W_K * H_K * STEPS_PER_CHUNK * e2e_steps * ws / t_e2e / 1e9, "unit": UNIT,
           "h2d_bytes_per_step": W_K * H_K, "d2h_bytes_per_step": W_K * H_K + 3 * 4 * Hb * Wb,
           "steps": e2e_steps, "jobs_identical": bool(e2e_same),
           "api": "one lgca_run_job_async per job (state in, 100 steps, state and 32x32 sums out)",
           "pipelining": "two lattices alternate; copies overlap the other lattice's steps; "
                         "each step launch holds all but a few SMs, so steps run one at a time"}

    gate = gate_measurement(gpu, torch, hbm_peak) if rank == 0 else None
    L.close()
    batched = None
    if rank == 0 and not args.no_batched:
        # the batched workload: 512 mixed lattices x 1000 steps, batched vs one at a time
        from lgca_gb300 import batched as BT
        batched = BT.compare(512, 1000, tune=True)
        batched.pop("tuned", None)
        batched.update(oracle_check(batched.pop("final_sha")))
        # HBM roofline of the batched kernel: algorithmic bytes of one step of
        # all members (2 D/8 B per site, + 1/8 B with a solid plane) per step time
        step_s = batched["batched_s"] / batched["steps"]
        bytes_step = batched_bytes_per_step()
        batched["roofline"] = {"bound": "hbm", "achieved": bytes_step / step_s / 1e9,
                               "peak": hbm_peak, "unit": "GB/s",
                               "frac": bytes_step / step_s / 1e9 / hbm_peak,
                               "bytes_per_step": bytes_step,
                               "traffic": profiled_traffic("batch_512_mixed.md"),
                               "kernel": "k_batch_persist (persistent form, grid barrier per step)"}
    served = None
    if rank == 0 and not args.no_served:
        served = served_leg(args.served_rate, args.served_duration)
    if rank == 0:
        cpu = cpu_baseline() if ws == 1 else None
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": t_dev / args.steps * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "u64", "data": "synthetic",
            "config": {"workload": WORKLOAD, "global_batch": ws, "lattice": [W_K, H_K],
                       "lattice_steps_per_step": STEPS_PER_CHUNK, "block": BLOCK,
                       "l2": "flushed between timed steps (256 MiB write, outside the events)",
                       "parallelism": f"replicas x{ws}"},
            "wall_s": t_wall, "e2e": e2e, "roofline": roofline, "roofline_gate": gate,
            "batched": batched, "served": served,
            "cpu_baseline": cpu, "clocks": clk.summary(),
            # step-kernel launches of each call (lgca_step_plan), plus a block-sum
            # kernel unless the sums are fused into the resident kernel
            "gpu_launches": (launches_per_call + (0 if family == 6 else 1)) * args.steps,
        }
        print(json.dumps(line), flush=True)
    if ws > 1:
        torch.distributed.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-batched", action="store_true",
                    help="skip the 512-lattice batched vs one-at-a-time comparison")
    ap.add_argument("--no-served", action="store_true", help="skip the served-form leg")
    ap.add_argument("--served-rate", type=float, default=800.0)
    ap.add_argument("--served-duration", type=float, default=20.0)
    args = ap.parse_args()
    if args.warmup < 3:
        ap.error("--warmup must be >= 3")
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
