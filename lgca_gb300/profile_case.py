"""Run one lattice workload on the GPU for a fixed number of steps: a small,
self-contained program for profilers (ncu) and for quick timings.

    python -m lgca_gb300.profile_case --model 3 --W 32768 --H 16384 --steps 3
    python -m lgca_gb300.profile_case --geometry karman --W 8192 --H 2048 --force-x 16 --force-p 0.02
    python -m lgca_gb300.profile_case --geometry karman --W 8192 --H 2048 --force-x 16 --force-p 0.02 --chunk 100
    python -m lgca_gb300.profile_case --batch 512 --steps 4   # the batched workload, one step per call

Prints the average time per step (host clock around the steps and a wait).
"""
from __future__ import annotations

import argparse
import time

import lgca_gb300 as gpu
from lgca_gb300 import geometry as G


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--model", type=int, default=3)
    ap.add_argument("--W", type=int, default=32768)
    ap.add_argument("--H", type=int, default=16384)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=1)
    ap.add_argument("--depth", type=int, default=1)
    ap.add_argument("--variant", type=int, default=0,
                    help="0 auto, 1 one step per pass, 2 register wavefront, 3 shared-memory tiles, "
                         "4 persistent bands, 5 two words per lane, 6 resident")
    ap.add_argument("--chunk", type=int, default=0,
                    help="steps per call (default: 1, or the depth); the automatic choice takes "
                         "the resident form for large enough lattices and calls where it fits")
    ap.add_argument("--geometry", default="periodic", choices=["periodic", "pipe", "karman"])
    ap.add_argument("--force-x", type=int, default=-1)
    ap.add_argument("--force-p", type=float, default=0.0)
    ap.add_argument("--p", type=float, default=0.5)
    ap.add_argument("--block", type=int, default=0,
                    help="also compute the BxB block sums of each call's result (into device "
                         "buffers, fused into the step launch where the resident kernel runs)")
    ap.add_argument("--batch", type=int, default=0,
                    help="run the first N jobs of the batched workload as one batch instead")
    ap.add_argument("--launches", action="store_true",
                    help="(with --batch) one launch per step instead of the persistent form")
    args = ap.parse_args(argv)

    gpu.build()
    if args.batch:
        from lgca_gb300 import batched as BT
        jobs = BT.make_jobs(args.batch)
        lats = [BT.build(j) for j in jobs]
        with gpu.GpuBatch() as B:
            B.set_persistent(not args.launches)
            for L in lats:
                B.add(L)
            for _ in range(args.warmup):
                B.step(1)
            B.sync()
            t0 = time.perf_counter()
            for _ in range(args.steps):
                B.step(1)
            B.sync()
            dt = time.perf_counter() - t0
        sites = sum(j["W"] * j["H"] for j in jobs)
        print(f"batch of {args.batch}: {dt / args.steps * 1e3:.4f} ms/step (host clock), "
              f"{sites * args.steps / dt / 1e9:.1f} GSite-updates/s")
        for L in lats:
            L.close()
        return
    L = gpu.GpuLattice(args.model, args.W, args.H, seed=3)
    if args.geometry == "pipe":
        L.set_cell_types(G.pipe(args.W, args.H))
    elif args.geometry == "karman":
        L.set_cell_types(G.disc(args.W, args.H, args.W // 8, args.H // 2, args.H // 16))
    L.init_random(args.p, args.p)
    L.set_forcing_column(args.force_x, args.force_p)
    if args.variant != 4:
        L.set_temporal_depth(args.depth)
    L.set_kernel_variant(args.variant)
    L.collide_and_propagate(args.warmup)
    L.sync()
    per_call = args.chunk or (1 if args.depth == 1 else args.depth)
    sums = None
    if args.block:
        import torch
        B = args.block
        sums = torch.empty((3, -(-args.H // B), -(-args.W // B)), dtype=torch.int32, device="cuda")
    t0 = time.perf_counter()
    for _ in range(args.steps):
        if sums is not None:
            L.collide_and_propagate_sums(per_call, args.block, sums[0].data_ptr(),
                                         sums[1].data_ptr(), sums[2].data_ptr())
        else:
            L.collide_and_propagate(per_call)
    L.sync()
    dt = time.perf_counter() - t0
    n = args.steps * per_call
    print(f"{args.W}x{args.H} model {args.model} depth {args.depth} variant {args.variant}: {n} steps, {dt / n * 1e3:.4f} ms/step (host clock), "
          f"{args.W * args.H * n / dt / 1e9:.1f} GSite-updates/s")
    L.close()


if __name__ == "__main__":
    main()
