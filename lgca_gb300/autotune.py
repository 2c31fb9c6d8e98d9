"""Measured autotuning of the kernel choices.

Two tables, both chosen by timing candidates on the GPU:

* single lattice, per (model, size class): kernel family and steps per pass
  over global memory -- one step per pass with one or two words per lane,
  register wavefront or shared-memory tiles with 2, 4 or 8 steps per pass,
  or the resident kernel (every step of a call on chip) where it fits;
* batch members, per (model family, size class): the batched one-step
  kernel with one or two words per lane, or the batched register wavefront
  with 2, 4 or 8 steps per pass (8 for HPP only).

A size class is the power of two of the site count (W*H rounded down).
Candidates are timed on a copy of the caller's lattice (checkpoint/restore),
so tuning never changes a lattice's state.  Results are cached in memory and,
optionally, in a JSON file.
"""
from __future__ import annotations

import json
import math
import os
import time

import lgca_gb300 as gpu

# (variant, depth, warps per block): 5 = one step per pass, two words per
# lane; 1 = one word per lane; 2 = register wavefront; 3 = shared-memory
# tiles; 6 = resident (one step per pass where the lattice does not fit it).
# Warps per block applies to the one-step kernels (0 = per launch).
SINGLE_CANDIDATES = [(5, 1, 4), (5, 1, 8), (5, 1, 2), (1, 1, 4), (1, 1, 2),
                     (2, 2, 0), (2, 4, 0), (2, 8, 0), (3, 2, 0), (3, 4, 0), (3, 8, 0),
                     (6, 1, 0)]
# (kernel variant, steps per pass) of a batch member: one step per launch
# with two or one words per lane, or passes of 2, 4, 8 steps on the wavefront
BATCH_CANDIDATES = [(5, 1), (1, 1), (2, 2), (2, 4), (2, 8)]
BATCH_DEFAULT = (5, 1)


def size_class(W: int, H: int) -> int:
    return int(math.log2(max(1, W * H)))


def family(model: int) -> int:
    return 0 if model == gpu.HPP else (1 if model == gpu.FHP_I else 2)


class Autotuner:
    def __init__(self, cache_path: str | None = None):
        self.cache_path = cache_path
        self.single: dict[str, tuple[int, int, int]] = {}
        self.batch: dict[str, tuple[int, int]] = {}
        if cache_path and os.path.exists(cache_path):
            with open(cache_path) as f:
                d = json.load(f)
            self.single = {k: tuple(v) for k, v in d.get("single", {}).items() if len(v) == 3}
            self.batch = {k: tuple(v) for k, v in d.get("batch", {}).items()
                          if isinstance(v, list) and len(v) == 2}

    def save(self) -> None:
        if self.cache_path:
            with open(self.cache_path, "w") as f:
                json.dump({"single": self.single, "batch": self.batch}, f, indent=1)

    # ------------------------------------------------------------ single lattice
    def tune_lattice(self, L: "gpu.GpuLattice", steps: int = 16) -> tuple[int, int, int]:
        """Choose (variant, depth, warps per block) for L's (model, size
        class) by timing the candidates on a twin of L; apply the choice to L
        and return it."""
        key = f"{L.model}:{size_class(L.dim_x, L.dim_y)}"
        if key not in self.single:
            blob = L.checkpoint()
            twin = gpu.GpuLattice(L.model, L.dim_x, L.dim_y)
            best, best_t = (5, 1, 0), float("inf")
            for variant, depth, bw in SINGLE_CANDIDATES:
                twin.restore(blob)
                twin.set_kernel_variant(variant)
                twin.set_temporal_depth(depth)
                twin.set_block_warps(bw)
                n = max(steps, 2 * depth)
                twin.collide_and_propagate(depth)  # warm-up (and kernel load)
                twin.sync()
                t0 = time.perf_counter()
                twin.collide_and_propagate(n)
                twin.sync()
                t = (time.perf_counter() - t0) / n
                if t < best_t:
                    best, best_t = (variant, depth, bw), t
            twin.close()
            self.single[key] = best
        variant, depth, bw = self.single[key]
        L.set_kernel_variant(variant)
        L.set_temporal_depth(depth)
        L.set_block_warps(bw)
        return variant, depth, bw

    # ------------------------------------------------------------ batch members
    def tune_batch_members(self, lattices, steps: int = 32, sample: int = 6,
                           min_sites: int = 1 << 25, margin: float = 0.03,
                           repeats: int = 2) -> dict:
        """Choose (kernel variant, steps per pass) per (model family, size
        class) of batch members: each untuned class is timed alone, as a
        batch of twins of up to `sample` of its members repeated until they
        hold `min_sites` sites (so that the class fills the device as the
        whole batch does), with each candidate (best of `repeats`).  The
        default (two words per lane, one step per launch) stays unless
        another candidate is faster by more than `margin`.  Apply the choice
        to the members."""
        groups: dict[str, list] = {}
        for L in lattices:
            groups.setdefault(f"{family(L.model)}:{size_class(L.dim_x, L.dim_y)}", []).append(L)
        for key in [k for k in groups if k not in self.batch]:
            members = groups[key][:sample]
            blobs = [L.checkpoint() for L in members]
            per = sum(L.dim_x * L.dim_y for L in members)
            n = len(members) * max(1, min(-(-min_sites // per), 1024 // len(members)))
            twins = []
            for i in range(n):
                L = members[i % len(members)]
                T = gpu.GpuLattice(L.model, L.dim_x, L.dim_y)
                T.restore(blobs[i % len(members)])
                twins.append(T)
            fam = int(key.split(":")[0])
            times = {}
            with gpu.GpuBatch() as B:
                for T in twins:
                    B.add(T)
                for cand in BATCH_CANDIDATES:
                    if cand[1] == 8 and fam != 0:
                        continue  # the FHP wavefront keeps at most 4 time levels
                    for T in twins:
                        apply_batch_choice(T, cand)
                    best_t = float("inf")
                    for _ in range(repeats):
                        B.step(8)  # warm-up (and kernel load)
                        B.sync()
                        best_t = min(best_t, _timed_steps(B, steps))
                    times[cand] = best_t
            for T in twins:
                T.close()
            best = min(times, key=times.get)
            self.batch[key] = (best if times[best] < (1.0 - margin) * times[BATCH_DEFAULT]
                               else BATCH_DEFAULT)
        for key, members in groups.items():
            for L in members:
                apply_batch_choice(L, self.batch[key])
        return dict(self.batch)


def _timed_steps(B: "gpu.GpuBatch", steps: int) -> float:
    """Seconds of `steps` batch steps on the batch's stream: CUDA events where
    torch is present (the second of two calls is timed, so that its host-side
    preparation overlaps the first call's steps), else wall time around the
    call and its wait."""
    try:
        import torch
    except ImportError:
        torch = None
    if torch is not None and torch.cuda.is_available():
        s = torch.cuda.ExternalStream(B.stream_ptr())
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        B.step(steps)
        e0.record(s)
        B.step(steps)
        e1.record(s)
        e1.synchronize()
        return e0.elapsed_time(e1) * 1e-3
    t0 = time.perf_counter()
    B.step(steps)
    B.sync()
    return time.perf_counter() - t0


def apply_batch_choice(L: "gpu.GpuLattice", choice) -> None:
    variant, depth = choice
    L.set_kernel_variant(variant)
    L.set_temporal_depth(depth)


def describe(tuner: Autotuner) -> dict:
    names = {1: "one-step/1 word", 5: "one-step/2 words", 2: "wavefront", 3: "smem tiles"}
    return {k: f"{names.get(v[0], v[0])}, depth {v[1]}, {v[2] or 'auto'} warps/block"
            for k, v in tuner.single.items()}


__all__ = ["Autotuner", "size_class", "family", "SINGLE_CANDIDATES", "BATCH_CANDIDATES", "describe"]
