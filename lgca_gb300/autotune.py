"""Measured autotuning of the kernel choices.

Two tables, both chosen by timing candidates on the GPU:

* single lattice, per (model, size class): kernel family and steps per pass
  over global memory -- one step per pass with one or two words per lane,
  register wavefront or shared-memory tiles with 2, 4 or 8 steps per pass;
* batch members, per (model family, size class): words per lane of the
  batched one-step kernel.

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
# tiles.  Warps per block applies to the one-step kernels (0 = per launch).
SINGLE_CANDIDATES = [(5, 1, 4), (5, 1, 8), (5, 1, 2), (1, 1, 4), (1, 1, 2),
                     (2, 2, 0), (2, 4, 0), (2, 8, 0), (3, 2, 0), (3, 4, 0), (3, 8, 0)]
WPT_CANDIDATES = {1: 1, 2: 5}  # words per lane -> kernel variant of a batch member


def size_class(W: int, H: int) -> int:
    return int(math.log2(max(1, W * H)))


def family(model: int) -> int:
    return 0 if model == gpu.HPP else (1 if model == gpu.FHP_I else 2)


class Autotuner:
    def __init__(self, cache_path: str | None = None):
        self.cache_path = cache_path
        self.single: dict[str, tuple[int, int, int]] = {}
        self.batch: dict[str, int] = {}
        if cache_path and os.path.exists(cache_path):
            with open(cache_path) as f:
                d = json.load(f)
            self.single = {k: tuple(v) for k, v in d.get("single", {}).items() if len(v) == 3}
            self.batch = {k: int(v) for k, v in d.get("batch", {}).items()}

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
    def tune_batch_members(self, lattices, steps: int = 24, sample: int = 6,
                           margin: float = 0.03, repeats: int = 2) -> dict[str, int]:
        """Choose words per lane per (model family, size class) where it
        matters: inside a batch that holds twins of up to `sample` members of
        every class (so the device is as loaded as in the real batch), each
        untuned class is timed with each candidate while the others keep two
        words per lane (best of `repeats`); two words stay unless one word
        makes the whole batch faster by more than `margin`.  Apply the choice
        (as the members' kernel variant)."""
        groups: dict[str, list] = {}
        for L in lattices:
            groups.setdefault(f"{family(L.model)}:{size_class(L.dim_x, L.dim_y)}", []).append(L)
        todo = [key for key in groups if key not in self.batch]
        if todo:
            twins: dict[str, list] = {}
            for key, members in groups.items():
                twins[key] = []
                for L in members[:sample]:
                    T = gpu.GpuLattice(L.model, L.dim_x, L.dim_y)
                    T.restore(L.checkpoint())
                    T.set_kernel_variant(WPT_CANDIDATES[2])
                    twins[key].append(T)
            with gpu.GpuBatch() as B:
                for ts in twins.values():
                    for T in ts:
                        B.add(T)

                def timed() -> float:
                    B.step(2)
                    B.sync()
                    t0 = time.perf_counter()
                    B.step(steps)
                    B.sync()
                    return time.perf_counter() - t0

                for key in todo:
                    times = {}
                    for wpt, variant in WPT_CANDIDATES.items():
                        for T in twins[key]:
                            T.set_kernel_variant(variant)
                        times[wpt] = min(timed() for _ in range(repeats))
                    for T in twins[key]:
                        T.set_kernel_variant(WPT_CANDIDATES[2])
                    self.batch[key] = 1 if times[1] < (1.0 - margin) * times[2] else 2
            for ts in twins.values():
                for T in ts:
                    T.close()
        for key, members in groups.items():
            for L in members:
                L.set_kernel_variant(WPT_CANDIDATES[self.batch[key]])
        return dict(self.batch)


def describe(tuner: Autotuner) -> dict:
    names = {1: "one-step/1 word", 5: "one-step/2 words", 2: "wavefront", 3: "smem tiles"}
    return {k: f"{names.get(v[0], v[0])}, depth {v[1]}, {v[2] or 'auto'} warps/block"
            for k, v in tuner.single.items()}


__all__ = ["Autotuner", "size_class", "family", "SINGLE_CANDIDATES", "describe"]
