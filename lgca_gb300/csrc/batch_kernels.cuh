// Kernels of the batched step (launched from batch.cu): the per-step batch
// kernel over the device work-list, the per-call key table and the step
// counter of graph replays.  Kept apart from the launchers so that the
// kernel bodies also build as host C++ (the CPU emulation in the tests).
#pragma once
#include "internal.cuh"
#include "../../include/lgca/rng.h"

// the per-word step bodies
#include "step_body.cuh"

namespace lgca_gpu {

// One launch per step for all members.  Each member's warp tasks are padded
// to whole blocks (8 warps x T tasks per warp), so block b belongs to lattice
// block_lat[b] alone and needs no search; warp w of a block takes the
// block's tasks w, w + 8, ... (T of them), reusing the lattice's entry, keys
// and buffer pointers, so the entry's load latency is paid once per T tasks.
// The entry selects model, geometry mode and words per lane.  GMAX is the
// largest geometry mode among the members: batches without slip cells use a
// kernel compiled without the slip-aware paths, held to 64 registers (4
// blocks of 8 warps per SM).
template <int GMAX, int T>
__global__ void __launch_bounds__(256, GMAX == GEOM_FULL ? 3 : 4)
    k_batch(const BatchEntry *__restrict__ E, const int *__restrict__ block_lat, int s_local,
            const int *__restrict__ s_base)
{
    pdl_launch_dependents();
    // The work-list, the key table and the step counter were written before
    // the chain of batch steps began (copies and plain kernels, which
    // complete before the chain's first kernel starts) and stay unchanged
    // along it, so they are read before the wait; only the states come from
    // the previous step.
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const BatchEntry &e = E[block_lat[blockIdx.x]];
    const int base = blockIdx.x * 8 * T - e.task0;  // the block's first task of its lattice
    const int s = *s_base + s_local;
    const ulonglong2 k = __ldg(reinterpret_cast<const ulonglong2 *>(e.keys) + s);
    const StepIO io{(s & 1) ? e.buf1 : e.buf0, (s & 1) ? e.buf0 : e.buf1, k.x, k.y};
    const StepArgs &a = e.a;
    pdl_wait();
    for (int i = 0; i < T; ++i) {
        const int local = base + warp + 8 * i;
        if (local >= e.tasks) break;  // padding: warp-uniform
        int y, w;  // the lane's row and item (flattened same-parity mapping)
        flat_site(local, lane, e.a.g.H, e.items, e.a.fmagic, y, w);
#define LGCA_BATCH_CASE(F, MODEL, GM)                                                          \
    case F * 9 + GM * 3:                                                                       \
        if (GM <= GMAX) step_word<MODEL, GM, true>(a, io, y, w, lane);                         \
        break;                                                                                 \
    case F * 9 + GM * 3 + 1:                                                                   \
        if (GM <= GMAX) step_pair<MODEL, GM, true, false, false, true>(a, io, y, w, lane);     \
        break;                                                                                 \
    case F * 9 + GM * 3 + 2:                                                                   \
        if (GM <= GMAX) step_pair<MODEL, GM, true, false, true, true>(a, io, y, w, lane);      \
        break;
#define LGCA_BATCH_CASES(F, MODEL)                                                             \
    LGCA_BATCH_CASE(F, MODEL, GEOM_NONE)                                                       \
    LGCA_BATCH_CASE(F, MODEL, GEOM_NOSLIP)                                                     \
    LGCA_BATCH_CASE(F, MODEL, GEOM_FULL)
        switch (e.code) {
            LGCA_BATCH_CASES(0, M_HPP)
            LGCA_BATCH_CASES(1, M_FHP_I)
            LGCA_BATCH_CASES(2, M_FHP_II)
        default: break;
        }
#undef LGCA_BATCH_CASES
#undef LGCA_BATCH_CASE
    }
}

// keys[l][s] = (chirality key, forcing key) of member l at its step t0 + s
__global__ void k_batch_keys(const BatchEntry *__restrict__ E, int n, int max_steps)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (long long)n * max_steps) return;
    const int l = (int)(i / max_steps), s = (int)(i - (long long)l * max_steps);
    const BatchEntry &e = E[l];
    if (s >= e.nsteps) return;
    const uint64_t t = e.t0 + (uint64_t)s;
    e.keys[2 * s] = lgca_rng_key(e.seed, LGCA_STREAM_CHIR, t);
    e.keys[2 * s + 1] = lgca_rng_key(e.seed, LGCA_STREAM_FORCE, t);
}

__global__ void k_advance(int *s_base, int by)
{
    if (threadIdx.x == 0 && blockIdx.x == 0) *s_base += by;
}

__global__ void k_set_base(int *s_base, int v)
{
    if (threadIdx.x == 0 && blockIdx.x == 0) *s_base = v;
}

}  // namespace lgca_gpu
