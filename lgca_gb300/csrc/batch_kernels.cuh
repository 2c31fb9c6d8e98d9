// Kernels of the batched step (launched from batch.cu): the per-step batch
// kernel over the device work-list and its persistent form, the batch's
// register-wavefront passes, the per-call key table and the step counter of
// graph replays.  Kept apart from the launchers so that the
// kernel bodies also build as host C++ (the CPU emulation in the tests).
#pragma once
#include "internal.cuh"
#include "../../include/lgca/rng.h"

// the per-word step bodies and the wavefront warp body
#include "step_body.cuh"
#include "wave_body.cuh"

namespace lgca_gpu {

// Work-list block `blk` at batch-local step s: warp w of the block takes the
// block's tasks w, w + 8, ... (T of them).  `wait` runs between the reads of
// the work-list and keys (written before a chain of steps began) and the
// first state access (programmatic dependent launch).
template <int GMAX, int T, class Wait>
__device__ __forceinline__ void batch_block(const BatchEntry *__restrict__ E,
                                            const int *__restrict__ block_lat, int blk, int s,
                                            Wait wait)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const BatchEntry &e = E[block_lat[blk]];
    const int base = blk * 8 * T - e.task0;  // the block's first task of its lattice
    const ulonglong2 k = __ldg(reinterpret_cast<const ulonglong2 *>(e.keys) + s);
    const StepIO io{(s & 1) ? e.buf1 : e.buf0, (s & 1) ? e.buf0 : e.buf1, k.x, k.y};
    const StepArgs &a = e.a;
    wait();
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
    batch_block<GMAX, T>(E, block_lat, blockIdx.x, *s_base + s_local, [] { pdl_wait(); });
}

// Persistent form: one cooperative launch runs steps s0 .. s0 + nsteps - 1
// over the same work-list; each resident block takes work-list blocks
// blockIdx.x, blockIdx.x + gridDim.x, ... and a grid barrier separates the
// steps.  The barrier counter *bar starts at zero; a wait longer than
// wait_ns sets *err and every block stops.  (State loads go through L2, so
// a step sees the previous step's stores of other blocks after the barrier.)
template <int GMAX, int T>
__global__ void __launch_bounds__(256, 3)
    k_batch_persist(const BatchEntry *__restrict__ E, const int *__restrict__ block_lat,
                    int nblocks, int s0, int nsteps, unsigned *bar, int *err, uint64_t wait_ns)
{
    __shared__ int stop;
    for (int s = 0; s < nsteps; ++s) {
        for (int blk = blockIdx.x; blk < nblocks; blk += gridDim.x)
            batch_block<GMAX, T>(E, block_lat, blk, s0 + s, [] {});
        if (s + 1 == nsteps) break;
        __syncthreads();
        if (threadIdx.x == 0) {
            __threadfence();  // this block's stores of step s, before it arrives
            atomicAdd(bar, 1u);
            const unsigned want = (unsigned)(s + 1) * gridDim.x;
            volatile unsigned *vb = bar;
            volatile int *ve = err;
            stop = 0;
#ifdef __CUDA_ARCH__
            uint64_t t0, t;
            asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t0));
            while (*vb < want) {
                asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
                if (*ve || t - t0 > wait_ns) {
                    atomicExch(err, 1);
                    stop = 1;
                    break;
                }
                __nanosleep(32);
            }
#endif
            __threadfence();
        }
        __syncthreads();
        if (stop) return;
    }
}

// One launch per K-step pass for the members on the register wavefront.
// Block b belongs to member block_lat[b]; its 4 warps take consecutive
// (strip, slab) tasks of the member.  Pass j of a member covers its steps
// r + j*K .. r + j*K + K-1 of the call (its r single steps came first, on
// k_batch), so it reads buffer (r + j) & 1 and its keys start at step r + j*K.
template <int GMAX, int K>
__global__ void __launch_bounds__(32 * WAVE_BLOCK_WARPS)
    k_batch_wave(const BatchEntry *__restrict__ E, const int *__restrict__ block_lat, int j_local,
                 const int *__restrict__ j_base)
{
    pdl_launch_dependents();
    // the work-list, keys and pass counter were written before the chain of
    // steps began (see k_batch); only the states come from the previous pass
    const BatchEntry &e = E[block_lat[blockIdx.x]];
    const int local = blockIdx.x * WAVE_BLOCK_WARPS + (int)(threadIdx.x >> 5) - e.task0;
    const int j = *j_base + j_local;
    const TableKeys<K> keys(e.keys + 2 * (e.r + j * K));
    const bool odd = ((e.r + j) & 1) != 0;
    const uint64_t *src = odd ? e.buf1 : e.buf0;
    uint64_t *dst = odd ? e.buf0 : e.buf1;
    pdl_wait();
    if (local >= e.tasks) return;  // padding: warp-uniform
    const int sx = local % e.nstrips, sy = local / e.nstrips;
#define LGCA_WAVE_CASE(F, MODEL, GM)                                                           \
    case F * 9 + GM * 3:                                                                       \
    case F * 9 + GM * 3 + 1:                                                                   \
    case F * 9 + GM * 3 + 2:                                                                   \
        if constexpr (GM <= GMAX && (K <= 4 || MODEL == M_HPP))                                \
            wave_strip<MODEL, GM, K>(e.a, src, dst, keys, e.S, sx, sy);                        \
        break;
#define LGCA_WAVE_CASES(F, MODEL)                                                              \
    LGCA_WAVE_CASE(F, MODEL, GEOM_NONE)                                                        \
    LGCA_WAVE_CASE(F, MODEL, GEOM_NOSLIP)                                                      \
    LGCA_WAVE_CASE(F, MODEL, GEOM_FULL)
    switch (e.code) {
        LGCA_WAVE_CASES(0, M_HPP)
        LGCA_WAVE_CASES(1, M_FHP_I)
        LGCA_WAVE_CASES(2, M_FHP_II)
    default: break;
    }
#undef LGCA_WAVE_CASES
#undef LGCA_WAVE_CASE
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
