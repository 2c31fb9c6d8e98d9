// Batched step: many independent lattices of any sizes, models and
// geometries advance together, one launch per step and model family over a
// device-side work-list of warp tasks (lattice, row, chunk of words).  Each
// task runs the same per-word step code as the single-lattice kernels, with
// the lattice's own buffers, geometry, forcing and keys, so every lattice
// gives exactly the bits it gives alone.
//
// Work-list: the lattices of one model family sorted by steps to do
// (descending); prefix[l] = first task of lattice l.  At step s the active
// lattices are a prefix of the list, so a launch covers tasks
// [0, prefix[n_active]).  A warp finds its lattice by binary search.
#include "internal.cuh"
#include "../../include/lgca/rng.h"

// the per-word step bodies
#include "step_body.cuh"

namespace lgca_gpu {

template <int MODEL>
__global__ void __launch_bounds__(256) k_batch(const BatchEntry *__restrict__ E,
                                               const int *__restrict__ prefix, int n_active,
                                               int s_local, const int *__restrict__ s_base)
{
    const int lane = threadIdx.x & 31;
    const int g = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    const int total = prefix[n_active];
    if (g >= total) return;
    int lo = 0, hi = n_active - 1;  // largest l with prefix[l] <= g
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (prefix[mid] <= g) lo = mid;
        else hi = mid - 1;
    }
    const BatchEntry &e = E[lo];
    const int s = *s_base + s_local;
    const int local = g - prefix[lo];
    const int y = local / e.per_row, c = local - y * e.per_row;
    const uint64_t t = e.t0 + (uint64_t)s;
    const StepIO io{(s & 1) ? e.buf1 : e.buf0, (s & 1) ? e.buf0 : e.buf1,
                    lgca_rng_key(e.seed, LGCA_STREAM_CHIR, t),
                    lgca_rng_key(e.seed, LGCA_STREAM_FORCE, t)};
    const StepArgs &a = e.a;
    switch (e.gm * 2 + (e.wpt == 2 ? 1 : 0)) {
    case GEOM_NONE * 2: step_word<MODEL, GEOM_NONE>(a, io, y, c * 32 + lane, lane); break;
    case GEOM_NONE * 2 + 1: step_pair<MODEL, GEOM_NONE>(a, io, y, c * 32 + lane, lane); break;
    case GEOM_NOSLIP * 2: step_word<MODEL, GEOM_NOSLIP>(a, io, y, c * 32 + lane, lane); break;
    case GEOM_NOSLIP * 2 + 1: step_pair<MODEL, GEOM_NOSLIP>(a, io, y, c * 32 + lane, lane); break;
    case GEOM_FULL * 2: step_word<MODEL, GEOM_FULL>(a, io, y, c * 32 + lane, lane); break;
    default: step_pair<MODEL, GEOM_FULL>(a, io, y, c * 32 + lane, lane); break;
    }
}

__global__ void k_advance(int *s_base, int by)
{
    if (threadIdx.x == 0 && blockIdx.x == 0) *s_base += by;
}

cudaError_t launch_batch(int model_family, const BatchEntry *E, const int *prefix, int n_active,
                         int total_tasks, int s_local, const int *s_base, cudaStream_t st)
{
    if (total_tasks <= 0) return cudaSuccess;
    const unsigned grid = (unsigned)((total_tasks + 7) / 8);
    switch (model_family) {
    case M_HPP: k_batch<M_HPP><<<grid, 256, 0, st>>>(E, prefix, n_active, s_local, s_base); break;
    case M_FHP_I: k_batch<M_FHP_I><<<grid, 256, 0, st>>>(E, prefix, n_active, s_local, s_base); break;
    default: k_batch<M_FHP_II><<<grid, 256, 0, st>>>(E, prefix, n_active, s_local, s_base); break;
    }
    return cudaGetLastError();
}

cudaError_t launch_advance(int *s_base, int by, cudaStream_t st)
{
    k_advance<<<1, 32, 0, st>>>(s_base, by);
    return cudaGetLastError();
}

}  // namespace lgca_gpu
