// Batched step: many independent lattices of any sizes, models and
// geometries advance together, one launch per step over a device-side
// work-list of warp tasks (lattice, row, chunk of words).  Each
// task runs the same per-word step code as the single-lattice kernels, with
// the lattice's own buffers, geometry, forcing and keys, so every lattice
// gives exactly the bits it gives alone.
//
// Work-list: all members sorted by steps to do (descending); prefix[l] =
// first task of lattice l, block_lat[b] = lattice of block b's first task.
// At step s the active lattices are a prefix of the list, so a launch covers
// tasks [0, prefix[n_active]).  The chirality and forcing keys of every
// (member, step) are computed once per batch call into a table.
#include "batch_kernels.cuh"

#include <algorithm>

namespace lgca_gpu {

template <int T>
static cudaError_t launch_batch_t(const BatchEntry *E, const int *block_lat, int total_tasks,
                                  int s_local, const int *s_base, int gmax, cudaStream_t st)
{
    const dim3 grid((unsigned)(total_tasks / (8 * T)));  // tasks come in whole blocks
    switch (gmax) {
    case GEOM_NONE:
        return launch_pdl(k_batch<GEOM_NONE, T>, grid, dim3(256), 0, st, E, block_lat, s_local, s_base);
    case GEOM_NOSLIP:
        return launch_pdl(k_batch<GEOM_NOSLIP, T>, grid, dim3(256), 0, st, E, block_lat, s_local,
                          s_base);
    default:
        return launch_pdl(k_batch<GEOM_FULL, T>, grid, dim3(256), 0, st, E, block_lat, s_local, s_base);
    }
}

cudaError_t launch_batch(const BatchEntry *E, const int *block_lat, int total_tasks, int s_local,
                         const int *s_base, int gmax, int warp_tasks, cudaStream_t st)
{
    if (total_tasks <= 0) return cudaSuccess;
    switch (warp_tasks) {
    case 1: return launch_batch_t<1>(E, block_lat, total_tasks, s_local, s_base, gmax, st);
    case 2: return launch_batch_t<2>(E, block_lat, total_tasks, s_local, s_base, gmax, st);
    case 4: return launch_batch_t<4>(E, block_lat, total_tasks, s_local, s_base, gmax, st);
    case 8: return launch_batch_t<8>(E, block_lat, total_tasks, s_local, s_base, gmax, st);
    default: return cudaErrorInvalidValue;
    }
}

template <int GMAX, int T>
static cudaError_t launch_persist_t(const BatchEntry *E, const int *block_lat, int nblocks, int s0,
                                   int nsteps, unsigned *bar, int *err, uint64_t wait_ns,
                                   cudaStream_t st)
{
    auto kern = k_batch_persist<GMAX, T>;
    int dev = 0, nsm = 0, per_sm = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, 256, 0);
    if (e != cudaSuccess) return e;
    if (per_sm < 1) return cudaErrorLaunchOutOfResources;
    const int blocks = std::max(1, std::min(nblocks, per_sm * nsm));  // all resident at once
    void *args[] = {(void *)&E, (void *)&block_lat, (void *)&nblocks, (void *)&s0,
                    (void *)&nsteps, (void *)&bar, (void *)&err, (void *)&wait_ns};
    return cudaLaunchCooperativeKernel((void *)kern, dim3((unsigned)blocks), dim3(256), args, 0, st);
}

template <int T>
static cudaError_t launch_persist_g(const BatchEntry *E, const int *block_lat, int nblocks, int s0,
                                   int nsteps, unsigned *bar, int *err, uint64_t wait_ns, int gmax,
                                   cudaStream_t st)
{
    switch (gmax) {
    case GEOM_NONE:
        return launch_persist_t<GEOM_NONE, T>(E, block_lat, nblocks, s0, nsteps, bar, err, wait_ns, st);
    case GEOM_NOSLIP:
        return launch_persist_t<GEOM_NOSLIP, T>(E, block_lat, nblocks, s0, nsteps, bar, err, wait_ns, st);
    default:
        return launch_persist_t<GEOM_FULL, T>(E, block_lat, nblocks, s0, nsteps, bar, err, wait_ns, st);
    }
}

cudaError_t launch_batch_persist(const BatchEntry *E, const int *block_lat, int total_tasks, int s0,
                                 int nsteps, unsigned *bar, int *err, uint64_t wait_ns, int gmax,
                                 int warp_tasks, cudaStream_t st)
{
    if (total_tasks <= 0 || nsteps <= 0) return cudaSuccess;
    const int nblocks = total_tasks / (8 * warp_tasks);
    switch (warp_tasks) {
    case 1: return launch_persist_g<1>(E, block_lat, nblocks, s0, nsteps, bar, err, wait_ns, gmax, st);
    case 2: return launch_persist_g<2>(E, block_lat, nblocks, s0, nsteps, bar, err, wait_ns, gmax, st);
    case 4: return launch_persist_g<4>(E, block_lat, nblocks, s0, nsteps, bar, err, wait_ns, gmax, st);
    case 8: return launch_persist_g<8>(E, block_lat, nblocks, s0, nsteps, bar, err, wait_ns, gmax, st);
    default: return cudaErrorInvalidValue;
    }
}

template <int K>
static cudaError_t launch_wave_k(const BatchEntry *E, const int *block_lat, int total_tasks,
                                 int j_local, const int *j_base, int gmax, cudaStream_t st)
{
    const dim3 grid((unsigned)(total_tasks / WAVE_BLOCK_WARPS)), block(32 * WAVE_BLOCK_WARPS);
    switch (gmax) {
    case GEOM_NONE:
        return launch_pdl(k_batch_wave<GEOM_NONE, K>, grid, block, 0, st, E, block_lat, j_local, j_base);
    case GEOM_NOSLIP:
        return launch_pdl(k_batch_wave<GEOM_NOSLIP, K>, grid, block, 0, st, E, block_lat, j_local,
                          j_base);
    default:
        return launch_pdl(k_batch_wave<GEOM_FULL, K>, grid, block, 0, st, E, block_lat, j_local, j_base);
    }
}

cudaError_t launch_batch_wave(const BatchEntry *E, const int *block_lat, int total_tasks, int j_local,
                              const int *j_base, int gmax, int K, cudaStream_t st)
{
    if (total_tasks <= 0) return cudaSuccess;
    switch (K) {
    case 2: return launch_wave_k<2>(E, block_lat, total_tasks, j_local, j_base, gmax, st);
    case 4: return launch_wave_k<4>(E, block_lat, total_tasks, j_local, j_base, gmax, st);
    case 8: return launch_wave_k<8>(E, block_lat, total_tasks, j_local, j_base, gmax, st);
    default: return cudaErrorInvalidValue;
    }
}

cudaError_t launch_batch_keys(const BatchEntry *E, int n, int max_steps, cudaStream_t st)
{
    const long long work = (long long)n * max_steps;
    if (work <= 0) return cudaSuccess;
    k_batch_keys<<<(unsigned)((work + 255) / 256), 256, 0, st>>>(E, n, max_steps);
    return cudaGetLastError();
}

cudaError_t launch_set_base(int *s_base, int v, cudaStream_t st)
{
    k_set_base<<<1, 32, 0, st>>>(s_base, v);
    return cudaGetLastError();
}

cudaError_t launch_advance(int *s_base, int by, cudaStream_t st)
{
    k_advance<<<1, 32, 0, st>>>(s_base, by);
    return cudaGetLastError();
}

}  // namespace lgca_gpu
