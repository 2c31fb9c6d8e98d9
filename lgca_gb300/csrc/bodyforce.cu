// Random-cell body force with the reference's sequential semantics.
//
// Reference: OMP_Lattice<M>::apply_body_force, keva92/lgca
// src/omp_lattice.cpp:254-346.  The reference draws cells one after the other
// (rand() % num_cells, here candidate k of the FSEQ stream), skips non-FLUID
// cells, reverses a particle where the rule allows and stops once `forcing`
// particles were reverted (checked after each draw, so the first draw is
// always processed) or after 2*num_cells draws.
//
// Parallel form: a cell's rule can only succeed at its first draw -- after a
// reversal the condition is false, after a failed test the cell is unchanged
// -- so candidate k reverts gain(cell_k) particles (0, 1 or 2, evaluated on
// the initial state) iff it is the first occurrence of its cell, and it is
// processed iff k == 0 or the reversals of candidates 0..k-1 are fewer than
// `forcing`.
//
// One cooperative launch walks the candidates in chunks of (blocks x 4096)
// and stops at the chunk where the running total reaches `forcing`, so the
// work follows the target, not the lattice size.  Per chunk: mark first
// occurrences (atomicMin of k per cell in a table of one word per cell),
// barrier, sum the gains per block, barrier, block 0 scans the block sums and
// finds the block where the total reaches the target, barrier, apply (the
// crossing block orders its candidates with a block-wide scan), barrier.
// At the end the table entries of the candidates drawn are reset, so the
// table is all ones between calls and no call clears the whole table; a call
// that finds the table not marked clean (the first call on fresh memory, a
// call on more cells than the last, or after a call that stopped early)
// clears it first.  Grid barriers are bounded: a wait past BF_WAIT_NS sets
// the error flag and every block returns.
#include "internal.cuh"
#include "../../include/lgca/rng.h"

#include <algorithm>

namespace lgca_gpu {

static constexpr unsigned FULL = 0xffffffffu;
static constexpr int BF_THREADS = 256;
static constexpr int BF_PER_THREAD = 16;
static constexpr long long BF_PER_BLOCK = (long long)BF_THREADS * BF_PER_THREAD;
static constexpr int BF_MAX_BLOCKS = 512;
static constexpr uint64_t BF_WAIT_NS = 2000000000ull;

// Per-call state, zeroed by the launcher before the kernel.
struct BodyForceState {
    unsigned long long total;  // reversals so far
    unsigned long long base;   // total before the current chunk
    unsigned int bar;          // grid-barrier arrivals
    int cross_block;           // block of the current chunk where the target is reached (-1: none)
    int done;                  // no further chunk
    int err;                   // a barrier wait gave up
};
// Kept across calls at a fixed place: the first `clean_cells` table entries
// hold all ones.
struct BodyForceSticky {
    unsigned long long clean_cells;
};

struct BodyForceArgs {
    PlaneGeom g;
    uint64_t *planes;
    const uint64_t *solid, *slip;
    uint64_t key;
    unsigned long long ncells, ncand;
    unsigned long long target;  // (unsigned) forcing
    int model, dir;             // dir: 'x' or 'y'
    uint32_t *first;
    unsigned *block_gain;
    BodyForceState *st;
    BodyForceSticky *sticky;
    unsigned long long *reverted;  // device: the reversals (all ones after an error)
    int *err_out;                  // optional: set to 1 after an error
};

__device__ __forceinline__ unsigned long long bf_cell(const BodyForceArgs &a, unsigned long long k)
{
    return (unsigned long long)(int)(lgca_rng_draw(a.key, k) >> 33) % a.ncells;
}

__device__ __forceinline__ int bf_gain(const BodyForceArgs &a, unsigned long long cell)
{
    const int y = (int)(cell / (unsigned)a.g.W), x = (int)(cell - (unsigned long long)y * a.g.W);
    const size_t o = (size_t)y * a.g.pitch + (x >> 6);
    const int b = x & 63;
    if (a.solid && ((a.solid[o] >> b) & 1ull)) return 0;
    if (a.slip && ((a.slip[o] >> b) & 1ull)) return 0;
    // the cell's own bits are unchanged until its candidate applies them
    auto bit = [&](int d) -> int { return (int)((a.planes[(size_t)d * a.g.ps + o] >> b) & 1ull); };
    if (a.model == M_HPP) {
        if (a.dir == 'x') return (!bit(0) && bit(2)) ? 1 : 0;
        return (bit(1) && !bit(3)) ? 1 : 0;
    }
    if (a.dir == 'x') return (!bit(0) && bit(3)) ? 1 : 0;
    return ((bit(1) && !bit(5)) ? 1 : 0) + ((bit(2) && !bit(4)) ? 1 : 0);
}

__device__ __forceinline__ void bf_apply(const BodyForceArgs &a, unsigned long long cell)
{
    const int y = (int)(cell / (unsigned)a.g.W), x = (int)(cell - (unsigned long long)y * a.g.W);
    const size_t o = (size_t)y * a.g.pitch + (x >> 6);
    const unsigned long long m = 1ull << (x & 63);
    auto plane = [&](int d) -> unsigned long long * {
        return reinterpret_cast<unsigned long long *>(a.planes + (size_t)d * a.g.ps + o);
    };
    auto bit = [&](int d) -> bool { return (*plane(d) & m) != 0; };
    if (a.model == M_HPP) {
        if (a.dir == 'x') { atomicOr(plane(0), m); atomicAnd(plane(2), ~m); }
        else { atomicAnd(plane(1), ~m); atomicOr(plane(3), m); }
        return;
    }
    if (a.dir == 'x') { atomicOr(plane(0), m); atomicAnd(plane(3), ~m); return; }
    const bool f15 = bit(1) && !bit(5), f24 = bit(2) && !bit(4);
    if (f15) { atomicAnd(plane(1), ~m); atomicOr(plane(5), m); }
    if (f24) { atomicAnd(plane(2), ~m); atomicOr(plane(4), m); }
}

// Gain of candidate k if it is the first occurrence of its cell.  The table
// is read through L2: other blocks' atomicMin of this chunk may have changed
// a line this SM's L1 still holds from an earlier chunk.
__device__ __forceinline__ int bf_cand_gain(const BodyForceArgs &a, unsigned long long k,
                                            unsigned long long &cell)
{
    if (k >= a.ncand) return 0;
    cell = bf_cell(a, k);
    if (__ldcg(a.first + cell) != (uint32_t)k) return 0;
    return bf_gain(a, cell);
}

__device__ __forceinline__ uint64_t bf_clock_ns()
{
    uint64_t t = 0;
#ifdef __CUDA_ARCH__
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
#endif
    return t;
}

// Grid barrier number `n` (1, 2, ...): every block arrives once per barrier.
// (Cooperative launch: all blocks are resident, so every wait ends unless a
// block stopped; the time limit covers that case.)  Returns false when the
// wait gave up or another block reported an error.
__device__ bool bf_barrier(const BodyForceArgs &a, unsigned n)
{
    __shared__ int ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        atomicAdd(&a.st->bar, 1u);
        volatile unsigned *bar = &a.st->bar;
        volatile int *err = &a.st->err;
        const unsigned want = n * gridDim.x;
        const uint64_t t0 = bf_clock_ns();
        ok = 1;
        while (*bar < want) {
            if (*err || bf_clock_ns() - t0 > BF_WAIT_NS) {
                atomicExch(&a.st->err, 1);
                ok = 0;
                break;
            }
            __nanosleep(64);
        }
        __threadfence();
    }
    __syncthreads();
    return ok != 0;
}

// The whole call; false when a grid barrier gave up.
__device__ bool bf_run(const BodyForceArgs &a)
{
    __shared__ unsigned warp_tot[BF_THREADS / 32];
    __shared__ unsigned long long running, applied;
    __shared__ int clean;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const unsigned long long chunk = (unsigned long long)gridDim.x * BF_PER_BLOCK;
    unsigned nbar = 0;
    if (threadIdx.x == 0)
        clean = *(volatile unsigned long long *)&a.sticky->clean_cells >= a.ncells ? 1 : 0;
    __syncthreads();
    if (!clean) {  // set the table to all ones
        const unsigned long long stride = (unsigned long long)gridDim.x * BF_THREADS;
        for (unsigned long long i = (unsigned long long)blockIdx.x * BF_THREADS + threadIdx.x;
             i < a.ncells; i += stride)
            a.first[i] = 0xffffffffu;
    }
    if (!bf_barrier(a, ++nbar)) return false;
    // until the last barrier the table is not clean (a stop in between leaves it dirty)
    if (blockIdx.x == 0 && threadIdx.x == 0) a.sticky->clean_cells = 0;

    unsigned long long k0;
    for (k0 = 0; k0 < a.ncand; k0 += chunk) {
        const unsigned long long base = k0 + (unsigned long long)blockIdx.x * BF_PER_BLOCK;
        // ---- mark first occurrences
        for (int j = 0; j < BF_PER_THREAD; ++j) {
            const unsigned long long k = base + (unsigned long long)j * BF_THREADS + threadIdx.x;
            if (k < a.ncand) atomicMin(a.first + bf_cell(a, k), (uint32_t)k);
        }
        if (!bf_barrier(a, ++nbar)) return false;
        // ---- gains per block
        {
            unsigned s = 0;
            for (int j = 0; j < BF_PER_THREAD; ++j) {
                unsigned long long cell;
                s += (unsigned)bf_cand_gain(a, base + (unsigned long long)j * BF_THREADS + threadIdx.x,
                                            cell);
            }
            for (int off = 16; off > 0; off >>= 1) s += __shfl_xor_sync(FULL, s, off);
            if (lane == 0) warp_tot[wid] = s;
            __syncthreads();
            if (threadIdx.x == 0) {
                unsigned t = 0;
                for (int i = 0; i < BF_THREADS / 32; ++i) t += warp_tot[i];
                a.block_gain[blockIdx.x] = t;
            }
        }
        if (!bf_barrier(a, ++nbar)) return false;
        // ---- block 0: running total over the chunk's blocks, in order
        if (blockIdx.x == 0) {
            __shared__ unsigned long long part[BF_THREADS];
            __shared__ int cross;
            const unsigned long long before = *(volatile unsigned long long *)&a.st->total;
            // two block sums per thread (gridDim.x <= 2 * BF_THREADS)
            const int b0 = 2 * threadIdx.x, b1 = b0 + 1;
            const unsigned g0 = b0 < (int)gridDim.x ? __ldcg(a.block_gain + b0) : 0u;
            const unsigned g1 = b1 < (int)gridDim.x ? __ldcg(a.block_gain + b1) : 0u;
            part[threadIdx.x] = (unsigned long long)g0 + g1;
            if (threadIdx.x == 0) cross = 0x7fffffff;
            __syncthreads();
            for (int off = 1; off < BF_THREADS; off <<= 1) {  // inclusive scan of the pairs
                const unsigned long long v = threadIdx.x >= off ? part[threadIdx.x - off] : 0ull;
                __syncthreads();
                part[threadIdx.x] += v;
                __syncthreads();
            }
            const unsigned long long excl = before + (threadIdx.x ? part[threadIdx.x - 1] : 0ull);
            // the first block whose inclusive total reaches the target
            int my = -1;
            if (b0 < (int)gridDim.x && excl + g0 >= a.target) my = b0;
            else if (b1 < (int)gridDim.x && excl + g0 + g1 >= a.target) my = b1;
            if (my >= 0) atomicMin(&cross, my);
            __syncthreads();
            if (threadIdx.x == 0) {
                const int c = cross == 0x7fffffff ? -1 : cross;
                a.st->base = before;
                a.st->cross_block = c;
                if (c < 0) a.st->total = before + part[BF_THREADS - 1];
                a.st->done = (c >= 0 || k0 + chunk >= a.ncand) ? 1 : 0;
            }
        }
        if (!bf_barrier(a, ++nbar)) return false;
        // ---- apply: blocks before the crossing block apply every gain; the
        // crossing block applies candidate k iff k == 0 or the reversals
        // before it are fewer than the target, and records the total
        {
            const int cross = *(volatile int *)&a.st->cross_block;
            if (cross < 0 || (int)blockIdx.x < cross) {
                for (int j = 0; j < BF_PER_THREAD; ++j) {
                    unsigned long long cell;
                    if (bf_cand_gain(a, base + (unsigned long long)j * BF_THREADS + threadIdx.x, cell) > 0)
                        bf_apply(a, cell);
                }
            } else if ((int)blockIdx.x == cross) {
                if (threadIdx.x == 0) {
                    unsigned long long t = *(volatile unsigned long long *)&a.st->base;
                    for (int b = 0; b < cross; ++b) t += __ldcg(a.block_gain + b);
                    running = t;
                    applied = t;
                }
                __syncthreads();
                for (int j = 0; j < BF_PER_THREAD; ++j) {
                    const unsigned long long k = base + (unsigned long long)j * BF_THREADS + threadIdx.x;
                    unsigned long long cell = 0;
                    const unsigned gk = (unsigned)bf_cand_gain(a, k, cell);
                    unsigned incl = gk;  // inclusive scan in candidate order
                    for (int off = 1; off < 32; off <<= 1) {
                        const unsigned v = __shfl_up_sync(FULL, incl, off);
                        if (lane >= off) incl += v;
                    }
                    if (lane == 31) warp_tot[wid] = incl;
                    __syncthreads();
                    unsigned before = 0, all = 0;
                    for (int i = 0; i < BF_THREADS / 32; ++i) {
                        if (i < wid) before += warp_tot[i];
                        all += warp_tot[i];
                    }
                    const unsigned long long excl = running + before + incl - gk;
                    if (gk > 0 && (k == 0 || excl < a.target)) {
                        bf_apply(a, cell);
                        atomicAdd(&applied, (unsigned long long)gk);
                    }
                    __syncthreads();
                    if (threadIdx.x == 0) running += all;
                    __syncthreads();
                }
                if (threadIdx.x == 0) a.st->total = applied;
            }
        }
        if (!bf_barrier(a, ++nbar)) return false;
        if (*(volatile int *)&a.st->done) break;
    }
    // ---- reset the table entries of every candidate drawn
    {
        const unsigned long long kend = k0 + chunk < a.ncand ? k0 + chunk : a.ncand;
        const unsigned long long stride = (unsigned long long)gridDim.x * BF_THREADS;
        for (unsigned long long k = (unsigned long long)blockIdx.x * BF_THREADS + threadIdx.x; k < kend;
             k += stride)
            a.first[bf_cell(a, k)] = 0xffffffffu;
    }
    if (!bf_barrier(a, ++nbar)) return false;
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        a.sticky->clean_cells = a.ncells;
        *a.reverted = *(volatile unsigned long long *)&a.st->total;
    }
    return true;
}

__global__ void __launch_bounds__(BF_THREADS) k_body_force(BodyForceArgs a)
{
    if (!bf_run(a) && blockIdx.x == 0 && threadIdx.x == 0) {
        *a.reverted = ~0ull;
        if (a.err_out) atomicOr(a.err_out, 1);
    }
}

size_t body_force_scratch_bytes(size_t num_cells)
{
    return ((num_cells * sizeof(uint32_t) + 255) & ~(size_t)255) + BF_MAX_BLOCKS * sizeof(unsigned) +
           256;
}

cudaError_t launch_body_force(int model, const PlaneGeom &g, uint64_t *planes,
                              const uint64_t *solid, const uint64_t *slip, uint64_t key,
                              long long forcing, int bf_dir, void *scratch, void *sticky,
                              unsigned long long *reverted_dev, int *err_out, cudaStream_t s)
{
    const unsigned long long ncells = (unsigned long long)g.W * (unsigned long long)g.H;
    BodyForceArgs a;
    a.g = g;
    a.planes = planes;
    a.solid = solid;
    a.slip = slip;
    a.key = key;
    a.ncells = ncells;
    a.ncand = 2ull * ncells;
    a.target = (unsigned long long)(unsigned)(int)forcing;
    a.model = model;
    a.dir = bf_dir;
    char *p = static_cast<char *>(scratch);
    a.first = reinterpret_cast<uint32_t *>(p);
    p += (ncells * sizeof(uint32_t) + 255) & ~(size_t)255;
    a.block_gain = reinterpret_cast<unsigned *>(p);
    p += BF_MAX_BLOCKS * sizeof(unsigned);
    a.st = reinterpret_cast<BodyForceState *>(p);
    a.sticky = static_cast<BodyForceSticky *>(sticky);
    a.reverted = reverted_dev;
    a.err_out = err_out;
    static_assert(sizeof(BodyForceState) <= 256, "body-force state fits its 256 bytes");
    static_assert(sizeof(BodyForceSticky) <= BODY_FORCE_STICKY_BYTES, "sticky state size");
    if (!(bf_dir == 'x' || bf_dir == 'y'))
        return cudaMemsetAsync(reverted_dev, 0, sizeof(unsigned long long), s);
    cudaError_t e = cudaMemsetAsync(a.st, 0, sizeof(BodyForceState), s);
    if (e != cudaSuccess) return e;
    // one cooperative launch: every block resident at once (grid barriers)
    int dev = 0, nsm = 0, per_sm = 0;
    if ((e = cudaGetDevice(&dev)) != cudaSuccess) return e;
    if ((e = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) return e;
    if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_body_force, BF_THREADS, 0)) !=
        cudaSuccess)
        return e;
    if (per_sm < 1) return cudaErrorLaunchOutOfResources;
    long long blocks = std::min<long long>((long long)per_sm * nsm, BF_MAX_BLOCKS);
    blocks = std::min<long long>(blocks, (long long)((a.ncand + BF_PER_BLOCK - 1) / BF_PER_BLOCK));
    blocks = std::max<long long>(blocks, 1);
    void *args[] = {(void *)&a};
    return cudaLaunchCooperativeKernel((void *)k_body_force, dim3((unsigned)blocks), dim3(BF_THREADS),
                                       args, 0, s);
}

}  // namespace lgca_gpu
