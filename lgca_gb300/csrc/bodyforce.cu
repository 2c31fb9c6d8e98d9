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
// `forcing`.  Candidates are handled in chunks: mark first occurrences
// (atomicMin of k per cell), sum the gains per block, find the block where
// the running total reaches `forcing`, apply.  Kernels of later chunks exit at
// once when an earlier chunk reached the target.
#include "internal.cuh"
#include "../../include/lgca/rng.h"

namespace lgca_gpu {

static constexpr unsigned FULL = 0xffffffffu;
static constexpr int BF_THREADS = 256;
static constexpr int BF_PER_THREAD = 16;
static constexpr long long BF_PER_BLOCK = (long long)BF_THREADS * BF_PER_THREAD;
static constexpr int BF_BLOCKS_PER_CHUNK = 256;
static constexpr long long BF_CHUNK = BF_PER_BLOCK * BF_BLOCKS_PER_CHUNK;

struct BodyForceState {
    unsigned long long total;  // reversals so far
    int done;                  // target reached
    int cross_block;           // block of the current chunk where it was reached (-1: none)
    unsigned long long base;   // total before the current chunk
    unsigned long long cross_total;  // total after the crossing block
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

__global__ void k_bf_mark(BodyForceArgs a, unsigned long long k0)
{
    if (a.st->done) return;
    const unsigned long long base = k0 + (unsigned long long)blockIdx.x * BF_PER_BLOCK;
    for (int j = 0; j < BF_PER_THREAD; ++j) {
        const unsigned long long k = base + (unsigned long long)j * BF_THREADS + threadIdx.x;
        if (k < a.ncand) atomicMin(a.first + bf_cell(a, k), (uint32_t)k);
    }
}

__device__ __forceinline__ int bf_cand_gain(const BodyForceArgs &a, unsigned long long k,
                                            unsigned long long &cell)
{
    if (k >= a.ncand) return 0;
    cell = bf_cell(a, k);
    if (a.first[cell] != (uint32_t)k) return 0;
    return bf_gain(a, cell);
}

__global__ void k_bf_gain(BodyForceArgs a, unsigned long long k0)
{
    if (a.st->done) return;
    __shared__ unsigned warp_sum[BF_THREADS / 32];
    const unsigned long long base = k0 + (unsigned long long)blockIdx.x * BF_PER_BLOCK;
    unsigned s = 0;
    for (int j = 0; j < BF_PER_THREAD; ++j) {
        unsigned long long cell;
        s += (unsigned)bf_cand_gain(a, base + (unsigned long long)j * BF_THREADS + threadIdx.x, cell);
    }
    for (int off = 16; off > 0; off >>= 1) s += __shfl_xor_sync(FULL, s, off);
    if ((threadIdx.x & 31) == 0) warp_sum[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned t = 0;
        for (int i = 0; i < BF_THREADS / 32; ++i) t += warp_sum[i];
        a.block_gain[blockIdx.x] = t;
    }
}

// One block: running total over the chunk's blocks, in order.
__global__ void k_bf_find(BodyForceArgs a, int nblocks)
{
    if (a.st->done) return;
    if (threadIdx.x != 0) return;
    unsigned long long tot = a.st->total;
    a.st->base = tot;
    a.st->cross_block = -1;
    for (int b = 0; b < nblocks; ++b) {
        const unsigned long long nt = tot + a.block_gain[b];
        if (nt >= a.target) {
            a.st->cross_block = b;
            break;
        }
        tot = nt;
    }
}

// Apply the processed candidates of the chunk.  Blocks before the crossing
// block apply every gain; the crossing block orders its candidates with a
// block-wide scan and applies candidate k iff k == 0 or the reversals before
// it are fewer than the target, and records the resulting total.
__global__ void k_bf_apply(BodyForceArgs a, unsigned long long k0)
{
    if (a.st->done) return;
    const int cross = a.st->cross_block;
    if (cross >= 0 && (int)blockIdx.x > cross) return;
    const unsigned long long base = k0 + (unsigned long long)blockIdx.x * BF_PER_BLOCK;
    if ((int)blockIdx.x != cross) {
        for (int j = 0; j < BF_PER_THREAD; ++j) {
            unsigned long long cell;
            if (bf_cand_gain(a, base + (unsigned long long)j * BF_THREADS + threadIdx.x, cell) > 0)
                bf_apply(a, cell);
        }
        return;
    }
    __shared__ unsigned warp_tot[BF_THREADS / 32];
    __shared__ unsigned long long running, applied;
    if (threadIdx.x == 0) {
        unsigned long long t = a.st->base;
        for (int b = 0; b < cross; ++b) t += a.block_gain[b];
        running = t;
        applied = t;
    }
    __syncthreads();
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
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
    if (threadIdx.x == 0) a.st->cross_total = applied;
}

// Close the chunk: update the running total, stop when the target was reached
// or the candidates are exhausted.
__global__ void k_bf_close(BodyForceArgs a, unsigned long long k0, int nblocks)
{
    if (a.st->done || threadIdx.x != 0) return;
    if (a.st->cross_block >= 0) {
        a.st->total = a.st->cross_total;
        a.st->done = 1;
        return;
    }
    unsigned long long t = a.st->base;
    for (int b = 0; b < nblocks; ++b) t += a.block_gain[b];
    a.st->total = t;
    if (k0 + (unsigned long long)nblocks * BF_PER_BLOCK >= a.ncand) a.st->done = 1;
}

size_t body_force_scratch_bytes(size_t num_cells)
{
    return ((num_cells * sizeof(uint32_t) + 255) & ~(size_t)255) +
           BF_BLOCKS_PER_CHUNK * sizeof(unsigned) + sizeof(BodyForceState) + 256;
}

cudaError_t launch_body_force(int model, const PlaneGeom &g, uint64_t *planes,
                              const uint64_t *solid, const uint64_t *slip, uint64_t key,
                              long long forcing, int bf_dir, void *scratch,
                              unsigned long long *reverted_dev, cudaStream_t s)
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
    p += BF_BLOCKS_PER_CHUNK * sizeof(unsigned);
    a.st = reinterpret_cast<BodyForceState *>(p);
    cudaError_t e = cudaMemsetAsync(a.st, 0, sizeof(BodyForceState), s);
    if (e != cudaSuccess) return e;
    if (bf_dir == 'x' || bf_dir == 'y') {
        e = cudaMemsetAsync(a.first, 0xff, ncells * sizeof(uint32_t), s);
        if (e != cudaSuccess) return e;
        for (unsigned long long k0 = 0; k0 < a.ncand; k0 += (unsigned long long)BF_CHUNK) {
            const unsigned long long left = a.ncand - k0;
            const int nb = (int)(left >= (unsigned long long)BF_CHUNK
                                     ? BF_BLOCKS_PER_CHUNK
                                     : (left + BF_PER_BLOCK - 1) / BF_PER_BLOCK);
            k_bf_mark<<<nb, BF_THREADS, 0, s>>>(a, k0);
            k_bf_gain<<<nb, BF_THREADS, 0, s>>>(a, k0);
            k_bf_find<<<1, 32, 0, s>>>(a, nb);
            k_bf_apply<<<nb, BF_THREADS, 0, s>>>(a, k0);
            k_bf_close<<<1, 32, 0, s>>>(a, k0, nb);
        }
    }
    e = cudaMemcpyAsync(reverted_dev, &a.st->total, sizeof(unsigned long long),
                        cudaMemcpyDeviceToDevice, s);
    if (e != cudaSuccess) return e;
    return cudaGetLastError();
}

}  // namespace lgca_gpu
