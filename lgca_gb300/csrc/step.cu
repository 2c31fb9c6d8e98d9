// Plain lattice step (one step per pass over global memory).
//
// Reference: OMP_Lattice<M>::collide_and_propagate, keva92/lgca
// src/omp_lattice.cpp:100-249.  The reference pulls, for every cell and
// channel d, the bit of channel d of the cell at offset_to_neighbor[INV_DIR[d]]
// plus the periodic edge corrections (src/lgca_models.h:79-132 HPP,
// :292-365 / :483-566 / :701-784 FHP).  With an even number of rows those
// tables describe a torus; the source cell of channel d of site (x, y) is
//
//   d   FHP, y even   FHP, y odd    HPP
//   0   (x-1, y)      (x-1, y)      (x-1, y)
//   1   (x-1, y-1)    (x,   y-1)    (x,   y-1)
//   2   (x,   y-1)    (x+1, y-1)    (x+1, y)
//   3   (x+1, y)      (x+1, y)      (x,   y+1)
//   4   (x,   y+1)    (x+1, y+1)
//   5   (x-1, y+1)    (x,   y+1)
//   6   (x,   y)      (x,   y)
//
// all coordinates modulo (W, H).  On bit-planes every channel is read from a
// single row, and an x offset of +-1 is a one-bit shift of the word with the
// missing bit taken from the neighbouring word (a warp shuffle, or a load at
// a warp edge / the periodic x seam).
//
// Mapping: one warp per (row, chunk of 32 words), one word (64 sites) per
// lane.  Each lane loads D words and stores D words; the only other traffic
// is one word per shifted plane at the two warp edges.
#include "internal.cuh"
#include "../../include/lgca/rng.h"

namespace lgca_gpu {

static constexpr unsigned FULL = 0xffffffffu;

// Forcing decision at site (fx, y): a FLUID cell with channel 0 empty and the
// west-moving channel (3 for FHP, 2 for HPP) occupied reverses with
// probability thr / 2^32.  Used by the lanes that fetch the forced word from
// another chunk.
// What changes from one step to the next: the two buffers and the keys.
struct StepIO {
    const uint64_t *__restrict__ src;
    uint64_t *__restrict__ dst;
    uint64_t ckey, fkey;  // chirality / forcing keys of the step
};

template <int MODEL, int GM>
__device__ __forceinline__ uint64_t force_flip_at(const StepArgs &a, const StepIO &io, int y)
{
    constexpr int WEST = (MODEL == M_HPP) ? 2 : 3;
    const int fw = a.fx >> 6, fb = a.fx & 63;
    const unsigned r0 = (unsigned)y * a.g.pitch + fw;
    uint64_t n0 = io.src[r0], nw = io.src[WEST * (unsigned)a.g.ps + r0];
    uint64_t fluid = ~0ull;
    if (GM >= GEOM_NOSLIP) fluid &= ~a.solid[r0];
    if (GM == GEOM_FULL) fluid &= ~a.slip[r0];
    const uint64_t u = lgca_rng_draw(io.fkey, lgca_rng_index((uint32_t)y, (uint32_t)a.fx)) >> 32;
    const uint64_t cand = (~n0 & nw & fluid) >> fb & 1ull;
    return (u < a.force_thr) ? cand : 0ull;
}

template <int MODEL, int GM>
__device__ __forceinline__ void step_word(const StepArgs &a, const StepIO &io, const int y,
                                          const int w, const int lane)
{
    constexpr int D = ModelTraits<MODEL>::D;
    const PlaneGeom &g = a.g;
    const bool active = w < g.nw;
    const int ym = (y == 0) ? g.H - 1 : y - 1;
    const int yp = (y == g.H - 1) ? 0 : y + 1;
    // 32-bit offsets: a lattice has at most 2^31 sites, so D * H * pitch < 2^29 words
    const unsigned rowm = (unsigned)ym * g.pitch, row0 = (unsigned)y * g.pitch,
                   rowp = (unsigned)yp * g.pitch;
    const uint64_t *__restrict__ s = io.src;
    const unsigned ps = (unsigned)g.ps;
    const bool even = (y & 1) == 0;

    // which plane comes from which row (see the table above)
    // HPP: 0 -> row y, 1 -> row y-1, 2 -> row y, 3 -> row y+1
    // FHP: 0,3,6 -> row y, 1,2 -> row y-1, 4,5 -> row y+1
    auto row_of = [&](int d) -> unsigned {
        if (MODEL == M_HPP) return d == 1 ? rowm : (d == 3 ? rowp : row0);
        return (d == 1 || d == 2) ? rowm : ((d == 4 || d == 5) ? rowp : row0);
    };

    uint64_t n[7];
#pragma unroll
    for (int d = 0; d < D; ++d) n[d] = active ? __ldg(s + (d * ps + row_of(d) + w)) : 0ull;

    uint64_t solid = 0, slip = 0;
    if (GM >= GEOM_NOSLIP && active) solid = __ldg(a.solid + row0 + w);
    if (GM == GEOM_FULL && active) slip = __ldg(a.slip + row0 + w);

    // forcing column: applied to the source words before the pull
    constexpr int WEST = (MODEL == M_HPP) ? 2 : 3;
    const bool forcing = a.force_thr != 0;
    if (forcing && active && w == (a.fx >> 6)) {
        const int fb = a.fx & 63;
        const uint64_t u =
            lgca_rng_draw(io.fkey, lgca_rng_index((uint32_t)y, (uint32_t)a.fx)) >> 32;
        const uint64_t fl = (u < a.force_thr) ? ((~n[0] & n[WEST] & ~solid & ~slip) >> fb & 1ull) : 0ull;
        n[0] |= fl << fb;
        n[WEST] &= ~(fl << fb);
    }

    // neighbour words at the warp edges and the periodic x seam
    const bool need_w = active && (lane == 0 || w == 0);
    const bool need_e = active && (lane == 31 || w == g.nw - 1);
    const int widx = (w == 0) ? g.nw - 1 : w - 1;
    const int wbit = (w == 0) ? g.L : 63;
    const int eidx = (w == g.nw - 1) ? 0 : w + 1;
    const int epos = (w == g.nw - 1) ? g.L : 63;
    const int wx = (w == 0) ? g.W - 1 : 64 * w - 1;  // site of the fetched west bit
    const int ex = (w == g.nw - 1) ? 0 : 64 * w + 64; // site of the fetched east bit

    // x-1 pull: (v << 1) | bit of site x-1
    auto shl = [&](uint64_t v, int d, unsigned row) -> uint64_t {
        const uint32_t hi = __shfl_up_sync(FULL, (uint32_t)(v >> 32), 1);
        uint64_t in = hi >> 31;
        if (need_w) {
            in = (__ldg(s + (d * ps + row + widx)) >> wbit) & 1ull;
            if (d == 0 && row == row0 && forcing && wx == a.fx) in |= force_flip_at<MODEL, GM>(a, io, y);
        }
        return (v << 1) | in;
    };
    // x+1 pull: (v >> 1) | bit of site x+1 placed at the last valid bit
    auto shr = [&](uint64_t v, int d, unsigned row) -> uint64_t {
        const uint32_t lo = __shfl_down_sync(FULL, (uint32_t)v, 1);
        uint64_t in = lo & 1u;
        if (need_e) {
            in = __ldg(s + (d * ps + row + eidx)) & 1ull;
            if (d == WEST && row == row0 && forcing && ex == a.fx)
                in &= ~force_flip_at<MODEL, GM>(a, io, y);
        }
        return (v >> 1) | (in << epos);
    };

    uint64_t p[7];
    if (MODEL == M_HPP) {
        p[0] = shl(n[0], 0, row0);
        p[1] = n[1];
        p[2] = shr(n[2], 2, row0);
        p[3] = n[3];
    } else {
        p[0] = shl(n[0], 0, row0);
        p[3] = shr(n[3], 3, row0);
        if (even) {
            p[1] = shl(n[1], 1, rowm);
            p[5] = shl(n[5], 5, rowp);
            p[2] = n[2];
            p[4] = n[4];
        } else {
            p[2] = shr(n[2], 2, rowm);
            p[4] = shr(n[4], 4, rowp);
            p[1] = n[1];
            p[5] = n[5];
        }
        if (D == 7) p[6] = n[6];
    }
    if (!active) return;

    uint64_t c[7];
#pragma unroll
    for (int d = 0; d < D; ++d) c[d] = p[d];
    if (MODEL != M_HPP) {
        const uint64_t chir =
            a.chir ? __ldg(a.chir + row0 + w)
                   : lgca_rng_draw(io.ckey, lgca_rng_index((uint32_t)y, (uint32_t)w));
        collide<MODEL>(c, chir);
    } else {
        collide<MODEL>(c, 0ull);
    }

    uint64_t out[7];
    if (GM == GEOM_NONE) {
#pragma unroll
        for (int d = 0; d < D; ++d) out[d] = c[d];
    } else {
        const uint64_t fluid = ~(solid | slip);
        // slip cells: mirror in x on the first/last row, in y on the first/last
        // column (the latter wins at corners), unchanged elsewhere
        const bool nsrow = (y == 0) || (y == g.H - 1);
        const uint64_t ew = (w == 0 ? 1ull : 0ull) | (w == g.nw - 1 ? (1ull << g.L) : 0ull);
#pragma unroll
        for (int d = 0; d < D; ++d) {
            uint64_t o = (fluid & c[d]) | (solid & p[Dirs<MODEL>::inv(d)]);
            if (GM == GEOM_FULL) {
                const uint64_t sx = nsrow ? p[Dirs<MODEL>::mirx(d)] : p[d];
                const uint64_t sl = (ew & p[Dirs<MODEL>::miry(d)]) | (~ew & sx);
                o |= slip & sl;
            }
            out[d] = o;
        }
    }
    if (w == g.nw - 1) {  // clear the tail bits past site W-1
#pragma unroll
        for (int d = 0; d < D; ++d) out[d] &= g.lastmask;
    }
    uint64_t *__restrict__ dp = io.dst + row0 + w;
#pragma unroll
    for (int d = 0; d < D; ++d) dp[d * ps] = out[d];
}

// Grid: x = 32-word chunk of a row, y = group of STEP_WARPS rows; one warp
// per (row, chunk).
static constexpr int STEP_WARPS = 8;

template <int MODEL, int GM>
__global__ void __launch_bounds__(32 * STEP_WARPS) k_step(const StepArgs a)
{
    const int y = blockIdx.y * STEP_WARPS + threadIdx.y;
    if (y >= a.g.H) return;  // whole warp
    const StepIO io{a.src, a.dst, a.chir_key, a.force_key};
    step_word<MODEL, GM>(a, io, y, blockIdx.x * 32 + threadIdx.x, threadIdx.x);
}

template <int MODEL>
static cudaError_t launch_model(int gm, const StepArgs &a, cudaStream_t st)
{
    const dim3 block(32, STEP_WARPS);
    const dim3 grid((unsigned)a.chunks, (unsigned)((a.g.H + STEP_WARPS - 1) / STEP_WARPS));
    if (grid.y > 65535u) return cudaErrorInvalidConfiguration;
    switch (gm) {
    case GEOM_NONE: k_step<MODEL, GEOM_NONE><<<grid, block, 0, st>>>(a); break;
    case GEOM_NOSLIP: k_step<MODEL, GEOM_NOSLIP><<<grid, block, 0, st>>>(a); break;
    default: k_step<MODEL, GEOM_FULL><<<grid, block, 0, st>>>(a); break;
    }
    return cudaGetLastError();
}

// ------------------------------------------------------------------
// Persistent form: one cooperative launch advances nsteps steps, the blocks
// meeting at a grid-wide barrier between steps.  For lattices that fit in L2
// this removes the per-step launch, ramp-up and tail of the one-step kernel.

__device__ __forceinline__ uint64_t globaltimer_ns()
{
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Barrier over all blocks of a cooperative launch (all co-resident).  The
// wait is bounded: a block that waits longer than PERSIST_WAIT_NS, or sees
// the error flag, records the error and returns false; the kernel then stops
// and the host reports LGCA_ERR_TIMEOUT.
static constexpr uint64_t PERSIST_WAIT_NS = 2000000000ull;

__device__ bool grid_barrier(PersistSync *sy, unsigned nblocks)
{
    __shared__ int ok;
    __syncthreads();
    if (threadIdx.x == 0 && threadIdx.y == 0) {
        ok = 1;
        volatile unsigned *vgen = &sy->gen;
        volatile int *verr = &sy->err;
        const unsigned g = *vgen;
        __threadfence();
        const unsigned arrived = atomicAdd(&sy->count, 1u);
        if (arrived == nblocks - 1) {
            atomicExch(&sy->count, 0u);
            __threadfence();
            atomicAdd(&sy->gen, 1u);
        } else {
            const uint64_t t0 = globaltimer_ns();
            while (*vgen == g) {
                if (*verr) { ok = 0; break; }
                if (globaltimer_ns() - t0 > PERSIST_WAIT_NS) {
                    atomicExch(&sy->err, 1);
                    ok = 0;
                    break;
                }
                __nanosleep(64);
            }
        }
        __threadfence();
    }
    __syncthreads();
    return ok != 0;
}

template <int MODEL, int GM>
__global__ void __launch_bounds__(32 * STEP_WARPS) k_persist(const StepArgs a, uint64_t *buf0,
                                                             uint64_t *buf1, uint64_t seed,
                                                             uint64_t t0, int nsteps,
                                                             PersistSync *sy)
{
    __shared__ uint64_t keys[2];
    const unsigned nblocks = gridDim.x;
    const int lane = threadIdx.x;
    const int gwarp = blockIdx.x * STEP_WARPS + threadIdx.y;
    const int nwarps = gridDim.x * STEP_WARPS;
    const int tasks = a.g.H * a.chunks;
    if (threadIdx.x == 0 && threadIdx.y == 0) {
        keys[0] = lgca_rng_key(seed, LGCA_STREAM_CHIR, t0);
        keys[1] = lgca_rng_key(seed, LGCA_STREAM_FORCE, t0);
    }
    __syncthreads();
    for (int s = 0; s < nsteps; ++s) {
        const StepIO io{(s & 1) ? buf1 : buf0, (s & 1) ? buf0 : buf1, keys[0], keys[1]};
        for (int task = gwarp; task < tasks; task += nwarps) {
            const int y = task / a.chunks;
            const int chunk = task - y * a.chunks;
            step_word<MODEL, GM>(a, io, y, chunk * 32 + lane, lane);
        }
        if (s + 1 == nsteps) break;
        __syncthreads();  // everyone has read this step's keys
        if (threadIdx.x == 0 && threadIdx.y == 0) {
            keys[0] = lgca_rng_key(seed, LGCA_STREAM_CHIR, t0 + s + 1);
            keys[1] = lgca_rng_key(seed, LGCA_STREAM_FORCE, t0 + s + 1);
        }
        if (!grid_barrier(sy, nblocks)) return;
    }
}

template <int MODEL, int GM>
static cudaError_t persist_launch(const StepArgs &a, uint64_t *buf0, uint64_t *buf1, uint64_t seed,
                                  uint64_t t0, int nsteps, PersistSync *sy, cudaStream_t st)
{
    auto kern = k_persist<MODEL, GM>;
    int dev = 0, nsm = 0, per_sm = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    if (e == cudaSuccess)
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, 32 * STEP_WARPS, 0);
    if (e != cudaSuccess) return e;
    if (per_sm < 1) return cudaErrorLaunchOutOfResources;
    const int tasks = a.g.H * a.chunks;
    int blocks = nsm * per_sm;
    const int need = (tasks + STEP_WARPS - 1) / STEP_WARPS;
    if (blocks > need) blocks = need;
    StepArgs aa = a;
    void *args[] = {(void *)&aa, (void *)&buf0, (void *)&buf1, (void *)&seed,
                    (void *)&t0, (void *)&nsteps, (void *)&sy};
    return cudaLaunchCooperativeKernel((void *)kern, dim3(blocks), dim3(32, STEP_WARPS), args, 0,
                                       st);
}

template <int MODEL>
static cudaError_t persist_model(int gm, const StepArgs &a, uint64_t *b0, uint64_t *b1,
                                 uint64_t seed, uint64_t t0, int n, PersistSync *sy,
                                 cudaStream_t st)
{
    switch (gm) {
    case GEOM_NONE: return persist_launch<MODEL, GEOM_NONE>(a, b0, b1, seed, t0, n, sy, st);
    case GEOM_NOSLIP: return persist_launch<MODEL, GEOM_NOSLIP>(a, b0, b1, seed, t0, n, sy, st);
    default: return persist_launch<MODEL, GEOM_FULL>(a, b0, b1, seed, t0, n, sy, st);
    }
}

cudaError_t launch_persistent(int model, int gm, const StepArgs &a, uint64_t *buf0, uint64_t *buf1,
                              uint64_t seed, uint64_t t0, int nsteps, PersistSync *sy,
                              cudaStream_t st)
{
    if ((long long)a.g.H * a.chunks > 0x7fffffffLL) return cudaErrorInvalidValue;
    switch (model) {
    case M_HPP: return persist_model<M_HPP>(gm, a, buf0, buf1, seed, t0, nsteps, sy, st);
    case M_FHP_I: return persist_model<M_FHP_I>(gm, a, buf0, buf1, seed, t0, nsteps, sy, st);
    default: return persist_model<M_FHP_II>(gm, a, buf0, buf1, seed, t0, nsteps, sy, st);
    }
}

cudaError_t launch_step(int model, int gm, const StepArgs &a, cudaStream_t st)
{
    switch (model) {
    case M_HPP: return launch_model<M_HPP>(gm, a, st);
    case M_FHP_I: return launch_model<M_FHP_I>(gm, a, st);
    default: return launch_model<M_FHP_II>(gm, a, st);  // FHP-II and FHP-III share one rule set
    }
}

}  // namespace lgca_gpu
