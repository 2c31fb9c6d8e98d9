// One-step kernels (one word or two words per lane), the persistent band
// kernel and their launchers.  The per-word step itself (pull table,
// forcing, collision, boundaries) is in step_body.cuh.
#include "step_body.cuh"

#include <cmath>

namespace lgca_gpu {

static constexpr int STEP_WARPS = 8;  // largest block: 8 warps

// Grid: 1-D, blockDim.y warps per block; warp task = blockIdx.x * blockDim.y
// + threadIdx.y in the flattened same-parity mapping (flat_site).
template <int MODEL, int GM>
__global__ void __launch_bounds__(32 * STEP_WARPS) k_step(const __grid_constant__ StepArgs a)
{
    pdl_launch_dependents();
    const long long task = (long long)blockIdx.x * blockDim.y + threadIdx.y;
    if (task >= flat_tasks(a.g.H, a.g.nw)) return;  // whole warp
    int y, w;
    flat_site(task, threadIdx.x, a.g.H, a.g.nw, a.fmagic, y, w);
    // the chirality word does not depend on the previous step: draw it first
    uint64_t ch = 0;
    if (MODEL != M_HPP && a.chir == nullptr)
        ch = lgca_rng_draw(a.chir_key, lgca_rng_index((uint32_t)y, (uint32_t)w));
    const StepIO io{a.src, a.dst, a.chir_key, a.force_key};
    pdl_wait();
    step_word<MODEL, GM, true, true>(a, io, y, w, threadIdx.x, 32, ch);
}

template <int MODEL, int GM, bool ODD>
__global__ void __launch_bounds__(32 * STEP_WARPS) k_step2(const __grid_constant__ StepArgs a)
{
    pdl_launch_dependents();
    const int np = (a.g.nw + 1) >> 1;
    const long long task = (long long)blockIdx.x * blockDim.y + threadIdx.y;
    if (task >= flat_tasks(a.g.H, np)) return;
    int y, t;
    flat_site(task, threadIdx.x, a.g.H, np, a.fmagic, y, t);
    uint64_t c0 = 0, c1 = 0;
    if (MODEL != M_HPP && a.chir == nullptr) {
        // draws of words 2t and 2t+1: mix(key + index * gamma), indices 1 apart
        const uint64_t z = a.chir_key + lgca_rng_index((uint32_t)y, (uint32_t)(2 * t)) * LGCA_RNG_GAMMA;
        c0 = lgca_mix64(z);
        c1 = lgca_mix64(z + LGCA_RNG_GAMMA);
    }
    const StepIO io{a.src, a.dst, a.chir_key, a.force_key};
    pdl_wait();
    step_pair<MODEL, GM, true, true, ODD>(a, io, y, t, threadIdx.x, 32, c0, c1);
}

int sm_count()
{
    static int cache[64] = {};
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev < 0 || dev >= 64) return 1;
    if (!cache[dev]) {
        int n = 0;
        cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
        cache[dev] = n > 0 ? n : 1;
    }
    return cache[dev];
}

// Warps per block: the caller's choice, else 4, 8 or 2 (in that order of
// preference) by how evenly the grid's blocks spread over the SMs (the
// busiest SM gets ceil(blocks / SMs) blocks; the efficiency is the mean over
// that).  Timed on GB300: 4 is best or within 2 % on large and L2-resident
// lattices; 2 wins on small ones that fill a fraction of the SMs.
static int pick_warps(int requested, long long chunks, long long warp_rows)
{
    if (requested == 1 || requested == 2 || requested == 4 || requested == 8) return requested;
    const double sms = (double)sm_count();
    // A grid resident in one wave (at most 32 warps per SM) that still gives
    // every SM three or more 8-warp blocks steps fastest in 8-warp blocks:
    // half the blocks to schedule per step, and the step is short enough for
    // that to show (FHP-III 8192x2048 and 4096x4096: 4.86 and 4.59 us per
    // step, against 5.05 and 4.70 us with 4-warp blocks).
    const double warps = (double)chunks * (double)warp_rows;
    if (warps >= 24.0 * sms && warps <= 32.0 * sms) return 8;
    int best = 4;
    double best_eff = -1.0;
    for (const int bw : {4, 8, 2}) {
        const double per_sm = (double)(chunks * ((warp_rows + bw - 1) / bw)) / sms;
        const double eff = per_sm / std::ceil(per_sm);
        if (eff > best_eff + 0.02) {
            best = bw;
            best_eff = eff;
        }
    }
    return best;
}

template <int MODEL>
static cudaError_t launch_model2(int gm, const StepArgs &args, cudaStream_t st)
{
    StepArgs a = args;
    const int np = (a.g.nw + 1) / 2;  // word pairs per row (the last may be half)
    a.fmagic = flat_magic(a.g.H, np);
    const long long tasks = flat_tasks(a.g.H, np);
    const int bw = pick_warps(a.bw, 1, tasks);
    const long long blocks = (tasks + bw - 1) / bw;
    if (blocks > 0x7fffffffLL) return cudaErrorInvalidConfiguration;
    const dim3 grid((unsigned)blocks), block(32, bw);
    if (a.g.nw & 1) {
        switch (gm) {
        case GEOM_NONE: return launch_pdl(k_step2<MODEL, GEOM_NONE, true>, grid, block, 0, st, a);
        case GEOM_NOSLIP: return launch_pdl(k_step2<MODEL, GEOM_NOSLIP, true>, grid, block, 0, st, a);
        default: return launch_pdl(k_step2<MODEL, GEOM_FULL, true>, grid, block, 0, st, a);
        }
    }
    switch (gm) {
    case GEOM_NONE: return launch_pdl(k_step2<MODEL, GEOM_NONE, false>, grid, block, 0, st, a);
    case GEOM_NOSLIP: return launch_pdl(k_step2<MODEL, GEOM_NOSLIP, false>, grid, block, 0, st, a);
    default: return launch_pdl(k_step2<MODEL, GEOM_FULL, false>, grid, block, 0, st, a);
    }
}

template <int MODEL>
static cudaError_t launch_model(int gm, const StepArgs &args, cudaStream_t st)
{
    if (args.wpt == 2 && (args.g.W % 64) == 0)
        return launch_model2<MODEL>(gm, args, st);
    StepArgs a = args;
    a.fmagic = flat_magic(a.g.H, a.g.nw);
    const long long tasks = flat_tasks(a.g.H, a.g.nw);
    const int bw = pick_warps(a.bw, 1, tasks);
    const long long blocks = (tasks + bw - 1) / bw;
    if (blocks > 0x7fffffffLL) return cudaErrorInvalidConfiguration;
    const dim3 grid((unsigned)blocks), block(32, bw);
    switch (gm) {
    case GEOM_NONE: return launch_pdl(k_step<MODEL, GEOM_NONE>, grid, block, 0, st, a);
    case GEOM_NOSLIP: return launch_pdl(k_step<MODEL, GEOM_NOSLIP>, grid, block, 0, st, a);
    default: return launch_pdl(k_step<MODEL, GEOM_FULL>, grid, block, 0, st, a);
    }
}

// ------------------------------------------------------------------
// Persistent band form: one cooperative launch advances nsteps steps.  Block
// b (one per SM) owns the rows of band b and steps them; a step of band b
// needs only the edge rows of bands b-1 and b+1 from the previous step, and
// must not overwrite the previous-step rows those bands still read.  So
// after each step a block publishes its step count and waits for its two
// neighbours to reach the same count -- no grid-wide barrier.  The waits are
// bounded: past wait_ns nanoseconds, or when another block reported a
// timeout, a block records the error in *err and stops; the host reports
// LGCA_ERR_TIMEOUT.  *err is sticky: a launch that finds it set does nothing,
// so the steps queued behind a failed call do not run on a partial state.
// `withhold` names a block that never publishes its step (-1: none), so that
// a test can make its neighbours' waits run out; every wait still ends.

__device__ __forceinline__ uint64_t globaltimer_ns()
{
    uint64_t t = 0;
#ifdef __CUDA_ARCH__  // (host builds of the kernel bodies for the CPU emulation read 0)
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
#endif
    return t;
}

template <int MODEL, int GM, int WPT>
__global__ void k_band(const __grid_constant__ StepArgs a, uint64_t *buf0, uint64_t *buf1,
                       uint64_t seed, uint64_t t0, int nsteps, int *flags, int *err,
                       uint64_t wait_ns, int withhold)
{
    __shared__ uint64_t keys[2];
    __shared__ int stop;
    const int nb = gridDim.x, b = blockIdx.x;
    const int bl = (b + nb - 1) % nb, br = (b + 1) % nb;
    const int y0 = (int)((long long)a.g.H * b / nb), y1 = (int)((long long)a.g.H * (b + 1) / nb);
    const int per_row = WPT == 2 ? ((a.g.nw + 1) / 2 + 31) / 32 : (a.g.nw + 31) / 32;
    const int tasks = (y1 - y0) * per_row;
    const int lane = threadIdx.x, warp = threadIdx.y, nwarps = blockDim.y;
    const bool leader = lane == 0 && warp == 0;
    if (leader) {
        keys[0] = lgca_rng_key(seed, LGCA_STREAM_CHIR, t0);
        keys[1] = lgca_rng_key(seed, LGCA_STREAM_FORCE, t0);
        stop = *(volatile int *)err;  // an earlier call gave up: do not step a partial state
    }
    __syncthreads();
    if (stop) return;  // (block-uniform)
    for (int s = 0; s < nsteps; ++s) {
        const StepIO io{(s & 1) ? buf1 : buf0, (s & 1) ? buf0 : buf1, keys[0], keys[1]};
        for (int task = warp; task < tasks; task += nwarps) {
            const int y = y0 + task / per_row, c = task % per_row;
            if (WPT == 2) step_pair<MODEL, GM, true>(a, io, y, c * 32 + lane, lane);
            else step_word<MODEL, GM, true>(a, io, y, c * 32 + lane, lane);
        }
        if (s + 1 == nsteps) break;
        __syncthreads();  // the band's step s is written; keys[] no longer read
        if (leader) {
            __threadfence();
            if (b != withhold) atomicExch(flags + b, s + 1);
            volatile int *vf = flags;
            volatile int *verr = err;
            const uint64_t tw = globaltimer_ns();
            while (vf[bl] < s + 1 || vf[br] < s + 1) {
                if (*verr || globaltimer_ns() - tw > wait_ns) {
                    atomicExch(err, 1);
                    stop = 1;
                    break;
                }
                __nanosleep(32);
            }
            __threadfence();
            keys[0] = lgca_rng_key(seed, LGCA_STREAM_CHIR, t0 + s + 1);
            keys[1] = lgca_rng_key(seed, LGCA_STREAM_FORCE, t0 + s + 1);
        }
        __syncthreads();
        if (stop) return;
    }
}

template <int MODEL, int GM, int WPT>
static cudaError_t band_launch(const StepArgs &a, uint64_t *buf0, uint64_t *buf1, uint64_t seed,
                               uint64_t t0, int nsteps, int *flags, int *err, int max_blocks,
                               const PersistWait &w, cudaStream_t st)
{
    auto kern = k_band<MODEL, GM, WPT>;
    int dev = 0, nsm = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return e;
    // largest block (warps) of which one fits per SM
    int warps = 0;
    for (int w = 32; w >= 4; w /= 2) {
        int per_sm = 0;
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, 32 * w, 0);
        if (e != cudaSuccess) return e;
        if (per_sm >= 1) { warps = w; break; }
    }
    if (warps == 0) return cudaErrorLaunchOutOfResources;
    int blocks = nsm < a.g.H ? nsm : a.g.H;
    if (blocks > max_blocks) blocks = max_blocks;
    StepArgs aa = a;
    uint64_t wait_ns = w.wait_ns;
    int withhold = w.withhold;
    void *args[] = {(void *)&aa,    (void *)&buf0,  (void *)&buf1, (void *)&seed,
                    (void *)&t0,    (void *)&nsteps, (void *)&flags, (void *)&err,
                    (void *)&wait_ns, (void *)&withhold};
    return cudaLaunchCooperativeKernel((void *)kern, dim3(blocks), dim3(32, warps), args, 0, st);
}

template <int MODEL, int GM>
static cudaError_t band_wpt(const StepArgs &a, uint64_t *b0, uint64_t *b1, uint64_t seed,
                            uint64_t t0, int n, int *flags, int *err, int maxb, const PersistWait &w,
                            cudaStream_t st)
{
    if (a.wpt == 2 && (a.g.nw % 2) == 0 && (a.g.W % 64) == 0)  // band form: whole pairs
        return band_launch<MODEL, GM, 2>(a, b0, b1, seed, t0, n, flags, err, maxb, w, st);
    return band_launch<MODEL, GM, 1>(a, b0, b1, seed, t0, n, flags, err, maxb, w, st);
}

template <int MODEL>
static cudaError_t band_model(int gm, const StepArgs &a, uint64_t *b0, uint64_t *b1,
                              uint64_t seed, uint64_t t0, int n, int *flags, int *err, int maxb,
                              const PersistWait &w, cudaStream_t st)
{
    switch (gm) {
    case GEOM_NONE: return band_wpt<MODEL, GEOM_NONE>(a, b0, b1, seed, t0, n, flags, err, maxb, w, st);
    case GEOM_NOSLIP: return band_wpt<MODEL, GEOM_NOSLIP>(a, b0, b1, seed, t0, n, flags, err, maxb, w, st);
    default: return band_wpt<MODEL, GEOM_FULL>(a, b0, b1, seed, t0, n, flags, err, maxb, w, st);
    }
}

cudaError_t launch_persistent(int model, int gm, const StepArgs &a, uint64_t *buf0, uint64_t *buf1,
                              uint64_t seed, uint64_t t0, int nsteps, int *flags, int *err,
                              int max_blocks, const PersistWait &w, cudaStream_t st)
{
    if (w.wait_ns == 0) return cudaErrorInvalidValue;
    switch (model) {
    case M_HPP: return band_model<M_HPP>(gm, a, buf0, buf1, seed, t0, nsteps, flags, err, max_blocks, w, st);
    case M_FHP_I: return band_model<M_FHP_I>(gm, a, buf0, buf1, seed, t0, nsteps, flags, err, max_blocks, w, st);
    default: return band_model<M_FHP_II>(gm, a, buf0, buf1, seed, t0, nsteps, flags, err, max_blocks, w, st);
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
