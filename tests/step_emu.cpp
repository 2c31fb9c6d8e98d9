// Host emulation of the CUDA one-step kernels for CPU parity checks of the
// kernel code itself.  lgca_gb300/csrc/step.cu (with the step bodies of
// step_body.cuh) is compiled here as plain C++ by g++; each warp is 32 host
// threads running in lockstep, and a warp shuffle is an exchange through a
// shared array between two barrier waits.  Paths: the step bodies under the
// one-step kernels' lane mapping (flat_site) -- the one-word body, the
// two-words-per-lane body, and that body with the batch kernel's seam
// shuffles (WRAP) -- and the kernels k_step2 and k_step themselves on their
// grids (blocks of 4 warps).  tests/test_step_emulated.py compares the
// result with the oracle.
//
//   step_emu IN OUT
//   IN:  int32 model, W, H, steps, force_x, path (0 one-word body, 1 pair
//        body, 2 pair body with WRAP, 3 kernel k_step2, 4 kernel k_step);
//        uint64 seed, t0, force_thr; H*W uint8 cells (bit d = channel d);
//        H*W uint8 cell types (0 fluid, 1 no-slip, 2 slip)
//   OUT: H*W uint8 cells after `steps` steps
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>

#include <barrier>
#include <thread>
#include <vector>

#include <cuda_runtime.h>

// ---- device intrinsics on the host
namespace emu {
struct Warp {
    uint32_t v[32];
    std::barrier<> bar{32};
};
thread_local int lane = 0;
thread_local Warp *warp = nullptr;

inline uint32_t exchange(uint32_t v, int src)
{
    warp->v[lane] = v;
    warp->bar.arrive_and_wait();
    const uint32_t r = warp->v[src];
    warp->bar.arrive_and_wait();
    return r;
}
}  // namespace emu

// source lanes outside [0, width) wrap within the lane's segment
inline uint32_t __shfl_sync(unsigned, uint32_t v, int src, int width = 32)
{
    const int base = emu::lane & ~(width - 1);
    return emu::exchange(v, base + (src & (width - 1)));
}
// a source before the segment start returns the lane's own value
inline uint32_t __shfl_up_sync(unsigned, uint32_t v, unsigned delta, int width = 32)
{
    const int base = emu::lane & ~(width - 1);
    const int s = emu::lane - (int)delta;
    return emu::exchange(v, s < base ? emu::lane : s);
}
inline uint32_t __shfl_down_sync(unsigned, uint32_t v, unsigned delta, int width = 32)
{
    const int base = emu::lane & ~(width - 1);
    const int s = emu::lane + (int)delta;
    return emu::exchange(v, s >= base + width ? emu::lane : s);
}
// warp vote: every lane offers its predicate, each gets the OR of all
inline int __any_sync(unsigned, int pred)
{
    emu::warp->v[emu::lane] = pred != 0;
    emu::warp->bar.arrive_and_wait();
    int any = 0;
    for (int i = 0; i < 32; ++i) any |= (int)emu::warp->v[i];
    emu::warp->bar.arrive_and_wait();
    return any;
}
template <class T> inline T __ldcg(const T *p) { return *p; }
template <class T> inline T __ldg(const T *p) { return *p; }
// grid coordinates of the emulated thread
thread_local uint3 threadIdx;
thread_local uint3 blockIdx;
thread_local dim3 blockDim;
thread_local dim3 gridDim;
// used only by the persistent band kernel of step.cu, which is compiled here
// but not run
inline void __syncthreads() { std::abort(); }
inline void __nanosleep(unsigned) { std::abort(); }
inline void __threadfence() { std::abort(); }
inline int atomicExch(int *, int) { std::abort(); }
// kernel qualifiers with no host meaning
#ifndef __launch_bounds__
#define __launch_bounds__(...)
#endif
#ifndef __grid_constant__
#define __grid_constant__
#endif

#include "../lgca_gb300/csrc/step.cu"

using namespace lgca_gpu;

// ---- one emulated launch per step
template <int MODEL, int GM, int PATH, bool ODD>
static void run_steps(StepArgs a, uint64_t *buf0, uint64_t *buf1, uint64_t seed, uint64_t t0,
                      int steps)
{
    const int items = PATH == 0 ? a.g.nw : (a.g.nw + 1) / 2;
    const long long tasks = flat_tasks(a.g.H, items);
    const uint32_t magic = flat_magic(a.g.H, items);
    emu::Warp w;
    std::vector<std::thread> th;
    for (int ln = 0; ln < 32; ++ln)
        th.emplace_back([&, ln] {
            emu::lane = ln;
            emu::warp = &w;
            for (int s = 0; s < steps; ++s) {
                const uint64_t t = t0 + (uint64_t)s;
                StepIO io{(s & 1) ? buf1 : buf0, (s & 1) ? buf0 : buf1,
                          lgca_rng_key(seed, LGCA_STREAM_CHIR, t),
                          lgca_rng_key(seed, LGCA_STREAM_FORCE, t)};
                for (long long k = 0; k < tasks; ++k) {
                    int y, it;
                    flat_site(k, ln, a.g.H, items, magic, y, it);
                    if (PATH == 0) step_word<MODEL, GM>(a, io, y, it, ln);
                    else if (PATH == 1) step_pair<MODEL, GM, false, false, ODD, false>(a, io, y, it, ln);
                    else step_pair<MODEL, GM, false, false, ODD, true>(a, io, y, it, ln);
                }
                w.bar.arrive_and_wait();  // the step is written before the next reads it
            }
        });
    for (auto &x : th) x.join();
}

// the kernels k_step2 (PATH 3) and k_step (PATH 4) on grids of 4-warp blocks
template <int MODEL, int GM, int PATH, bool ODD>
static void run_kernel(StepArgs a, uint64_t *buf0, uint64_t *buf1, uint64_t seed, uint64_t t0,
                       int steps)
{
    constexpr int WARPS = 4;
    const int items = PATH == 4 ? a.g.nw : (a.g.nw + 1) / 2;
    const long long tasks = flat_tasks(a.g.H, items);
    const long long blocks = (tasks + WARPS - 1) / WARPS;
    a.fmagic = flat_magic(a.g.H, items);
    std::vector<emu::Warp> warps(WARPS);
    std::barrier<> done(32 * WARPS);
    std::vector<std::thread> th;
    for (int i = 0; i < 32 * WARPS; ++i)
        th.emplace_back([&, i] {
            threadIdx = make_uint3((unsigned)(i & 31), (unsigned)(i >> 5), 0);
            blockDim = dim3(32, WARPS, 1);
            emu::lane = i & 31;
            emu::warp = &warps[i >> 5];
            for (int s = 0; s < steps; ++s) {
                StepArgs as = a;
                const uint64_t t = t0 + (uint64_t)s;
                as.src = (s & 1) ? buf1 : buf0;
                as.dst = (s & 1) ? buf0 : buf1;
                as.chir_key = lgca_rng_key(seed, LGCA_STREAM_CHIR, t);
                as.force_key = lgca_rng_key(seed, LGCA_STREAM_FORCE, t);
                for (long long b = 0; b < blocks; ++b) {
                    blockIdx = make_uint3((unsigned)b, 0, 0);
                    if (PATH == 3) k_step2<MODEL, GM, ODD>(as);
                    else k_step<MODEL, GM>(as);
                    done.arrive_and_wait();  // blocks in turn, steps in order
                }
            }
        });
    for (auto &x : th) x.join();
}

template <int MODEL, int GM>
static bool dispatch_path(int path, bool odd, StepArgs a, uint64_t *b0, uint64_t *b1,
                          uint64_t seed, uint64_t t0, int steps)
{
    if (path == 3 && odd) run_kernel<MODEL, GM, 3, true>(a, b0, b1, seed, t0, steps);
    else if (path == 3) run_kernel<MODEL, GM, 3, false>(a, b0, b1, seed, t0, steps);
    else if (path == 4) run_kernel<MODEL, GM, 4, false>(a, b0, b1, seed, t0, steps);
    else if (path == 0) run_steps<MODEL, GM, 0, false>(a, b0, b1, seed, t0, steps);
    else if (path == 1 && odd) run_steps<MODEL, GM, 1, true>(a, b0, b1, seed, t0, steps);
    else if (path == 1) run_steps<MODEL, GM, 1, false>(a, b0, b1, seed, t0, steps);
    else if (odd) run_steps<MODEL, GM, 2, true>(a, b0, b1, seed, t0, steps);
    else run_steps<MODEL, GM, 2, false>(a, b0, b1, seed, t0, steps);
    return true;
}

template <int MODEL>
static bool dispatch_geom(int gm, int path, bool odd, StepArgs a, uint64_t *b0, uint64_t *b1,
                          uint64_t seed, uint64_t t0, int steps)
{
    if (gm == GEOM_NONE) return dispatch_path<MODEL, GEOM_NONE>(path, odd, a, b0, b1, seed, t0, steps);
    if (gm == GEOM_NOSLIP)
        return dispatch_path<MODEL, GEOM_NOSLIP>(path, odd, a, b0, b1, seed, t0, steps);
    return dispatch_path<MODEL, GEOM_FULL>(path, odd, a, b0, b1, seed, t0, steps);
}

int main(int argc, char **argv)
{
    if (argc != 3) {
        std::fprintf(stderr, "usage: step_emu IN OUT\n");
        return 2;
    }
    FILE *f = std::fopen(argv[1], "rb");
    if (!f) return 2;
    int32_t hdr[6];
    uint64_t u[3];
    if (std::fread(hdr, sizeof(hdr), 1, f) != 1 || std::fread(u, sizeof(u), 1, f) != 1) return 2;
    const int model = hdr[0], W = hdr[1], H = hdr[2], steps = hdr[3], fx = hdr[4], path = hdr[5];
    const uint64_t seed = u[0], t0 = u[1], thr = u[2];
    std::vector<uint8_t> cells((size_t)W * H), types((size_t)W * H);
    if (std::fread(cells.data(), 1, cells.size(), f) != cells.size() ||
        std::fread(types.data(), 1, types.size(), f) != types.size())
        return 2;
    std::fclose(f);
    if ((path == 1 || path == 2 || path == 3) && W % 64 != 0) return 3;

    const int D = num_dir(model);
    PlaneGeom g{};
    g.W = W;
    g.H = H;
    g.nw = (W + 63) / 64;
    g.pitch = (g.nw + 1) & ~1;
    g.ps = (size_t)H * g.pitch;
    g.L = (W - 1) & 63;
    g.lastmask = (g.L == 63) ? ~0ull : ((1ull << (g.L + 1)) - 1ull);
    std::vector<uint64_t> b0(D * g.ps, 0), b1(D * g.ps, 0), solid(g.ps, 0), slip(g.ps, 0);
    bool any_solid = false, any_slip = false;
    for (int y = 0; y < H; ++y)
        for (int x = 0; x < W; ++x) {
            const size_t o = (size_t)y * g.pitch + (x >> 6);
            const uint64_t bit = 1ull << (x & 63);
            const uint8_t c = cells[(size_t)y * W + x];
            for (int d = 0; d < D; ++d)
                if ((c >> d) & 1) b0[d * g.ps + o] |= bit;
            const uint8_t ty = types[(size_t)y * W + x];
            if (ty == 1) solid[o] |= bit, any_solid = true;
            if (ty == 2) slip[o] |= bit, any_slip = true;
        }
    const int gm = any_slip ? GEOM_FULL : (any_solid ? GEOM_NOSLIP : GEOM_NONE);
    StepArgs a{};
    a.solid = solid.data();
    a.slip = slip.data();
    a.chir = nullptr;
    a.g = g;
    a.chunks = (g.nw + 31) / 32;
    a.force_thr = fx >= 0 ? thr : 0;
    a.fx = fx;
    a.wpt = (path == 0 || path == 4) ? 1 : 2;
    const bool odd = (g.nw & 1) != 0;
    if (model == 0) dispatch_geom<M_HPP>(gm, path, odd, a, b0.data(), b1.data(), seed, t0, steps);
    else if (model == 1) dispatch_geom<M_FHP_I>(gm, path, odd, a, b0.data(), b1.data(), seed, t0, steps);
    else dispatch_geom<M_FHP_II>(gm, path, odd, a, b0.data(), b1.data(), seed, t0, steps);
    const std::vector<uint64_t> &res = (steps & 1) ? b1 : b0;

    for (int y = 0; y < H; ++y)
        for (int x = 0; x < W; ++x) {
            const size_t o = (size_t)y * g.pitch + (x >> 6);
            uint8_t c = 0;
            for (int d = 0; d < D; ++d) c |= (uint8_t)(((res[d * g.ps + o] >> (x & 63)) & 1) << d);
            cells[(size_t)y * W + x] = c;
        }
    // the padding word of odd word counts and the tail bits must stay zero
    for (int d = 0; d < D; ++d)
        for (int y = 0; y < H; ++y) {
            const size_t row = d * g.ps + (size_t)y * g.pitch;
            if ((res[row + g.nw - 1] & ~g.lastmask) != 0) return 4;
            if (g.pitch > g.nw && res[row + g.nw] != 0) return 5;
        }
    f = std::fopen(argv[2], "wb");
    if (!f) return 2;
    std::fwrite(cells.data(), 1, cells.size(), f);
    std::fclose(f);
    return 0;
}
