// Host emulation of the temporally blocked kernels (lgca_gb300/csrc/wave.cu
// k_wave, multistep.cu k_multistep) for CPU parity checks of the kernel
// code itself.  The kernel bodies are compiled here as plain C++ by g++;
// blocks run one after another, every thread of a block is a host thread, a
// warp shuffle is an exchange among the warp's 32 threads between two
// barrier waits, __syncthreads is a barrier of the block, and the block's
// shared memory is one host array.  Grids and tile shapes are the ones the
// launchers in those files use.  tests/test_step_emulated.py compares the
// result with the oracle.
//
//   multistep_emu IN OUT
//   IN:  int32 model, W, H, steps, force_x, kernel (0 wavefront, 1 tiles),
//        depth; uint64 seed, t0, force_thr; H*W uint8 cells; H*W uint8
//        cell types (0 fluid, 1 no-slip, 2 slip)
//   OUT: H*W uint8 cells after `steps` steps (`steps` a multiple of depth)
#include <cstdint>
#include <cstdio>
#include <cstring>

#include <barrier>
#include <memory>
#include <thread>
#include <vector>

#include <cuda_runtime.h>

// ---- the CUDA thread model on the host
namespace emu {
struct Warp {
    uint32_t v[32];
    std::barrier<> bar{32};
};
struct Block {
    explicit Block(int n) : bar(n), warps((n + 31) / 32) {}
    std::barrier<> bar;
    std::vector<Warp> warps;
};
thread_local int lane = 0;
thread_local Warp *warp = nullptr;
thread_local Block *block = nullptr;

inline uint32_t exchange(uint32_t v, int src)
{
    warp->v[lane] = v;
    warp->bar.arrive_and_wait();
    const uint32_t r = warp->v[src];
    warp->bar.arrive_and_wait();
    return r;
}
}  // namespace emu

thread_local uint3 threadIdx;
thread_local uint3 blockIdx;
thread_local dim3 blockDim;

inline uint32_t __shfl_sync(unsigned, uint32_t v, int src, int width = 32)
{
    const int base = emu::lane & ~(width - 1);
    return emu::exchange(v, base + (src & (width - 1)));
}
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
inline void __syncthreads() { emu::block->bar.arrive_and_wait(); }
inline int __ffsll(long long x) { return __builtin_ffsll(x); }
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
// the launchers in the included files are compiled but never called here
template <class F> inline cudaError_t cudaFuncSetAttribute(F *f, cudaFuncAttribute attr, int value)
{
    return cudaFuncSetAttribute(reinterpret_cast<const void *>(f), attr, value);
}
// kernel qualifiers with no host meaning
#ifndef __launch_bounds__
#define __launch_bounds__(...)
#endif
#ifndef __grid_constant__
#define __grid_constant__
#endif

#include "../lgca_gb300/csrc/multistep.cu"
#include "../lgca_gb300/csrc/wave.cu"

namespace lgca_gpu {
// the block's dynamic shared memory (blocks run one at a time)
uint64_t smem[1 << 15];
}  // namespace lgca_gpu

using namespace lgca_gpu;

template <class F> static void run_grid(dim3 grid, int nthreads, F body)
{
    for (unsigned by = 0; by < grid.y; ++by)
        for (unsigned bx = 0; bx < grid.x; ++bx) {
            emu::Block blk(nthreads);
            std::vector<std::thread> th;
            for (int i = 0; i < nthreads; ++i)
                th.emplace_back([&, i] {
                    threadIdx = make_uint3((unsigned)i, 0, 0);
                    blockIdx = make_uint3(bx, by, 0);
                    blockDim = dim3((unsigned)nthreads, 1, 1);
                    emu::lane = i & 31;
                    emu::warp = &blk.warps[i >> 5];
                    emu::block = &blk;
                    body();
                });
            for (auto &x : th) x.join();
        }
}

// one pass of K steps, grid and shapes as in launch_k (wave.cu)
template <int MODEL, int GM, int K> static void wave_pass(const MultiStepArgs &m)
{
    const PlaneGeom &g = m.base.g;
    const int nstrips = (g.nw + 29) / 30;
    int S = 64;
    while (S > 8 && (long long)nstrips * ((g.H + S - 1) / S) < 4 * 152 * 8) S >>= 1;
    const long long warps = (long long)nstrips * ((g.H + S - 1) / S);
    const unsigned blocks = (unsigned)((warps + 3) / 4);
    run_grid(dim3(blocks), 128, [&] { k_wave<MODEL, GM, K>(m, S, nstrips); });
}

// one pass of K steps, grid and shapes as in launch_tile (multistep.cu)
template <int MODEL, int GM, int K> static void tile_pass(const MultiStepArgs &m)
{
    constexpr int THO = 16;
    static_assert(Tile<MODEL, GM, K, THO>::SMEM <= sizeof(smem), "shared memory of the tile");
    const dim3 grid((unsigned)((m.base.g.nw + 31) / 32), (unsigned)((m.base.g.H + THO - 1) / THO));
    run_grid(grid, 256, [&] { k_multistep<MODEL, GM, K, THO>(m); });
}

template <int MODEL, int GM, int K> static void pass(int kernel, const MultiStepArgs &m)
{
    if (kernel == 0) wave_pass<MODEL, GM, K>(m);
    else tile_pass<MODEL, GM, K>(m);
}

template <int MODEL, int GM> static bool pass_depth(int kernel, int depth, const MultiStepArgs &m)
{
    switch (depth) {
    case 2: pass<MODEL, GM, 2>(kernel, m); return true;
    case 4: pass<MODEL, GM, 4>(kernel, m); return true;
    case 8:
        if (kernel == 1 || MODEL == M_HPP) {
            pass<MODEL, GM, 8>(kernel, m);
            return true;
        }
        return false;
    default: return false;
    }
}

template <int MODEL> static bool pass_geom(int gm, int kernel, int depth, const MultiStepArgs &m)
{
    if (gm == GEOM_NONE) return pass_depth<MODEL, GEOM_NONE>(kernel, depth, m);
    if (gm == GEOM_NOSLIP) return pass_depth<MODEL, GEOM_NOSLIP>(kernel, depth, m);
    return pass_depth<MODEL, GEOM_FULL>(kernel, depth, m);
}

int main(int argc, char **argv)
{
    if (argc != 3) {
        std::fprintf(stderr, "usage: multistep_emu IN OUT\n");
        return 2;
    }
    FILE *f = std::fopen(argv[1], "rb");
    if (!f) return 2;
    int32_t hdr[7];
    uint64_t u[3];
    if (std::fread(hdr, sizeof(hdr), 1, f) != 1 || std::fread(u, sizeof(u), 1, f) != 1) return 2;
    const int model = hdr[0], W = hdr[1], H = hdr[2], steps = hdr[3], fx = hdr[4];
    const int kernel = hdr[5], depth = hdr[6];
    const uint64_t seed = u[0], t0 = u[1], thr = u[2];
    std::vector<uint8_t> cells((size_t)W * H), types((size_t)W * H);
    if (std::fread(cells.data(), 1, cells.size(), f) != cells.size() ||
        std::fread(types.data(), 1, types.size(), f) != types.size())
        return 2;
    std::fclose(f);
    if (W % 64 != 0 || depth < 2 || steps % depth != 0) return 3;

    const int D = num_dir(model);
    PlaneGeom g{};
    g.W = W;
    g.H = H;
    g.nw = (W + 63) / 64;
    g.pitch = (g.nw + 1) & ~1;
    g.ps = (size_t)H * g.pitch;
    g.L = (W - 1) & 63;
    g.lastmask = (g.L == 63) ? ~0ull : ((1ull << (g.L + 1)) - 1ull);
    std::vector<uint64_t> buf[2] = {std::vector<uint64_t>(D * g.ps, 0),
                                    std::vector<uint64_t>(D * g.ps, 0)};
    std::vector<uint64_t> solid(g.ps, 0), slip(g.ps, 0);
    bool any_solid = false, any_slip = false;
    for (int y = 0; y < H; ++y)
        for (int x = 0; x < W; ++x) {
            const size_t o = (size_t)y * g.pitch + (x >> 6);
            const uint64_t bit = 1ull << (x & 63);
            const uint8_t c = cells[(size_t)y * W + x];
            for (int d = 0; d < D; ++d)
                if ((c >> d) & 1) buf[0][d * g.ps + o] |= bit;
            const uint8_t ty = types[(size_t)y * W + x];
            if (ty == 1) solid[o] |= bit, any_solid = true;
            if (ty == 2) slip[o] |= bit, any_slip = true;
        }
    const int gm = any_slip ? GEOM_FULL : (any_solid ? GEOM_NOSLIP : GEOM_NONE);
    int cur = 0;
    for (int done = 0; done < steps; done += depth) {
        MultiStepArgs m{};
        m.base.src = buf[cur].data();
        m.base.dst = buf[cur ^ 1].data();
        m.base.solid = solid.data();
        m.base.slip = slip.data();
        m.base.chir = nullptr;
        m.base.g = g;
        m.base.chunks = (g.nw + 31) / 32;
        m.base.force_thr = fx >= 0 ? thr : 0;
        m.base.fx = fx;
        m.depth = depth;
        for (int i = 0; i < depth; ++i) {
            const uint64_t t = t0 + (uint64_t)(done + i);
            m.chir_keys[i] = lgca_rng_key(seed, LGCA_STREAM_CHIR, t);
            m.force_keys[i] = lgca_rng_key(seed, LGCA_STREAM_FORCE, t);
        }
        bool ok;
        if (model == 0) ok = pass_geom<M_HPP>(gm, kernel, depth, m);
        else if (model == 1) ok = pass_geom<M_FHP_I>(gm, kernel, depth, m);
        else ok = pass_geom<M_FHP_II>(gm, kernel, depth, m);
        if (!ok) return 3;
        cur ^= 1;
    }
    const std::vector<uint64_t> &res = buf[cur];
    for (int y = 0; y < H; ++y)
        for (int x = 0; x < W; ++x) {
            const size_t o = (size_t)y * g.pitch + (x >> 6);
            uint8_t c = 0;
            for (int d = 0; d < D; ++d) c |= (uint8_t)(((res[d * g.ps + o] >> (x & 63)) & 1) << d);
            cells[(size_t)y * W + x] = c;
        }
    f = std::fopen(argv[2], "wb");
    if (!f) return 2;
    std::fwrite(cells.data(), 1, cells.size(), f);
    std::fclose(f);
    return 0;
}
