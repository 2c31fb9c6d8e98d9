// Host emulation of the resident step kernel (lgca_gb300/csrc/resident.cu)
// for CPU parity checks of the kernel code itself.  The kernel source is
// compiled here as plain C++ by g++; every thread of every block is a host
// thread and all blocks run at once, as a cooperative launch guarantees:
// a warp shuffle is an exchange through a shared array between two barrier
// waits of the warp's 32 threads, __syncthreads a barrier of the block's
// threads, the block's shared memory a host array, and the 64-bit halo
// items relaxed atomics.  Waits are bounded by the host clock.  tests/test_step_emulated.py compares the
// result with the oracle.
//
//   resident_emu IN OUT
//   IN:  int32 model, W, H, steps, force_x, nblk, chunk, withhold, aos, B, rowsync;
//        uint64 seed, t0, force_thr, wait_ns; H*W uint8 cells (bit d = channel d);
//        H*W uint8 cell types (0 fluid, 1 no-slip, 2 slip)
//   OUT: int32 err; H*W uint8 cells after `steps` steps, run as launches of
//        `chunk` steps each (converted from the planes); then, with aos & 2,
//        the H*W bytes the last launch wrote in the byte-per-cell layout.
//   aos & 1: the first launch reads its input in the byte-per-cell layout;
//   aos & 2: every launch also writes its result in that layout.
//   B > 0: the last launch also adds up the B x B block sums of its result,
//   written last as int32 N, Jx2, Jy (each ceil(H/B) x ceil(W/B)).
//   rowsync 1: the kernel's row-barrier form; 0: its block-barrier form.
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>

#include <atomic>
#include <barrier>
#include <chrono>
#include <memory>
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
thread_local std::barrier<> *block_bar = nullptr;
thread_local uint64_t *smem = nullptr;

inline uint32_t exchange(uint32_t v, int src)
{
    warp->v[lane] = v;
    warp->bar.arrive_and_wait();
    const uint32_t r = warp->v[src];
    warp->bar.arrive_and_wait();
    return r;
}
}  // namespace emu

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
inline int __any_sync(unsigned, int pred)
{
    emu::warp->v[emu::lane] = pred != 0;
    emu::warp->bar.arrive_and_wait();
    int any = 0;
    for (int i = 0; i < 32; ++i) any |= (int)emu::warp->v[i];
    emu::warp->bar.arrive_and_wait();
    return any;
}
inline int __all_sync(unsigned, int pred)
{
    emu::warp->v[emu::lane] = pred != 0;
    emu::warp->bar.arrive_and_wait();
    int all = 1;
    for (int i = 0; i < 32; ++i) all &= (int)emu::warp->v[i];
    emu::warp->bar.arrive_and_wait();
    return all;
}
inline void __syncwarp(unsigned = 0xffffffffu) { emu::warp->bar.arrive_and_wait(); }
inline void __syncthreads() { emu::block_bar->arrive_and_wait(); }
inline void __threadfence() { std::atomic_thread_fence(std::memory_order_seq_cst); }
inline void __nanosleep(unsigned) { std::this_thread::yield(); }
inline int atomicExch(int *p, int v) { return __atomic_exchange_n(p, v, __ATOMIC_SEQ_CST); }
inline int atomicAdd(int *p, int v) { return __atomic_fetch_add(p, v, __ATOMIC_RELAXED); }
inline int __popcll(unsigned long long x) { return __builtin_popcountll(x); }
template <class T> inline T __ldcg(const T *p) { return *p; }
template <class T> inline T __ldg(const T *p) { return *p; }
thread_local uint3 threadIdx;
thread_local uint3 blockIdx;
thread_local dim3 blockDim;
thread_local dim3 gridDim;
#ifndef __launch_bounds__
#define __launch_bounds__(...)
#endif
#ifndef __grid_constant__
#define __grid_constant__
#endif

#define LGCA_HOST_EMULATION 1
namespace lgca_gpu {
inline uint64_t *res_smem() { return emu::smem; }
inline ulonglong2 ld_items(const uint64_t *p)
{
    ulonglong2 v;
    v.x = __atomic_load_n(p, __ATOMIC_RELAXED);
    v.y = __atomic_load_n(p + 1, __ATOMIC_RELAXED);
    return v;
}
inline void st_items(uint64_t *p, uint64_t a, uint64_t b)
{
    __atomic_store_n(p, a, __ATOMIC_RELAXED);
    __atomic_store_n(p + 1, b, __ATOMIC_RELAXED);
}
// an mbarrier as one word: completed phases << 48 | arrivals per phase << 24
// | arrivals still missing in the current phase
inline void res_bar_init(uint64_t *bar, unsigned count)
{
    __atomic_store_n(bar, ((uint64_t)count << 24) | count, __ATOMIC_RELEASE);
}
inline void res_bar_arrive(uint64_t *bar)
{
    uint64_t w = __atomic_load_n(bar, __ATOMIC_RELAXED), nw;
    do {
        const uint64_t pend = w & 0xffffff, cnt = (w >> 24) & 0xffffff, ph = w >> 48;
        nw = pend == 1 ? ((ph + 1) << 48) | (cnt << 24) | cnt : w - 1;
    } while (!__atomic_compare_exchange_n(bar, &w, nw, true, __ATOMIC_ACQ_REL, __ATOMIC_RELAXED));
}
inline bool res_bar_done(const uint64_t *bar, unsigned parity)
{
    return ((__atomic_load_n(bar, __ATOMIC_ACQUIRE) >> 48) & 1) != parity;
}
inline uint64_t res_timer_ns()
{
    return (uint64_t)std::chrono::duration_cast<std::chrono::nanoseconds>(
               std::chrono::steady_clock::now().time_since_epoch())
        .count();
}
}  // namespace lgca_gpu
#include "../lgca_gb300/csrc/resident.cu"

using namespace lgca_gpu;

// one cooperative launch of the kernel: every block's threads at once
template <int MODEL, int GM, bool RS>
static void launch(const StepArgs &a, const ResidentArgs &R)
{
    constexpr int SP = ResPlanes<MODEL>::SP;
    const int warps = R.rpb * R.wpr;
    const size_t smem_words = res_smem_words(SP, a.g.nw, R.rpb, R.wpr);
    std::vector<std::vector<uint64_t>> sm(R.nblk, std::vector<uint64_t>(smem_words, 0));
    std::vector<std::unique_ptr<emu::Warp[]>> wp;
    std::vector<std::unique_ptr<std::barrier<>>> bb;
    for (int b = 0; b < R.nblk; ++b) {
        wp.emplace_back(new emu::Warp[warps]);
        bb.emplace_back(new std::barrier<>(32 * warps));
    }
    std::vector<std::thread> th;
    for (int b = 0; b < R.nblk; ++b)
        for (int i = 0; i < 32 * warps; ++i)
            th.emplace_back([&, b, i] {
                threadIdx = make_uint3((unsigned)(i & 31), (unsigned)(i >> 5), 0);
                blockIdx = make_uint3((unsigned)b, 0, 0);
                blockDim = dim3(32, warps, 1);
                gridDim = dim3(R.nblk, 1, 1);
                emu::lane = i & 31;
                emu::warp = &wp[b][i >> 5];
                emu::block_bar = bb[b].get();
                emu::smem = sm[b].data();
                k_resident<MODEL, GM, RS>(a, R);
                // a block's threads that returned early leave the barrier
                // alone: the kernel returns block-uniformly
            });
    for (auto &x : th) x.join();
}

template <int MODEL, bool RS>
static void launch_gm(int gm, const StepArgs &a, const ResidentArgs &R)
{
    if (gm == GEOM_NONE) launch<MODEL, GEOM_NONE, RS>(a, R);
    else if (gm == GEOM_NOSLIP) launch<MODEL, GEOM_NOSLIP, RS>(a, R);
    else launch<MODEL, GEOM_FULL, RS>(a, R);
}
template <int MODEL>
static void launch_sync(bool rs, int gm, const StepArgs &a, const ResidentArgs &R)
{
    if (rs) launch_gm<MODEL, true>(gm, a, R);
    else launch_gm<MODEL, false>(gm, a, R);
}

int main(int argc, char **argv)
{
    if (argc != 3) {
        std::fprintf(stderr, "usage: resident_emu IN OUT\n");
        return 2;
    }
    FILE *f = std::fopen(argv[1], "rb");
    if (!f) return 2;
    int32_t hdr[11];
    uint64_t u[4];
    if (std::fread(hdr, sizeof(hdr), 1, f) != 1 || std::fread(u, sizeof(u), 1, f) != 1) return 2;
    const int model = hdr[0], W = hdr[1], H = hdr[2], steps = hdr[3], fx = hdr[4], nblk = hdr[5],
              chunk = hdr[6], withhold = hdr[7], aos = hdr[8], sumsB = hdr[9], rowsync = hdr[10];
    const uint64_t seed = u[0], t0 = u[1], thr = u[2], wait_ns = u[3];
    std::vector<uint8_t> cells((size_t)W * H), types((size_t)W * H);
    if (std::fread(cells.data(), 1, cells.size(), f) != cells.size() ||
        std::fread(types.data(), 1, types.size(), f) != types.size())
        return 2;
    std::fclose(f);

    const int D = num_dir(model);
    PlaneGeom g{};
    g.W = W;
    g.H = H;
    g.nw = (W + 63) / 64;
    g.pitch = (g.nw + 1) & ~1;
    g.ps = (size_t)H * g.pitch;
    g.L = (W - 1) & 63;
    g.lastmask = (g.L == 63) ? ~0ull : ((1ull << (g.L + 1)) - 1ull);
    if (W % 64 != 0 || (g.nw & 1) || nblk < 1 || nblk > H || chunk < 1) return 3;
    const int np = g.nw / 2, wpr = (np + 31) / 32, rpb = (H + nblk - 1) / nblk;
    if (rpb * wpr > RES_MAX_WARPS) return 3;

    std::vector<uint64_t> buf[2] = {std::vector<uint64_t>(D * g.ps, 0), std::vector<uint64_t>(D * g.ps, 0)};
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
    std::vector<uint64_t> halo((size_t)RES_HALO_SLOTS * nblk * 2 * 2 * g.nw * 2, 0);
    int err = 0;

    StepArgs a{};
    a.solid = solid.data();
    a.slip = slip.data();
    a.chir = nullptr;
    a.g = g;
    a.chunks = (g.nw + 31) / 32;
    a.force_thr = fx >= 0 ? thr : 0;
    a.fx = fx;
    a.wpt = 2;
    std::vector<uint8_t> aos_in(cells), aos_out((size_t)W * H, 0xff);
    const int Wb = sumsB > 0 ? (W + sumsB - 1) / sumsB : 0, Hb = sumsB > 0 ? (H + sumsB - 1) / sumsB : 0;
    std::vector<int32_t> sums((size_t)3 * Wb * Hb, 0);
    int cur = 0;
    for (int done = 0; done < steps; done += chunk) {
        const int n = std::min(chunk, steps - done);
        a.src = buf[cur].data();
        a.dst = buf[cur ^ 1].data();
        ResidentArgs R{};
        R.halo = halo.data();
        R.epoch = 1 + (unsigned)(done / chunk) % 255;  // a new epoch per launch (slots zeroed once)
        R.err = &err;
        R.seed = seed;
        R.t0 = t0 + (uint64_t)done;
        R.nsteps = n;
        R.nblk = nblk;
        R.wpr = wpr;
        R.rpb = rpb;
        R.wait_ns = wait_ns;
        R.withhold = withhold;
        R.aos_in = (done == 0 && (aos & 1)) ? aos_in.data() : nullptr;
        R.aos_out = (aos & 2) ? aos_out.data() : nullptr;
        const bool last = done + n >= steps;
        R.sums_B = last ? sumsB : 0;
        R.sums_Wb = Wb;
        R.sums_N = sums.data();
        R.sums_Jx2 = sums.data() + (size_t)Wb * Hb;
        R.sums_Jy = sums.data() + (size_t)2 * Wb * Hb;
        if (model == 0) launch_sync<M_HPP>(rowsync != 0, gm, a, R);
        else if (model == 1) launch_sync<M_FHP_I>(rowsync != 0, gm, a, R);
        else launch_sync<M_FHP_II>(rowsync != 0, gm, a, R);
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
    FILE *o = std::fopen(argv[2], "wb");
    if (!o) return 2;
    const int32_t e32 = err;
    std::fwrite(&e32, sizeof(e32), 1, o);
    std::fwrite(cells.data(), 1, cells.size(), o);
    if (aos & 2) std::fwrite(aos_out.data(), 1, aos_out.size(), o);
    if (sumsB > 0) std::fwrite(sums.data(), sizeof(int32_t), sums.size(), o);
    std::fclose(o);
    return 0;
}
