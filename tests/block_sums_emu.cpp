// Host emulation of the integer block-sum kernels
// (lgca_gb300/csrc/block_sums.cuh) for CPU parity checks of the kernel code:
// compiled here as plain C++ by g++ and run on the grids of
// block_sums_model (aux.cu), one block of 128 host threads at a time, warp
// shuffles exchanging among a warp's 32 threads between barrier waits.
// tests/test_step_emulated.py compares the sums with the oracle's.
//
//   block_sums_emu IN OUT
//   IN:  int32 model, W, H, B; H*W uint8 cells (bit d = channel d)
//   OUT: int32 N, Jx2, Jy, each Hb*Wb (Hb = ceil(H/B), Wb = ceil(W/B))
#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <functional>

#include <barrier>
#include <thread>
#include <vector>

#include <cuda_runtime.h>

namespace emu {
struct Warp {
    uint32_t v[32];
    std::barrier<> bar{32};
};
thread_local int lane = 0;
thread_local Warp *warp = nullptr;
}  // namespace emu

thread_local uint3 threadIdx;
thread_local uint3 blockIdx;
thread_local dim3 blockDim;

inline int __shfl_xor_sync(unsigned, int v, int mask, int width = 32)
{
    emu::warp->v[emu::lane] = (uint32_t)v;
    emu::warp->bar.arrive_and_wait();
    const int src = (emu::lane & ~(width - 1)) | ((emu::lane ^ mask) & (width - 1));
    const int r = (int)emu::warp->v[src];
    emu::warp->bar.arrive_and_wait();
    return r;
}
inline int __popcll(unsigned long long x) { return __builtin_popcountll(x); }
template <class T> inline T __ldg(const T *p) { return *p; }
inline int min(int a, int b) { return a < b ? a : b; }
inline int max(int a, int b) { return a > b ? a : b; }

#include "../lgca_gb300/csrc/block_sums.cuh"

using namespace lgca_gpu;

// a grid of `blocks` blocks of 128 threads, one block at a time
static void run_grid(unsigned blocks, const std::function<void()> &body)
{
    if (blocks == 0) return;
    std::vector<emu::Warp> warps(4);
    std::barrier<> done(128);
    std::vector<std::thread> th;
    for (int i = 0; i < 128; ++i)
        th.emplace_back([&, i] {
            threadIdx = make_uint3((unsigned)i, 0, 0);
            blockDim = dim3(128, 1, 1);
            emu::lane = i & 31;
            emu::warp = &warps[i >> 5];
            for (unsigned b = 0; b < blocks; ++b) {
                blockIdx = make_uint3(b, 0, 0);
                body();
                done.arrive_and_wait();
            }
        });
    for (auto &x : th) x.join();
}

static unsigned grid_of(long long n, int threads) { return (unsigned)((n + threads - 1) / threads); }

// block_sums_model (aux.cu): the kernel and grid for B
template <int MODEL>
static void block_sums(const PlaneGeom &g, const uint64_t *planes, int B, int32_t *N,
                       int32_t *Jx2, int32_t *Jy)
{
    const int Wb = (g.W + B - 1) / B, Hb = (g.H + B - 1) / B;
    auto seg_grid = [&](long long warps) { return grid_of(warps * 32, 128); };
    switch (B) {
    case 8:
        run_grid(seg_grid(seg_block_sums_warps<8>(g.nw, Hb)),
                 [&] { k_block_sums_seg<MODEL, 8>(g, planes, Wb, Hb, N, Jx2, Jy); });
        break;
    case 16:
        run_grid(seg_grid(seg_block_sums_warps<16>(g.nw, Hb)),
                 [&] { k_block_sums_seg<MODEL, 16>(g, planes, Wb, Hb, N, Jx2, Jy); });
        break;
    case 32:
        run_grid(seg_grid(seg_block_sums_warps<32>(g.nw, Hb)),
                 [&] { k_block_sums_seg<MODEL, 32>(g, planes, Wb, Hb, N, Jx2, Jy); });
        break;
    case 64:
        run_grid(seg_grid(seg_block_sums_warps<64>(g.nw, Hb)),
                 [&] { k_block_sums_seg<MODEL, 64>(g, planes, Wb, Hb, N, Jx2, Jy); });
        break;
    default:
        if (B % 64 == 0 && B <= 2048 && ((B / 64) & (B / 64 - 1)) == 0) {
            const int K = B / 64, chunks = (g.nw + 31) / 32;
            const long long tasks = (long long)Hb * chunks;
            run_grid(grid_of(tasks, 4), [&] {
                k_block_sums_wide<MODEL>(g, planes, K, B, Wb, Hb, chunks, N, Jx2, Jy);
            });
        } else {
            run_grid(grid_of((long long)Wb * Hb, 128),
                     [&] { k_block_sums_any<MODEL>(g, planes, B, Wb, Hb, N, Jx2, Jy); });
        }
    }
}

int main(int argc, char **argv)
{
    if (argc != 3) {
        std::fprintf(stderr, "usage: block_sums_emu IN OUT\n");
        return 2;
    }
    FILE *f = std::fopen(argv[1], "rb");
    if (!f) return 2;
    int32_t hdr[4];
    if (std::fread(hdr, sizeof(hdr), 1, f) != 1) return 2;
    const int model = hdr[0], W = hdr[1], H = hdr[2], B = hdr[3];
    std::vector<uint8_t> cells((size_t)W * H);
    if (std::fread(cells.data(), 1, cells.size(), f) != cells.size()) return 2;
    std::fclose(f);
    if (B < 1) return 3;
    const int D = num_dir(model);
    PlaneGeom g{};
    g.W = W;
    g.H = H;
    g.nw = (W + 63) / 64;
    g.pitch = (g.nw + 1) & ~1;
    g.ps = (size_t)H * g.pitch;
    g.L = (W - 1) & 63;
    g.lastmask = (g.L == 63) ? ~0ull : ((1ull << (g.L + 1)) - 1ull);
    std::vector<uint64_t> planes(D * g.ps, 0);
    for (int y = 0; y < H; ++y)
        for (int x = 0; x < W; ++x)
            for (int d = 0; d < D; ++d)
                if ((cells[(size_t)y * W + x] >> d) & 1)
                    planes[d * g.ps + (size_t)y * g.pitch + (x >> 6)] |= 1ull << (x & 63);
    const int Wb = (W + B - 1) / B, Hb = (H + B - 1) / B;
    std::vector<int32_t> N((size_t)Wb * Hb, -1), Jx2(N.size(), -1), Jy(N.size(), -1);
    if (model == 0) block_sums<M_HPP>(g, planes.data(), B, N.data(), Jx2.data(), Jy.data());
    else if (model == 1) block_sums<M_FHP_I>(g, planes.data(), B, N.data(), Jx2.data(), Jy.data());
    else block_sums<M_FHP_II>(g, planes.data(), B, N.data(), Jx2.data(), Jy.data());
    f = std::fopen(argv[2], "wb");
    if (!f) return 2;
    std::fwrite(N.data(), 4, N.size(), f);
    std::fwrite(Jx2.data(), 4, Jx2.size(), f);
    std::fwrite(Jy.data(), 4, Jy.size(), f);
    std::fclose(f);
    return 0;
}
